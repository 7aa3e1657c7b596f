"""Autotuner (sel_scene_autotune): it may choose any BVH layout, leaf size, wavefront capacity and traversal
block size, and none of them may change an image (bit-exact hits, per-path random streams)."""
import numpy as np
import pytest

import selas_gb300 as sel
from selas_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("make", [scenes.cornell_box, lambda: scenes.textured_spheres(count=4, level=3)])
def test_tuned_scene_renders_the_same_image(device, make):
    rs = make()
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 96, 96)
    before = sc.pt_generate_image(cam, sel.pt_settings(8, 8, seed=77))
    res = sc.autotune(rs.sel_camera(sel, 128, 128), sel.pt_settings(16, 8, seed=5))
    trials = [res.trial[i] for i in range(res.trials)]
    assert len(trials) == 4 * 2 * 3 + 3  # 8-wide: 4 leaf sizes x 3 capacities x 2 blocks; binary: 3 capacities
    points = {(t.leaf_size, t.paths_in_flight, t.trace_block) for t in trials if t.bvh_kind == sel.SEL_BVH_WIDE8_Q8}
    assert {(4, 1 << 20, 128), (8, 1 << 23, 256)} <= points
    assert min(t.ms for t in trials) == res.best.ms and res.best.ms > 0
    info = sc.info()
    assert info.bvh_kind == res.best.bvh_kind
    after = sc.pt_generate_image(cam, sel.pt_settings(8, 8, seed=77))
    np.testing.assert_allclose(after, before, rtol=1e-5, atol=1e-8)
    sc.release()


def test_tuned_instanced_scene_renders_the_same_image(device):
    """The instanced configuration's space: leaf {2, 3, 4, 8} x capacity {1M, 4M, 8M} x block {128, 256} (the
    binary layout cannot hold instances), with the 256-thread instanced traversal among the points."""
    import dataclasses
    c = scenes.cornell_box()
    world = scenes.RenderScene(scenes.TriangleScene(), {}, c.lights, c.background, c.camera)
    iscene = scenes.InstancedRenderScene([world, dataclasses.replace(c, lights=[])],
                                         [[(5, 1, np.eye(4, dtype=np.float32))], []])
    built = iscene.build(sel, device)
    top = built[0]
    cam = iscene.sel_camera(sel, 64, 64)
    before = top.pt_generate_image(cam, sel.pt_settings(4, 8, seed=77))
    res = top.autotune(iscene.sel_camera(sel, 96, 96), sel.pt_settings(8, 8, seed=5))
    trials = [res.trial[i] for i in range(res.trials)]
    assert len(trials) == 4 * 3 * 2
    assert {(t.leaf_size, t.paths_in_flight, t.trace_block) for t in trials} >= {
        (leaf, cap, block) for leaf in (4, 8) for cap in (1 << 20, 1 << 22, 1 << 23) for block in (128, 256)}
    for block in (128, 256):
        st = sel.pt_settings(4, 8, seed=77)
        st.traceBlockSize = block
        np.testing.assert_allclose(top.pt_generate_image(cam, st), before, rtol=1e-5, atol=1e-8)
    iscene.release(built)

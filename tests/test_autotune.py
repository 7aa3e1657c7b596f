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
    assert len(trials) == 3 * 2 * 3 + 3  # 8-wide: 3 leaf sizes x 3 capacities x 2 blocks; binary: 3 capacities
    assert min(t.ms for t in trials) == res.best.ms and res.best.ms > 0
    info = sc.info()
    assert info.bvh_kind == res.best.bvh_kind
    after = sc.pt_generate_image(cam, sel.pt_settings(8, 8, seed=77))
    np.testing.assert_allclose(after, before, rtol=1e-5, atol=1e-8)
    sc.release()

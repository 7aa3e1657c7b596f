"""Path tracing and deferred path tracing of instanced scenes (CalculateSurfaceParams through
ModelDataFromRayIds: material and Ptex of the hit mesh's scene, Ng through the instances' localToWorld).

The instanced-terrain scene here is the instanced configuration at test size: an fBm heightfield, displaced
icosphere instances with per-face Ptex, and a second instancing level (clusters of three instances).  GPU and
oracle trace the same PCG32 streams, so their images agree pixel by pixel up to FP32 rounding of the
transcendental functions."""
import dataclasses

import numpy as np
import pytest

import oracle
from selas_gb300 import scenes

SEED = 0x5E1A5000


def _terrain():
    s = scenes.instanced_terrain(grid=65, instances=40, mesh_level=2, log2=2, groups=6, seed=0x5E1A5104)
    # look at the first instance from close by, so that instances fill most of a small image
    x, y, z = s.instances[0][0][2][:, 3]
    top = dataclasses.replace(s.parts[0], camera=dict(position=(x - 30.0, y + 14.0, z - 30.0), look_at=(x, y, z),
                                                      up=(0.0, 1.0, 0.0), fov_degrees=70.0))
    return scenes.InstancedRenderScene([top] + s.parts[1:], s.instances)


def _identity_cornell():
    c = scenes.cornell_box()
    world = scenes.RenderScene(scenes.TriangleScene(), {}, c.lights, c.background, c.camera)
    proto = dataclasses.replace(c, lights=[])
    return c, scenes.InstancedRenderScene([world, proto], [[(5, 1, np.eye(4, dtype=np.float32))], []])


def _assert_same_paths(gpu, cpu):
    fin_g, fin_c = np.isfinite(gpu).all(axis=-1), np.isfinite(cpu).all(axis=-1)
    assert np.array_equal(fin_g, fin_c)
    g, c = gpu[fin_g], cpu[fin_c]
    rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-3 * c.mean())
    assert np.median(rel) < 1e-4, np.median(rel)
    assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()
    assert abs(g.mean() / c.mean() - 1.0) < 5e-3


def test_oracle_identity_instance_equals_flat_scene():
    flat, inst = _identity_cornell()
    a = oracle.pt_render(flat, 32, 32, 0, 4, seed=SEED)
    b = oracle.graph_render(inst, 32, 32, 0, 4, seed=SEED)
    np.testing.assert_array_equal(a, b)
    a = oracle.deferred_render(flat, 32, 32, 0, 16, seed=SEED)
    b = oracle.graph_render(inst, 32, 32, 0, 16, seed=SEED, deferred=True, max_bounces=64)
    np.testing.assert_array_equal(a, b)


def test_oracle_terrain_sees_instances_at_both_levels():
    from selas_gb300 import make_rayhits
    s = _terrain()
    c = s.camera
    pos, look = np.float32(c["position"]), np.float32(c["look_at"])
    fwd = (look - pos) / np.linalg.norm(look - pos)
    rng = np.random.default_rng(1)
    d = (fwd + rng.normal(scale=0.1, size=(4000, 3))).astype(np.float32)
    r = make_rayhits(np.tile(pos, (4000, 1)), d)
    oracle.instanced_query(s.graph(), 0, r)
    assert (r["instID0"] != 0xFFFFFFFF).mean() > 0.2
    # rays from above every cluster reach second-level instances
    for _, _, m in s.instances[0][-6:]:
        c0 = m[:, 3]
        org = np.tile(np.float32(c0 + np.float32([0, 60, 0])), (500, 1))
        d = (np.float32([0, -1, 0]) + rng.normal(scale=0.08, size=(500, 3))).astype(np.float32)
        r = make_rayhits(org, d)
        oracle.instanced_query(s.graph(), 0, r)
        assert (r["instID1"] != 0xFFFFFFFF).sum() > 5
    img = oracle.graph_render(s, 40, 30, 0, 2)
    assert np.isfinite(img).all() and img[1].mean() > 0


def _gpu(device, iscene, size, spp_or_axis, deferred=False, max_bounces=8, **kw):
    import selas_gb300 as sel
    built = iscene.build(sel, device)
    cam = iscene.sel_camera(sel, *size)
    if deferred:
        img = built[0].deferred_generate_image(cam, sel.deferred_settings(spp_or_axis, max_bounces, SEED, **kw))
    else:
        img = built[0].pt_generate_image(cam, sel.pt_settings(spp_or_axis, max_bounces, SEED, **kw))
    iscene.release(built)
    return img.astype(np.float64)


@pytest.mark.gpu
def test_gpu_instanced_pt_traces_the_oracles_paths(device):
    s = _terrain()
    gpu = _gpu(device, s, (64, 48), 8)
    cpu = oracle.graph_render(s, 64, 48, 0, 8, seed=SEED) / 8.0
    for layer in (0, 1):
        _assert_same_paths(gpu[layer], cpu[layer])


@pytest.mark.gpu
def test_gpu_instanced_deferred_traces_the_oracles_paths(device):
    s = _terrain()
    gpu = _gpu(device, s, (64, 48), 3, deferred=True, max_bounces=16)
    cpu = oracle.graph_render(s, 64, 48, 0, 9, seed=SEED, deferred=True, samples_per_axis=3, max_bounces=16) / 9.0
    _assert_same_paths(gpu, cpu)


@pytest.mark.gpu
def test_gpu_second_level_instances_render(device):
    """Clusters (instances of a scene of instances) in view: same paths as the oracle."""
    s = _terrain()
    x, y, z = s.instances[0][-1][2][:, 3]  # the last cluster
    top = dataclasses.replace(s.parts[0], camera=dict(position=(x - 40.0, y + 20.0, z - 40.0), look_at=(x, y, z),
                                                      up=(0.0, 1.0, 0.0), fov_degrees=50.0))
    s2 = scenes.InstancedRenderScene([top] + s.parts[1:], s.instances)
    gpu = _gpu(device, s2, (48, 48), 4)
    cpu = oracle.graph_render(s2, 48, 48, 0, 4, seed=SEED) / 4.0
    _assert_same_paths(gpu[1], cpu[1])


@pytest.mark.gpu
def test_gpu_identity_instance_equals_flat_scene(device):
    import selas_gb300 as sel
    flat, inst = _identity_cornell()
    sc = flat.build(sel, device)
    a = sc.pt_generate_image(flat.sel_camera(sel, 40, 40), sel.pt_settings(8, 8, SEED)).astype(np.float64)
    sc.release()
    b = _gpu(device, inst, (40, 40), 8)
    np.testing.assert_allclose(b, a, rtol=1e-6, atol=1e-9)


def _vcm_radius(bounds):
    lo, hi = bounds
    return float(0.003 * np.linalg.norm(np.float32(hi) - np.float32(lo)))


def test_oracle_identity_instance_vcm_equals_flat_scene():
    flat, inst = _identity_cornell()
    lo, hi = flat.geometry.bounds()
    r = _vcm_radius((lo, hi))
    a = oracle.vcm_render(flat, 24, 24, 0, 2, max_len=6, radius0=r, seed=SEED)
    b = oracle.graph_vcm_render(inst, 24, 24, 0, 2, (lo, hi), max_len=6, radius0=r, seed=SEED)
    np.testing.assert_array_equal(a, b)


@pytest.mark.gpu
def test_gpu_instanced_vcm_traces_the_oracles_paths(device):
    """VCM on the instanced terrain (Ptex instances, two levels): light vertices and camera records keep their
    material's address, so connections and merges shade with the instance's own material table."""
    import selas_gb300 as sel
    s = _terrain()
    built = s.build(sel, device)
    info = built[0].info()
    bounds = (np.float32(info.bounds_lo), np.float32(info.bounds_hi))
    r = _vcm_radius(bounds) * 4.0
    gpu = built[0].vcm_generate_image(s.sel_camera(sel, 48, 40), sel.vcm_settings(4, 6, SEED, radius=r))
    s.release(built)
    cpu = oracle.graph_vcm_render(s, 48, 40, 0, 4, bounds, max_len=6, radius0=r, seed=SEED) / 4.0
    _assert_same_paths(gpu.astype(np.float64), cpu)


@pytest.mark.gpu
def test_gpu_identity_instance_vcm_equals_flat_scene(device):
    import selas_gb300 as sel
    flat, inst = _identity_cornell()
    lo, hi = flat.geometry.bounds()
    r = _vcm_radius((lo, hi))
    sc = flat.build(sel, device)
    a = sc.vcm_generate_image(flat.sel_camera(sel, 40, 40), sel.vcm_settings(3, 8, SEED, radius=r)).astype(np.float64)
    sc.release()
    built = inst.build(sel, device)
    b = built[0].vcm_generate_image(inst.sel_camera(sel, 40, 40), sel.vcm_settings(3, 8, SEED, radius=r))
    inst.release(built)
    np.testing.assert_allclose(b.astype(np.float64), a, rtol=1e-5, atol=1e-8)


@pytest.mark.gpu
def test_gpu_served_instanced_job_equals_direct_render(device):
    import selas_gb300 as sel
    s = _terrain()
    built = s.build(sel, device)
    cam = s.sel_camera(sel, 48, 40)
    direct = built[0].pt_generate_image(cam, sel.pt_settings(4, 6, seed=21))
    srv = sel.Server(device)
    img, st = srv.wait(srv.submit(sel.pt_job(built[0], cam, sel.pt_settings(4, 6, seed=21))))
    srv.release()
    assert st.status == 0
    np.testing.assert_allclose(img, direct, rtol=1e-5, atol=1e-8)
    s.release(built)


@pytest.mark.gpu
@pytest.mark.parametrize("deferred", [False, True])
def test_gpu_views_in_one_wavefront_equal_single_renders(device, deferred):
    """sel_render_views: view k equals the single-view render with seed + k; views of different sizes."""
    import selas_gb300 as sel
    s = _terrain()
    built = s.build(sel, device)
    base = s.camera
    cams = []
    for k, (w, h) in enumerate([(48, 40), (32, 32), (64, 24)]):
        pos = np.array(base["position"]) + np.array([8.0 * k, 0.0, -5.0 * k])
        cams.append(sel.camera(tuple(pos), base["look_at"], base["up"], base["fov_degrees"], w, h))
    st = sel.deferred_settings(3, 12, seed=40) if deferred else sel.pt_settings(6, 6, seed=40)
    st.pathsInFlight = 3000  # several batches, each with paths of every view
    views = built[0].render_views(cams, st, deferred=deferred)
    for k, cam in enumerate(cams):
        one = sel.deferred_settings(3, 12, seed=40 + k) if deferred else sel.pt_settings(6, 6, seed=40 + k)
        single = built[0].deferred_generate_image(cam, one) if deferred else built[0].pt_generate_image(cam, one)
        np.testing.assert_allclose(views[k], single, rtol=1e-5, atol=1e-8)
    s.release(built)

"""Round B-spline curves (sel_scene_attach_curve_mesh, the reference's RTC_GEOMETRY_TYPE_ROUND_BSPLINE_CURVE
geometries of ModelResource.cpp:300-332).  Embree's curve intersector is a closed binary, so the hits follow the
library's own definition (curve.cuh): the segment cut into eight round cones between the spline's spheres.  The
CPU oracle restates that definition; the device must return the same bits (t, u, v, Ng, primID, geomID)."""
import numpy as np
import pytest

import oracle
import selas_gb300 as sel
from selas_gb300 import scenes

SEED = 0x5E1A5000


def _records(org, d, any_hit=False):
    return sel.make_rays(org, d) if any_hit else sel.make_rayhits(org, d)


def test_oracle_straight_segment_is_a_tube():
    """Four equally spaced collinear control points of equal radius: the pieces are cylinders with spherical ends,
    so a ray across the axis hits at distance - r with Ng perpendicular to the axis, and u runs along it."""
    r = 0.25
    pts = np.array([[0, -1, 0, r], [0, 0, 0, r], [0, 1, 0, r], [0, 2, 0, r]], np.float32)
    ys = np.linspace(0.05, 0.95, 9, dtype=np.float32)
    org = np.column_stack([np.full(9, -5.0), ys, np.zeros(9)]).astype(np.float32)
    d = np.tile(np.float32([1, 0, 0]), (9, 1))
    rec = _records(org, d)
    oracle.curve_hits(pts, [0], 3, rec)
    assert (rec["geomID"] == 3).all() and (rec["primID"] == 0).all()
    np.testing.assert_allclose(rec["tfar"], 5.0 - r, rtol=1e-5)
    np.testing.assert_allclose(rec["Ng_y"], 0.0, atol=1e-5)
    # B-spline of collinear, evenly spaced points: centre y = u, so u follows the ray's height
    np.testing.assert_allclose(rec["u"], ys, atol=2e-3)
    assert (rec["v"] == 0).all()


def test_oracle_any_hit_and_misses():
    pts, idx = scenes.curve_strands(strands=4)
    org = np.float32([[0, 1, -6], [0, 50, -6]])
    d = np.float32([[0, 0, 1], [0, 0, 1]])
    rays = _records(org, d, any_hit=True)
    oracle.curve_hits(pts, idx, 0, rays)
    hits = _records(org, d)
    oracle.curve_hits(pts, idx, 0, hits)
    assert np.array_equal(rays["tfar"] == -np.inf, hits["geomID"] != 0xFFFFFFFF)
    assert hits["geomID"][1] == 0xFFFFFFFF


def _scene_rays(pts, n=20000, seed=3):
    rng = np.random.default_rng(seed)
    lo, hi = pts[:, :3].min(0) - 0.2, pts[:, :3].max(0) + 0.2
    target = rng.uniform(lo, hi, size=(n, 3))
    org = target + rng.normal(size=(n, 3)) * 4.0
    d = target - org
    return org.astype(np.float32), d.astype(np.float32)


def _floor():
    g = scenes.TriangleScene()
    g.add(1, np.float32([[-4, -0.01, -4], [4, -0.01, -4], [4, -0.01, 4], [-4, -0.01, 4]]),
          np.uint32([[0, 1, 2], [0, 2, 3]]))
    return g


def _expected(pts, idx, org, d, floor, any_hit=False):
    rec = _records(org, d, any_hit)
    if any_hit:
        oracle.occluded_bruteforce(floor.soup(), rec)
    else:
        oracle.intersect_bruteforce(floor.soup(), rec)
    oracle.curve_hits(pts, idx, 7, rec)
    return rec


@pytest.mark.gpu
def test_gpu_curve_hits_match_the_oracle(device):
    pts, idx = scenes.curve_strands()
    floor = _floor()
    sc = sel.Scene(device)
    floor.attach_to(sc)
    sc.attach_curve_mesh(7, pts, idx)
    sc.commit()
    org, d = _scene_rays(pts)
    got = _records(org, d)
    sc.intersect1M(got)
    want = _expected(pts, idx, org, d, floor)
    assert (want["geomID"] == 7).mean() > 0.1 and (want["geomID"] == 1).mean() > 0.05
    for f in ("geomID", "primID", "tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z", "instID0", "instID1"):
        np.testing.assert_array_equal(got[f], want[f], err_msg=f)
    got_a = _records(org, d, any_hit=True)
    sc.occluded1M(got_a)
    want_a = _expected(pts, idx, org, d, floor, any_hit=True)
    np.testing.assert_array_equal(got_a["tfar"] == -np.inf, want_a["tfar"] == -np.inf)
    sc.release()


@pytest.mark.gpu
def test_gpu_instanced_curves_equal_the_flat_scene(device):
    pts, idx = scenes.curve_strands(strands=12)
    proto = sel.Scene(device)
    proto.attach_curve_mesh(0, pts, idx)
    proto.commit()
    top = sel.Scene(device)
    top.attach_instance(4, proto, np.eye(4))
    top.commit()
    org, d = _scene_rays(pts, 8000, seed=5)
    a, b = _records(org, d), _records(org, d)
    proto.intersect1M(a)
    top.intersect1M(b)
    for f in ("geomID", "primID", "tfar", "u", "Ng_x", "Ng_y", "Ng_z"):
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    hit = a["geomID"] != 0xFFFFFFFF
    assert hit.mean() > 0.05 and (b["instID0"][hit] == 4).all()
    top.release()
    proto.release()


def _curve_render_scene(strands=24):
    pts, idx = scenes.curve_strands(strands=strands)
    return scenes.RenderScene(
        _floor(), {1: dict(shader=1, lightSetIndex=0, baseColor=(0.6, 0.6, 0.6), roughness=0.7, ior=1.5),
                   7: dict(shader=1, lightSetIndex=0, baseColor=(0.35, 0.2, 0.1), roughness=0.4, metallic=0.2,
                           ior=1.5)},
        [(0, dict(position=(0.0, 4.0, 0.0), direction=(0.0, -1.0, 0.0), x=(2.0, 0.0, 0.0), z=(0.0, 0.0, 2.0),
                  radiance=(20.0, 18.0, 15.0)))], (0.1, 0.1, 0.12),
        dict(position=(0.0, 1.5, -5.0), look_at=(0.0, 1.0, 0.0), up=(0.0, 1.0, 0.0), fov_degrees=45.0),
        curves={7: (pts, idx)})


def _same_paths(gpu, cpu):
    assert np.isfinite(gpu).all() and np.isfinite(cpu).all()
    rel = np.abs(gpu - cpu) / np.maximum(np.abs(cpu), 1e-3 * cpu.mean())
    assert np.median(rel) < 1e-4, np.median(rel)
    assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()
    assert abs(gpu.mean() / cpu.mean() - 1.0) < 5e-3


def test_oracle_renders_the_strands():
    """The strands stand between the camera and the floor: the oracle's image changes where they are."""
    rs = _curve_render_scene()
    with_curves = oracle.pt_render(rs, 24, 16, 0, 2, max_bounces=3, seed=SEED)
    rs.curves = None
    floor_only = oracle.pt_render(rs, 24, 16, 0, 2, max_bounces=3, seed=SEED)
    changed = np.abs(with_curves[1] - floor_only[1]).max(axis=-1) > 1e-6
    assert 0.02 < changed.mean() < 0.9


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["pt", "deferred", "vcm"])
def test_gpu_curve_scene_traces_the_oracles_paths(device, integrator):
    rs = _curve_render_scene()
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 48, 32)
    try:
        if integrator == "pt":
            gpu = sc.pt_generate_image(cam, sel.pt_settings(8, 6, SEED)).astype(np.float64)
            device.set_option(sel.SEL_OPTION_GRAPH_REPLAY, 0)
            eager = sc.pt_generate_image(cam, sel.pt_settings(8, 6, SEED)).astype(np.float64)
            device.set_option(sel.SEL_OPTION_GRAPH_REPLAY, 1)
            np.testing.assert_array_equal(gpu, eager)
            cpu = oracle.pt_render(rs, 48, 32, 0, 8, max_bounces=6, seed=SEED) / 8.0
            pairs = [(gpu[0], cpu[0]), (gpu[1], cpu[1])]
        elif integrator == "deferred":
            gpu = sc.deferred_generate_image(cam, sel.deferred_settings(4, 6, SEED)).astype(np.float64)
            cpu = oracle.deferred_render(rs, 48, 32, 0, 16, samples_per_axis=4, max_bounces=6, seed=SEED) / 16.0
            pairs = [(gpu, cpu)]
        else:  # an explicit merge radius: the default one follows the scene box, which the curves' boxes pad
            gpu = sc.vcm_generate_image(cam, sel.vcm_settings(4, 6, SEED, radius=0.02)).astype(np.float64)
            cpu = oracle.vcm_render(rs, 48, 32, 0, 4, max_len=6, radius0=0.02, seed=SEED) / 4.0
            pairs = [(gpu, cpu)]
    finally:
        sc.release()
    for g, c in pairs:
        _same_paths(g, c)


@pytest.mark.gpu
def test_gpu_instanced_curve_scene_traces_the_oracles_paths(device):
    """Strands in two instances of one prototype beside a floor (the oracle's per-scene traversal of the graph)."""
    rs = _curve_render_scene(strands=10)
    world = scenes.RenderScene(_floor(), {1: rs.materials[1]}, rs.lights, rs.background, rs.camera)
    proto = scenes.RenderScene(scenes.TriangleScene(), {7: rs.materials[7]}, [], (0.0, 0.0, 0.0), {},
                               curves=rs.curves)
    left = np.eye(4, dtype=np.float32)
    left[0, 3] = -1.2
    right = np.eye(4, dtype=np.float32)
    right[:3, :3] = np.float32([[0.0, 0.0, 0.8], [0.0, 0.8, 0.0], [-0.8, 0.0, 0.0]])
    right[0, 3] = 1.3
    iscene = scenes.InstancedRenderScene([world, proto], [[(3, 1, left), (4, 1, right)], []])  # mesh 1: floor
    built = iscene.build(sel, device)
    try:
        cam = rs.sel_camera(sel, 48, 32)
        gpu = built[0].pt_generate_image(cam, sel.pt_settings(8, 6, SEED)).astype(np.float64)
    finally:
        iscene.release(built)
    cpu = oracle.graph_render(iscene, 48, 32, 0, 8, max_bounces=6, seed=SEED) / 8.0
    for layer in range(2):
        _same_paths(gpu[layer], cpu[layer])


@pytest.mark.gpu
def test_gpu_curve_geometry_is_checked(device):
    pts, idx = scenes.curve_strands(strands=2)
    sc = sel.Scene(device)
    with pytest.raises(sel.SelError):
        sc.attach_curve_mesh(0, pts, np.uint32([pts.shape[0] - 2]))  # runs past the points
    bad = pts.copy()
    bad[0, 3] = -1.0
    with pytest.raises(sel.SelError):
        sc.attach_curve_mesh(0, bad, idx)
    sc.attach_curve_mesh(0, pts, idx)
    with pytest.raises(sel.SelError):
        sc.attach_curve_mesh(0, pts, idx)  # geomID taken
    with pytest.raises(sel.SelError):
        sc.set_texture(0, np.ones((2, 2, 3), np.float32))  # curves have no uvs
    with pytest.raises(sel.SelError):
        sc.set_vertex_attribute(0, 0, np.ones((pts.shape[0], 3), np.float32))
    sc.set_texture(5, np.ones((2, 2, 3), np.float32))
    with pytest.raises(sel.SelError):
        sc.attach_curve_mesh(5, pts, idx)
    sc.release()
    binary = sel.Scene(device, sel.SEL_BVH_BINARY_FP32)
    binary.attach_curve_mesh(0, pts, idx)
    with pytest.raises(sel.SelError):
        binary.commit()
    binary.release()

"""Vertex attributes (rtcSetGeometryVertexAttributeCount / rtcSetSharedGeometryBuffer(VERTEX_ATTRIBUTE),
ModelResource.cpp:183-197; rtcInterpolate0 in CalculateSurfaceParams, SurfaceParameters.cpp:157-190): shading
normals and tangents interpolated at the hit, through the instances' localToWorld, in the path tracer, the deferred
path tracer and VCM; sel_interpolate0 on the host."""
import dataclasses

import numpy as np
import pytest

import oracle
from selas_gb300 import scenes

SEED = 0x5E1A5000


def _assert_same_paths(gpu, cpu):
    fin_g, fin_c = np.isfinite(gpu).all(axis=-1), np.isfinite(cpu).all(axis=-1)
    assert np.array_equal(fin_g, fin_c)
    g, c = gpu[fin_g], cpu[fin_c]
    rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-3 * c.mean())
    assert np.median(rel) < 1e-4, np.median(rel)
    assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()
    assert abs(g.mean() / c.mean() - 1.0) < 5e-3


def test_oracle_vertex_normals_change_the_shading():
    rs = scenes.smooth_spheres()
    smooth = oracle.pt_render(rs, 48, 32, 0, 4, seed=SEED)
    faceted = oracle.pt_render(dataclasses.replace(rs, attrs=None), 48, 32, 0, 4, seed=SEED)
    assert np.isfinite(smooth).all()
    diff = np.abs(smooth[1] - faceted[1]).sum(-1)
    assert (diff > 1e-3).mean() > 0.05  # the spheres' pixels change, the floor's do not
    assert (diff == 0).mean() > 0.3


@pytest.mark.gpu
def test_gpu_interpolate0_matches_the_formula(device):
    import selas_gb300 as sel
    rs = scenes.smooth_spheres()
    sc = rs.build(sel, device)
    gid, v, idx = rs.geometry.meshes[0]
    n = rs.attrs[0]["normals"]
    t = rs.attrs[0]["tangents"]
    rng = np.random.default_rng(2)
    for _ in range(200):
        prim = int(rng.integers(0, idx.shape[0]))
        u, w2 = np.float32(rng.random()), np.float32(rng.random())
        if u + w2 > 1:
            u, w2 = np.float32(1) - u, np.float32(1) - w2
        w = np.float32(1) - u - w2
        a = idx[prim]
        for slot, data in ((0, n), (1, t)):
            want = (w * data[a[0]] + u * data[a[1]]) + w2 * data[a[2]]
            got = sc.interpolate0(gid, prim, float(u), float(w2), slot, data.shape[1])
            assert np.array_equal(got.view(np.uint32), want.astype(np.float32).view(np.uint32))
    with pytest.raises(sel.SelError):
        sc.interpolate0(rs.geometry.meshes[-1][0], 0, 0.2, 0.2, 0, 3)  # the floor has no normals
    sc.release()


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["pt", "deferred", "vcm"])
def test_gpu_vertex_attributes_trace_the_oracles_paths(device, integrator):
    import selas_gb300 as sel
    rs = scenes.smooth_spheres()
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 64, 48)
    if integrator == "pt":
        gpu = sc.pt_generate_image(cam, sel.pt_settings(8, 6, SEED)).astype(np.float64)
        cpu = oracle.pt_render(rs, 64, 48, 0, 8, max_bounces=6, seed=SEED) / 8.0
        for layer in (0, 1):
            _assert_same_paths(gpu[layer], cpu[layer])
    elif integrator == "deferred":
        gpu = sc.deferred_generate_image(cam, sel.deferred_settings(3, 16, SEED)).astype(np.float64)
        cpu = oracle.deferred_render(rs, 64, 48, 0, 9, samples_per_axis=3, max_bounces=16, seed=SEED) / 9.0
        _assert_same_paths(gpu, cpu)
    else:
        lo, hi = rs.geometry.bounds()
        r0 = 0.01 * float(np.linalg.norm(hi - lo))
        gpu = sc.vcm_generate_image(cam, sel.vcm_settings(3, 8, seed=SEED, radius=r0)).astype(np.float64)
        cpu = oracle.vcm_render(rs, 64, 48, 0, 3, max_len=8, radius0=r0, seed=SEED) / 3.0
        _assert_same_paths(gpu, cpu)
    sc.release()


@pytest.mark.gpu
def test_gpu_instanced_vertex_attributes_trace_the_oracles_paths(device):
    """Instances of a mesh with vertex normals and tangents: both go through the instances' localToWorld."""
    import selas_gb300 as sel
    rs = scenes.smooth_spheres(count=2)
    proto = dataclasses.replace(rs, lights=[], geometry=scenes.TriangleScene(rs.geometry.meshes[:1]),
                                materials={0: rs.materials[0]}, attrs={0: rs.attrs[0]})
    world = dataclasses.replace(rs, geometry=scenes.TriangleScene(rs.geometry.meshes[2:]), attrs=None,
                                materials={2: rs.materials[2]})
    rng = np.random.default_rng(4)
    insts = []
    for k in range(6):
        m = np.zeros((3, 4), np.float32)
        q = rng.normal(size=(3, 3))
        rot, _ = np.linalg.qr(q)
        m[:, :3] = rot * rng.uniform(0.7, 1.3)
        m[:, 3] = (rng.uniform(-3, 3), rng.uniform(0.5, 2.0), rng.uniform(-2, 2))
        insts.append((10 + k, 1, m))
    iscene = scenes.InstancedRenderScene([world, proto], [insts, []])
    built = iscene.build(sel, device)
    gpu = built[0].pt_generate_image(iscene.sel_camera(sel, 64, 48), sel.pt_settings(8, 6, SEED)).astype(np.float64)
    iscene.release(built)
    cpu = oracle.graph_render(iscene, 64, 48, 0, 8, max_bounces=6, seed=SEED) / 8.0
    _assert_same_paths(gpu[1], cpu[1])

"""Quad meshes (RTC_GEOMETRY_TYPE_QUAD, the geometry the reference makes for meshes with four indices per face,
ModelResource.cpp:272-281).  Embree's contract (RTC_GEOMETRY_TYPE_QUAD.3embree3): a quad is the triangles
(v0, v1, v3) and (v2, v3, v1); a hit reports the quad's index as primID, the hit triangle's Ng and the quad's
(u, v) - the second triangle's (u', v') become (1 - u', 1 - v') - and attributes interpolate bilinearly.  The
queries are bit-exact against the brute-force oracle over the same triangle pairs (ties between the two triangles
of a quad go to the first, which the pair numbering 2q, 2q + 1 gives both sides); renders trace the oracle's
paths."""
import dataclasses

import numpy as np
import pytest

import oracle
from conftest import HIT_FIELDS, assert_hits_equal
from selas_gb300 import scenes

SEED = 0x5E1A5000


def quad_field(n=300, seed=3, planar=False):
    """Random quads: planar parallelograms or bent ones, some degenerate (a triangle as v0, v1, v2, v2)."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(-10, 10, (n, 3))
    a = rng.normal(size=(n, 3)) * rng.uniform(0.5, 3, (n, 1))
    b = rng.normal(size=(n, 3)) * rng.uniform(0.5, 3, (n, 1))
    v = np.stack([o, o + a, o + a + b, o + b], 1)
    if not planar:
        v[:, 2] += rng.normal(size=(n, 3)) * 0.4
    v = v.astype(np.float32).reshape(-1, 3)
    q = np.arange(4 * n, dtype=np.uint32).reshape(n, 4)
    tri = rng.random(n) < 0.1
    q[tri, 3] = q[tri, 2]
    return v, q


def quad_scene(planar=False):
    g = scenes.TriangleScene()
    v, q = quad_field(planar=planar)
    g.add_quads(3, v, q)
    tv, ti = scenes.icosphere(2)
    g.add(5, (tv * 2.0 + np.float32([0, 0, 14])).astype(np.float32), ti.astype(np.uint32))
    return g


def rays(g, n=20000, seed=4):
    rng = np.random.default_rng(seed)
    lo, hi = g.bounds()
    org = rng.uniform(lo - 5, hi + 5, (n, 3)).astype(np.float32)
    tgt = rng.uniform(lo, hi, (n, 3))
    # a share of the rays aim at the quads' diagonals (v1 v3), where both triangles of a quad meet
    v = g.meshes[0][1].reshape(-1, 4, 3)
    k = rng.integers(0, v.shape[0], n // 4)
    s = rng.random((n // 4, 1))
    tgt[: n // 4] = v[k, 1] + s * (v[k, 3] - v[k, 1])
    d = tgt - org
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return org, d


def _oracle_hits(g, org, d):
    import selas_gb300 as sel
    want = sel.make_rayhits(org, d)
    oracle.intersect_bruteforce(g.soup(), want)
    g.embree_hits(want)
    return want


def test_oracle_quad_parametrisation():
    """On a planar quad p = v0 + u (v1 - v0) + v (v3 - v0) for hits on either triangle."""
    import selas_gb300 as sel
    g = scenes.TriangleScene()
    v = np.float32([[0, 0, 5], [4, 0, 5], [4, 2, 5], [0, 2, 5]])
    g.add_quads(0, v, np.uint32([[0, 1, 2, 3]]))
    uv = np.random.default_rng(1).random((500, 2)).astype(np.float32) * 0.98 + 0.01
    p = v[0] + uv[:, :1] * (v[1] - v[0]) + uv[:, 1:] * (v[3] - v[0])
    org = np.concatenate([p[:, :2], np.zeros((500, 1))], 1).astype(np.float32)
    d = np.tile(np.float32([0, 0, 1]), (500, 1))
    h = _oracle_hits(g, org, d)
    assert (h["geomID"] == 0).all() and (h["primID"] == 0).all()
    np.testing.assert_allclose(h["u"], uv[:, 0], atol=1e-5)
    np.testing.assert_allclose(h["v"], uv[:, 1], atol=1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("planar", [True, False])
def test_gpu_quad_queries_match_bruteforce(device, planar):
    import selas_gb300 as sel
    g = quad_scene(planar)
    org, d = rays(g)
    want = _oracle_hits(g, org, d)
    assert (want["geomID"] == 3).sum() > 2000
    rw = sel.make_rays(org, d)
    oracle.occluded_bruteforce(g.soup(), rw)
    for kind, mode in ((sel.SEL_BVH_WIDE8_Q8, sel.SEL_BUILD_DEVICE), (sel.SEL_BVH_WIDE8_Q8, sel.SEL_BUILD_HOST),
                       (sel.SEL_BVH_BINARY_FP32, None)):
        sc = sel.Scene(device, kind, mode)
        g.attach_to(sc)
        sc.commit()
        got = sel.make_rayhits(org, d)
        sc.intersect1M(got)
        assert_hits_equal(got, want, HIT_FIELDS)
        rg = sel.make_rays(org, d)
        sc.occluded1M(rg)
        assert_hits_equal(rg, rw, fields=("tfar",))
        sc.release()


@pytest.mark.gpu
def test_gpu_quad_interpolate0_is_bilinear(device):
    import selas_gb300 as sel
    v, q = quad_field(50, seed=9)
    attr = np.random.default_rng(2).normal(size=(v.shape[0], 4)).astype(np.float32)
    sc = sel.Scene(device)
    sc.attach_quad_mesh(1, v, q)
    sc.set_vertex_attribute(1, 1, attr)
    sc.commit()
    rng = np.random.default_rng(3)
    for prim in range(q.shape[0]):
        u, w = np.float32(rng.random()), np.float32(rng.random())
        out = sc.interpolate0(1, prim, float(u), float(w), 1, 4)
        t0, t1, t2, t3 = attr[q[prim, 0]], attr[q[prim, 1]], attr[q[prim, 2]], attr[q[prim, 3]]
        iu, iv = np.float32(1) - u, np.float32(1) - w
        want = iv * (iu * t0 + u * t1) + w * (iu * t3 + u * t2)
        np.testing.assert_array_equal(out, want.astype(np.float32))
    sc.release()


def quad_cornell():
    """The Cornell box with every wall and box face a quad (quad meshes), the floor carrying uvs and a checker
    image, the back wall vertex normals that lean the shading normal."""
    c = scenes.cornell_box()
    g = scenes.TriangleScene()
    attrs = {}
    for gid, v, idx in c.geometry.meshes:
        pairs = idx.reshape(-1, 2, 3)
        # each quad (a, b, c, d) was stored as the triangles (a, b, c), (a, c, d)
        quads = np.stack([pairs[:, 0, 0], pairs[:, 0, 1], pairs[:, 0, 2], pairs[:, 1, 2]], 1)
        g.add_quads(gid, v, quads)
    v0 = g.meshes[0][1]
    attrs[0] = {"uvs": (v0[:, [0, 2]] / 556.0 * 2.5).astype(np.float32)}
    v2 = g.meshes[2][1]
    lean = np.float32([[0.2, 0.1, -1], [-0.2, 0.1, -1], [-0.2, -0.1, -1], [0.2, -0.1, -1]])
    attrs[2] = {"normals": (lean / np.linalg.norm(lean, axis=1, keepdims=True))[: v2.shape[0]].astype(np.float32)}
    y, x = np.mgrid[0:8, 0:8]
    img = np.where(((x + y) % 2 == 0)[..., None], np.float32([0.9, 0.8, 0.1]), np.float32([0.1, 0.2, 0.9]))
    return dataclasses.replace(c, geometry=g, attrs=attrs, textures={0: img.astype(np.float32)})


def test_oracle_quad_cornell_is_the_triangle_cornell_without_attributes():
    """Without attributes the quad box is the same surfaces as the triangle box; both images agree in the mean."""
    plain = scenes.cornell_box()
    quads = dataclasses.replace(quad_cornell(), attrs=None, textures=None)
    a = oracle.pt_render(plain, 32, 32, 0, 16, seed=SEED)[1]
    b = oracle.pt_render(quads, 32, 32, 0, 16, seed=SEED)[1]
    assert abs(a.mean() / b.mean() - 1) < 0.03


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["pt", "deferred", "vcm"])
def test_gpu_quad_scene_traces_the_oracles_paths(device, integrator):
    import selas_gb300 as sel
    rs = quad_cornell()
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 40, 40)
    if integrator == "pt":
        gpu = sc.pt_generate_image(cam, sel.pt_settings(8, 6, SEED)).astype(np.float64)
        cpu = oracle.pt_render(rs, 40, 40, 0, 8, max_bounces=6, seed=SEED) / 8.0
        pairs = [(gpu[0], cpu[0]), (gpu[1], cpu[1])]
    elif integrator == "deferred":
        gpu = sc.deferred_generate_image(cam, sel.deferred_settings(3, 12, SEED)).astype(np.float64)
        cpu = oracle.deferred_render(rs, 40, 40, 0, 9, samples_per_axis=3, max_bounces=12, seed=SEED) / 9.0
        pairs = [(gpu, cpu)]
    else:
        gpu = sc.vcm_generate_image(cam, sel.vcm_settings(4, 6, SEED)).astype(np.float64)
        cpu = oracle.vcm_render(rs, 40, 40, 0, 4, max_len=6, seed=SEED) / 4.0
        pairs = [(gpu, cpu)]
    sc.release()
    for g, c in pairs:
        rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-3 * c.mean())
        assert np.median(rel) < 1e-4, np.median(rel)
        assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()


@pytest.mark.gpu
def test_gpu_quad_mesh_refuses_ptex(device):
    import selas_gb300 as sel
    rs = scenes.textured_spheres(count=1, level=1)
    sc = sel.Scene(device)
    v, q = quad_field(4)
    sc.attach_quad_mesh(0, v, q)
    rows, tex = next(iter(rs.ptex.values()))
    with pytest.raises(sel.SelError):
        sc.set_ptex(0, rows[:4], tex)
    sc.release()

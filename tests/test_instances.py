"""Two-level instancing (SceneResource.cpp:73-187 subscene instances of SubsceneResource.cpp:63-79 model
instances): the instanced traversal against the brute-force instanced oracle, bit for bit.

Semantics pinned here (the oracle restates them in oracle/oracle_query.cpp): the ray is carried into an
instance by the world-to-local rows of its transform; t stays in the world ray's parametrisation; Ng is the hit
mesh's object-space normal; instID[0] is the outermost instance's id, instID[1] the next one's; ties on t go to
the smaller (instID[0], instID[1], geomID, primID)."""
import numpy as np
import pytest

import oracle
from conftest import assert_hits_equal
from selas_gb300 import make_rayhits, make_rays
from selas_gb300.scenes import icosphere

INVALID = 0xFFFFFFFF


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _xform(rng, spread, scale_lo=0.5, scale_hi=2.0, shear=False):
    m = np.zeros((3, 4), np.float32)
    a = _rotation(rng) * rng.uniform(scale_lo, scale_hi)
    if shear:
        a = a @ np.diag(rng.uniform(0.5, 1.5, 3))
    m[:, :3] = a
    m[:, 3] = rng.uniform(-spread, spread, 3)
    return m


def _proper_triangles(v, f):
    """Drops triangles with repeated vertices or slivers (area / longest edge^2 < 0.05): on those the
    watertight test can return a t off the triangle, which a BVH culls and brute force does not."""
    t = v[f].astype(np.float64)
    area = np.linalg.norm(np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0]), axis=1)
    edge = np.max([np.linalg.norm(t[:, (k + 1) % 3] - t[:, k], axis=1) for k in range(3)], axis=0)
    return f[area > 0.05 * edge * edge].astype(np.uint32)


def scene_graph(seed=0x5E1A1257):
    """Scene 0: world (ground quad + 40 instances of scene 1 + 60 of scene 2 + 30 of scene 3);
    scene 1: a level-1 group holding its own triangles and 12 instances of scene 2 and 3 (so its instances
    are the second level); scenes 2, 3: leaf meshes (an icosphere of level 2, random triangles)."""
    rng = np.random.default_rng(seed)
    v_ico, f_ico = icosphere(2)
    rand_v = rng.uniform(-1, 1, (60, 3)).astype(np.float32)
    rand_f = _proper_triangles(rand_v, rng.integers(0, 60, (120, 3)))[:40]
    ground_v = np.array([[-40, -5, -40], [40, -5, -40], [40, -5, 40], [-40, -5, 40]], np.float32)
    ground_f = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    s2 = {"meshes": [(5, v_ico.astype(np.float32), f_ico.astype(np.uint32))], "instances": []}
    s3 = {"meshes": [(2, rand_v, rand_f), (9, rand_v * 0.5 + 0.25, rand_f[:10])], "instances": []}
    s1 = {"meshes": [(4, rand_v * 2.0, rand_f[:20])],
          "instances": [(100 + k, 2 if k % 2 else 3, _xform(rng, 4.0, 0.3, 1.0, shear=k % 3 == 0)) for k in range(12)]}
    top = {"meshes": [(1, ground_v, ground_f)], "instances": []}
    iid = 7
    for k in range(40):
        top["instances"].append((iid, 1, _xform(rng, 30.0, 0.5, 1.5)))
        iid += 3
    for k in range(60):
        top["instances"].append((iid, 2, _xform(rng, 30.0, 0.5, 3.0, shear=k % 4 == 0)))
        iid += 1
    for k in range(30):
        top["instances"].append((iid, 3, _xform(rng, 30.0)))
        iid += 2
    return [top, s1, s2, s3]


def graph_rays(n=40000, seed=0x5E1A1258):
    rng = np.random.default_rng(seed)
    org = rng.uniform(-45, 45, (n, 3)).astype(np.float32)
    target = rng.uniform(-30, 30, (n, 3)).astype(np.float32)
    d = (target - org).astype(np.float32)
    d[: n // 8] = rng.normal(size=(n // 8, 3))  # fully random directions
    d[n // 8: n // 8 + 64] = [0.0, -1.0, 0.0]    # axis-aligned
    return org, d.astype(np.float32)


def _oracle(graph, org, d, any_hit=False):
    if any_hit:
        r = make_rays(org, d)
    else:
        r = make_rayhits(org, d)
    oracle.instanced_query(graph, 0, r, any_hit=any_hit)
    return r


def _build(sel, device, graph, build_mode=None, leaf=None):
    scenes = [None] * len(graph)

    def make(i):
        if scenes[i] is not None:
            return scenes[i]
        for _, pi, _ in graph[i]["instances"]:
            make(pi)
        sc = sel.Scene(device, build_mode=build_mode)
        if leaf:
            sc.set_leaf_size(leaf)
        for gid, v, f in graph[i]["meshes"]:
            sc.attach_triangle_mesh(gid, v, f)
        for iid, pi, m in graph[i]["instances"]:
            sc.attach_instance(iid, scenes[pi], m)
        sc.commit()
        scenes[i] = sc
        return sc

    for i in range(len(graph)):
        make(i)
    return scenes


def _release(scenes):
    for sc in scenes:  # parents first
        sc.release()


# ---------------------------------------------------------------------------------------------------
# CPU: the oracle's own consistency
# ---------------------------------------------------------------------------------------------------
def test_affine_inverse_roundtrip():
    rng = np.random.default_rng(3)
    for _ in range(50):
        m = _xform(rng, 10.0, shear=True)
        w = oracle.affine_inverse(m)
        full = np.vstack([m.astype(np.float64), [0, 0, 0, 1]])
        inv = np.vstack([w.astype(np.float64), [0, 0, 0, 1]])
        assert np.abs(full @ inv - np.eye(4)).max() < 1e-5
    with pytest.raises(ValueError):
        oracle.affine_inverse(np.zeros((3, 4), np.float32))


def test_identity_instance_equals_flat_scene():
    g = scene_graph()
    org, d = graph_rays(8000)
    flat = [{"meshes": g[2]["meshes"], "instances": []}]
    inst = [{"meshes": [], "instances": [(42, 1, np.eye(4, dtype=np.float32))]}, g[2]]
    a = _oracle(flat, org * 0.05, d)
    b = _oracle(inst, org * 0.05, d)
    hit = a["geomID"] != INVALID
    assert hit.sum() > 100
    assert_hits_equal(b, a, fields=("tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z", "primID", "geomID"))
    assert (b["instID0"][hit] == 42).all() and (b["instID1"] == INVALID).all()


def test_translated_instance_keeps_world_t():
    g = scene_graph()
    rng = np.random.default_rng(5)
    org = rng.uniform(-0.3, 0.3, (2000, 3)).astype(np.float32) + np.float32([0, 0, -10])
    d = np.tile(np.float32([0, 0, 1]), (2000, 1))
    flat = [g[2]]
    shift = np.eye(4, dtype=np.float32)
    shift[:3, 3] = [0, 0, 5]
    inst = [{"meshes": [], "instances": [(3, 1, shift)]}, g[2]]
    a = _oracle(flat, org, d)
    b = _oracle(inst, org, d)
    hit = a["geomID"] != INVALID
    assert hit.sum() > 500
    np.testing.assert_array_equal(b["primID"][hit], a["primID"][hit])
    np.testing.assert_allclose(b["tfar"][hit], a["tfar"][hit] + 5.0, rtol=1e-6)


def test_nested_ids_and_tie_rule():
    # two coincident instances of the same mesh: every hit is a tie on t, won by the smaller instID
    g = scene_graph()
    org, d = graph_rays(4000)
    eye = np.eye(4, dtype=np.float32)
    two = [{"meshes": [], "instances": [(9, 1, eye), (4, 1, eye)]}, g[2]]
    r = _oracle(two, org * 0.05, d)
    hit = r["geomID"] != INVALID
    assert hit.sum() > 50 and (r["instID0"][hit] == 4).all()
    # the full graph: second-level hits carry both ids
    r = _oracle(g, *graph_rays(6000))
    lvl2 = r["instID1"] != INVALID
    assert lvl2.sum() > 20
    assert set(np.unique(r["instID1"][lvl2])) <= set(range(100, 112))


# ---------------------------------------------------------------------------------------------------
# GPU: the instanced traversal against the oracle
# ---------------------------------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("build_mode,leaf", [(None, None), (0, None), (None, 1), (None, 4)])
def test_gpu_instanced_queries_match_oracle(device, build_mode, leaf):
    import selas_gb300 as sel
    g = scene_graph()
    scenes = _build(sel, device, g, build_mode=build_mode, leaf=leaf)
    org, d = graph_rays()
    want = _oracle(g, org, d)
    got = make_rayhits(org, d)
    scenes[0].intersect1M(got)
    assert (want["geomID"] != INVALID).sum() > 10000
    assert (want["instID1"] != INVALID).sum() > 100
    assert_hits_equal(got, want)
    want_o = _oracle(g, org, d, any_hit=True)
    got_o = make_rays(org, d)
    scenes[0].occluded1M(got_o)
    np.testing.assert_array_equal(np.isneginf(got_o["tfar"]), np.isneginf(want_o["tfar"]))
    _release(scenes)


@pytest.mark.gpu
def test_gpu_identity_instance_equals_flat_scene(device):
    import selas_gb300 as sel
    g = scene_graph()
    flat = _build(sel, device, [g[2]])
    inst = _build(sel, device, [{"meshes": [], "instances": [(42, 1, np.eye(4, dtype=np.float32))]}, g[2]])
    org, d = graph_rays(20000)
    a, b = make_rayhits(org * 0.05, d), make_rayhits(org * 0.05, d)
    flat[0].intersect1M(a)
    inst[0].intersect1M(b)
    assert_hits_equal(b, a, fields=("tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z", "primID", "geomID"))
    hit = a["geomID"] != INVALID
    assert hit.sum() > 500 and (b["instID0"][hit] == 42).all()
    _release(inst)
    _release(flat)


@pytest.mark.gpu
def test_gpu_instanced_segments_and_untraceable_rays(device):
    import selas_gb300 as sel
    g = scene_graph()
    scenes = _build(sel, device, g)
    org, d = graph_rays(6000)
    rng = np.random.default_rng(9)
    tnear = rng.uniform(0, 2, org.shape[0]).astype(np.float32)
    tfar = (tnear + rng.uniform(0, 1.5, org.shape[0])).astype(np.float32)
    want = make_rayhits(org, d, tnear, tfar)
    oracle.instanced_query(g, 0, want)
    got = make_rayhits(org, d, tnear, tfar)
    scenes[0].intersect1M(got)
    assert_hits_equal(got, want)
    bad_o = np.array([[np.nan, 0, 0], [0, 0, 0], [np.inf, 1, 1]], np.float32)
    bad_d = np.array([[0, 1, 0], [0, 0, 0], [1, 0, 0]], np.float32)
    r = make_rayhits(bad_o, bad_d)
    scenes[0].intersect1M(r)
    assert (r["geomID"] == INVALID).all()
    _release(scenes)


@pytest.mark.gpu
def test_gpu_instance_rules(device):
    import selas_gb300 as sel
    g = scene_graph()
    leaf = _build(sel, device, [g[2]])[0]
    eye = np.eye(4, dtype=np.float32)
    # binary layout cannot hold instances
    b = sel.Scene(device, bvh_kind=sel.SEL_BVH_BINARY_FP32)
    b.attach_instance(1, leaf, eye)
    with pytest.raises(sel.SelError):
        b.commit()
    b.release()
    # instID collisions, singular and non-affine transforms
    p = sel.Scene(device)
    p.attach_triangle_mesh(3, *g[2]["meshes"][0][1:])
    with pytest.raises(sel.SelError):
        p.attach_instance(3, leaf, eye)
    with pytest.raises(sel.SelError):
        p.attach_instance(4, leaf, np.zeros((4, 4), np.float32))
    bad = eye.copy()
    bad[3, 0] = 1.0
    with pytest.raises(sel.SelError):
        p.attach_instance(5, leaf, bad)
    p.attach_instance(6, leaf, eye)
    p.commit()
    # a committed instanced scene cannot be released; re-committing it makes the parent stale
    with pytest.raises(sel.SelError):
        leaf.release()
    leaf.commit()
    r = make_rayhits(np.float32([[0, 0, -5]]), np.float32([[0, 0, 1]]))
    with pytest.raises(sel.SelError):
        p.intersect1M(r)
    p.commit()
    p.intersect1M(r)
    assert r["instID0"][0] == 6
    # three levels are refused
    q = sel.Scene(device)
    q.attach_instance(1, p, eye)
    q.commit()
    top = sel.Scene(device)
    top.attach_instance(1, q, eye)
    with pytest.raises(sel.SelError):
        top.commit()
    top.release()
    q.release()
    p.release()
    leaf.release()

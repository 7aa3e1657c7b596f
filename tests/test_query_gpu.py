"""GPU parity of the ray queries (C ABI -> sm_103a kernels) against the CPU oracle.

Closest-hit records (t, u, v, Ng, primID, geomID, instID) and any-hit bits must be bit-exact: both sides
implement the same watertight test with the same rounding steps and the same order-independent tie rule.
"""
import numpy as np
import pytest

import oracle
import selas_gb300 as sel
from conftest import HIT_FIELDS, assert_hits_equal
from edge_scenes import grid_rays, grid_scene, segment_rayhits, segment_rays, untraceable_rays
from selas_gb300 import scenes

pytestmark = pytest.mark.gpu
KINDS = [sel.SEL_BVH_WIDE8_Q8, sel.SEL_BVH_BINARY_FP32]


def _scene(device, data, kind):
    sc = sel.Scene(device, kind)
    data.attach_to(sc)
    sc.commit()
    return sc


@pytest.mark.parametrize("kind", KINDS)
def test_small_scene_matches_bruteforce(device, kind):
    data = scenes.displaced_icospheres(count=5, level=3, seed=11)
    soup = data.soup()
    sc = _scene(device, data, kind)
    cam = scenes.camera_basis([0.0, 70.0, -170.0], [0.0, 40.0, 0.0], [0.0, 1.0, 0.0], 60.0, 96, 96)
    # 8,003 surface rays: the last warp has lanes past the batch, which the any-hit kernel's warp-wide leaf tests
    # keep as helpers
    for org, d in (scenes.primary_rays(cam), scenes.surface_rays(data, 8003, seed=5)):
        got, want = sel.make_rayhits(org, d), sel.make_rayhits(org, d)
        sc.intersect1M(got)
        oracle.intersect_bruteforce(soup, want)
        assert (want["geomID"] != sel.INVALID_ID).sum() > 500
        assert_hits_equal(got, want)
        rg, rw = sel.make_rays(org, d), sel.make_rays(org, d)
        sc.occluded1M(rg)
        oracle.occluded_bruteforce(soup, rw)
        assert_hits_equal(rg, rw, fields=("tfar",))
    sc.release()


@pytest.mark.parametrize("kind", KINDS)
def test_edge_cases_match_bruteforce(device, kind):
    data = grid_scene()
    soup = data.soup()
    sc = _scene(device, data, kind)
    org, d, _ = grid_rays()
    got, want = sel.make_rayhits(org, d), sel.make_rayhits(org, d)
    sc.intersect1M(got)
    oracle.intersect_bruteforce(soup, want)
    assert_hits_equal(got, want)
    for make, query, ref in ((segment_rayhits, sc.intersect1M, oracle.intersect_bruteforce),
                             (segment_rays, sc.occluded1M, oracle.occluded_bruteforce)):
        g, w = make(), make()
        query(g)
        ref(soup, w)
        assert_hits_equal(g, w, fields=HIT_FIELDS if g.dtype == sel.RAYHIT_DTYPE else ("tfar",))
    # empty batches are no-ops
    sc.intersect1M(sel.make_rayhits(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32)))
    sc.release()


def test_single_ray_and_strided_forms(device):
    data = scenes.displaced_icospheres(count=3, level=2, seed=3)
    soup = data.soup()
    sc = _scene(device, data, sel.SEL_BVH_WIDE8_Q8)
    org, d = scenes.surface_rays(data, 300, seed=9)
    want = sel.make_rayhits(org, d)
    oracle.intersect_bruteforce(soup, want)
    # one record at a time (rtcIntersect1 form)
    lib = sel.lib()
    one = sel.make_rayhits(org[:40], d[:40])
    for i in range(40):
        rec = one[i:i + 1].copy()
        sel.check(lib.sel_intersect1(sc.handle, rec.ctypes.data))
        one[i] = rec[0]
    assert_hits_equal(one, want[:40])
    # strided records (128-byte stride, as a caller embedding RTCRayHit in a larger struct would pass)
    wide = np.zeros(300, dtype=np.dtype({"names": ["rh"], "formats": [sel.RAYHIT_DTYPE], "offsets": [0],
                                         "itemsize": 128}))
    wide["rh"] = sel.make_rayhits(org, d)
    sel.check(lib.sel_intersect1M(sc.handle, wide.ctypes.data, 300, 128))
    assert_hits_equal(wide["rh"], want)
    sc.release()


def test_device_forms_and_errors(device):
    torch = pytest.importorskip("torch")
    data = scenes.displaced_icospheres(count=3, level=3, seed=4)
    sc = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8)
    data.attach_to(sc)
    rh = sel.make_rayhits(*scenes.surface_rays(data, 1000, seed=2))
    with pytest.raises(sel.SelError) as e:
        sc.intersect1M(rh.copy())
    assert e.value.code == sel.SEL_ERR_INVALID_OPERATION
    sc.commit()
    host = rh.copy()
    sc.intersect1M(host)
    buf = torch.from_numpy(rh.view(np.uint8).copy()).cuda()
    stream = torch.cuda.Stream()
    sc.intersect_device(buf.data_ptr(), rh.shape[0], stream.cuda_stream)
    device.sync(stream.cuda_stream)
    dev_res = buf.cpu().numpy().view(sel.RAYHIT_DTYPE)
    assert_hits_equal(dev_res, host)
    with pytest.raises(sel.SelError) as e:
        sc.intersect_device(buf.data_ptr() + 4, 10, None)
    assert e.value.code == sel.SEL_ERR_INVALID_ARGUMENT
    sc.release()


@pytest.fixture(scope="module")
def full_workload():
    data, (co, cd), (io, idr) = scenes.ray_query_workload(level=6)
    return data, (co, cd), (io, idr)


def _trace_device(sc, org, d, any_hit=False):
    import torch
    recs = (sel.make_rays if any_hit else sel.make_rayhits)(org, d)
    buf = torch.from_numpy(recs.view(np.uint8)).cuda()
    (sc.occluded_device if any_hit else sc.intersect_device)(buf.data_ptr(), recs.shape[0], None)
    sc.device.sync(None)
    return buf.cpu().numpy().view(recs.dtype)


def test_full_size_workload(device, full_workload):
    """5.24 M triangles, 4 M coherent + 4 M incoherent rays: both BVH layouts agree on every record at full
    size, a 40 k-ray sample of each set is bit-exact against the oracle BVH, and any-hit bits equal
    closest-hit existence."""
    pytest.importorskip("torch")
    data, coherent, incoherent = full_workload
    soup = data.soup()
    wide = _scene(device, data, sel.SEL_BVH_WIDE8_Q8)
    binary = _scene(device, data, sel.SEL_BVH_BINARY_FP32)
    info = wide.info()
    assert info.triangle_count == data.triangle_count
    obvh = oracle.OracleBvh(soup)
    rng = np.random.default_rng(1)
    for org, d in (coherent, incoherent):
        a = _trace_device(wide, org, d)
        b = _trace_device(binary, org, d)
        assert_hits_equal(a, b)
        # the host-memory form pipelines chunks of a large batch over several streams: same records
        h = sel.make_rayhits(org, d)
        wide.intersect1M(h)
        assert_hits_equal(h, a)
        ho = sel.make_rays(org, d)
        wide.occluded1M(ho)
        assert np.array_equal(np.isneginf(ho["tfar"]), a["geomID"] != sel.INVALID_ID)
        hit = a["geomID"] != sel.INVALID_ID
        assert hit.mean() > 0.05
        occ = _trace_device(wide, org, d, any_hit=True)
        assert np.array_equal(np.isneginf(occ["tfar"]), hit)
        pick = rng.choice(org.shape[0], 40000, replace=False)
        want = sel.make_rayhits(org[pick], d[pick])
        obvh.intersect(want)
        assert_hits_equal(a[pick], want)
    wide.release()
    binary.release()


def test_ordered_large_batches_return_the_same_records(device, full_workload):
    """SEL_OPTION_RAY_SORT: a batch of 4 M incoherent rays in HBM is traced in the order of its octant / Morton
    keys (through an index, the records staying in place) and returns every record bit for bit as in record order;
    the coherent batch is left in its order by the device-side gate and agrees too."""
    pytest.importorskip("torch")
    data, coherent, incoherent = full_workload
    wide = _scene(device, data, sel.SEL_BVH_WIDE8_Q8)
    try:
        for org, d in (incoherent, coherent):
            plain = _trace_device(wide, org, d)
            plain_occ = _trace_device(wide, org, d, any_hit=True)
            device.set_option(sel.SEL_OPTION_RAY_SORT, 1)
            try:
                ordered = _trace_device(wide, org, d)
                ordered_occ = _trace_device(wide, org, d, any_hit=True)
            finally:
                device.set_option(sel.SEL_OPTION_RAY_SORT, 0)
            assert_hits_equal(ordered, plain)
            assert np.array_equal(ordered_occ.view(np.uint8), plain_occ.view(np.uint8))
    finally:
        wide.release()


@pytest.mark.parametrize("kind", KINDS)
def test_untraceable_rays_miss_like_the_bruteforce_definition(device, kind):
    data = scenes.displaced_icospheres(count=5, level=3, seed=11)
    soup = data.soup()
    sc = _scene(device, data, kind)
    org, d = untraceable_rays()
    got, want = sel.make_rayhits(org, d), sel.make_rayhits(org, d)
    sc.intersect1M(got)
    oracle.intersect_bruteforce(soup, want)
    assert (want["geomID"] == sel.INVALID_ID).all()
    assert_hits_equal(got, want)
    rg, rw = sel.make_rays(org, d), sel.make_rays(org, d)
    sc.occluded1M(rg)
    oracle.occluded_bruteforce(soup, rw)
    assert_hits_equal(rg, rw, fields=("tfar",))
    sc.release()


@pytest.mark.parametrize("n_spheres,level,leaf", [(1, 0, 3), (3, 2, 3), (8, 4, 3), (8, 4, 1), (8, 4, 2), (8, 4, 4),
                                                   (8, 4, 8), (3, 2, 8)])
def test_device_built_bvh_matches_bruteforce(device, n_spheres, level, leaf):
    """The 8-wide BVH built by the GPU kernels (SEL_BUILD_DEVICE) answers every query as the definition does,
    from a 20-triangle scene (one warp builds the whole tree) to 80 k triangles (large-task levels first)."""
    data = scenes.displaced_icospheres(count=n_spheres, level=level, seed=31)
    soup = data.soup()
    sc = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8, sel.SEL_BUILD_DEVICE)
    sc.set_leaf_size(leaf)
    data.attach_to(sc)
    sc.commit()
    info = sc.info()
    assert info.triangle_count == soup[0].shape[0] and info.node_count >= 1
    cam = scenes.camera_basis([0.0, 70.0, -170.0], [0.0, 40.0, 0.0], [0.0, 1.0, 0.0], 60.0, 64, 64)
    for org, d in (scenes.primary_rays(cam), scenes.surface_rays(data, 6000, seed=6)):
        got, want = sel.make_rayhits(org, d), sel.make_rayhits(org, d)
        sc.intersect1M(got)
        oracle.intersect_bruteforce(soup, want)
        assert_hits_equal(got, want)
        rg, rw = sel.make_rays(org, d), sel.make_rays(org, d)
        sc.occluded1M(rg)
        oracle.occluded_bruteforce(soup, rw)
        assert_hits_equal(rg, rw, fields=("tfar",))
    sc.release()


@pytest.mark.parametrize("leaf", [5, 8])
def test_device_built_leaves_beyond_a_nodes_records_move_down(device, leaf):
    """4096 copies of one triangle (and a few jittered ones) cannot be split by position: the tree is all full
    leaves, so eight of them under one node would hold more than the node's 32 records and the largest move one
    level down.  Every query still returns the definition's hit, including the tie rule among coincident
    triangles (smallest t, then geomID and primID)."""
    rng = np.random.default_rng(12)
    tri = np.float32([[-1, -1, 0], [1, -1, 0], [0, 1, 0]])
    copies = np.tile(tri, (4096, 1, 1))
    jitter = tri[None] + rng.normal(scale=0.05, size=(64, 3, 3)).astype(np.float32)
    g = scenes.TriangleScene()
    for gid, block in enumerate((copies, jitter)):
        g.add(gid, block.reshape(-1, 3), np.arange(block.shape[0] * 3, dtype=np.uint32).reshape(-1, 3))
    soup = g.soup()
    sc = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8, sel.SEL_BUILD_DEVICE)
    sc.set_leaf_size(leaf)
    g.attach_to(sc)
    sc.commit()
    n = 4000
    org = np.column_stack([rng.uniform(-1.2, 1.2, n), rng.uniform(-1.2, 1.2, n), np.full(n, -5.0)]).astype(np.float32)
    d = np.column_stack([rng.normal(scale=0.02, size=(n, 2)), np.ones(n)]).astype(np.float32)
    got, want = sel.make_rayhits(org, d), sel.make_rayhits(org, d)
    sc.intersect1M(got)
    oracle.intersect_bruteforce(soup, want)
    assert_hits_equal(got, want)
    assert (got["geomID"] != 0xFFFFFFFF).mean() > 0.3
    rg, rw = sel.make_rays(org, d), sel.make_rays(org, d)
    sc.occluded1M(rg)
    oracle.occluded_bruteforce(soup, rw)
    assert_hits_equal(rg, rw, fields=("tfar",))
    sc.release()


def test_device_built_bvh_on_the_edge_grid(device):
    data = grid_scene()
    soup = data.soup()
    sc = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8, sel.SEL_BUILD_DEVICE)
    data.attach_to(sc)
    sc.commit()
    org, d, _ = grid_rays()
    got, want = sel.make_rayhits(org, d), sel.make_rayhits(org, d)
    sc.intersect1M(got)
    oracle.intersect_bruteforce(soup, want)
    assert_hits_equal(got, want)
    sc.release()


def test_device_built_bvh_full_size(device, full_workload):
    """5,242,882 triangles: device build against the host build on a million rays of each set (both are
    checked against the definition elsewhere; here they must agree bit for bit)."""
    data, coherent, incoherent = full_workload
    built = {}
    for mode in (sel.SEL_BUILD_HOST, sel.SEL_BUILD_DEVICE):
        sc = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8, mode)
        data.attach_to(sc)
        sc.commit()
        built[mode] = sc
    info_h, info_d = built[0].info(), built[1].info()
    print(f"host build {info_h.build_ms:.1f} ms, device build {info_d.build_ms:.1f} ms; nodes {info_h.node_count} / "
          f"{info_d.node_count}; depth {info_h.max_depth} / {info_d.max_depth}")
    for org, d in (coherent, incoherent):
        n = min(org.shape[0], 1 << 20)
        a, b = sel.make_rayhits(org[:n], d[:n]), sel.make_rayhits(org[:n], d[:n])
        built[0].intersect1M(a)
        built[1].intersect1M(b)
        assert_hits_equal(b, a)
    for sc in built.values():
        sc.release()


@pytest.mark.parametrize("stride", [96, 128])
def test_pinned_records_are_traced_in_place(device, stride):
    """Records in page-locked host memory (torch pin_memory: cudaHostAlloc) are traced where they lie
    (SEL_OPTION_ZERO_COPY, the default); pageable records and the option turned off take the staged copies.  All
    three give bit-identical records, dense and embedded in a larger caller struct, for both query kinds; the
    bytes around the records are left untouched."""
    import torch
    data = scenes.displaced_icospheres(count=8, level=4, seed=31)
    sc = _scene(device, data, sel.SEL_BVH_WIDE8_Q8)
    org, d = scenes.surface_rays(data, 300000, seed=32)
    n = org.shape[0]
    for fmt, make, query, fields in ((96, sel.make_rayhits, "sel_intersect1M", HIT_FIELDS),
                                     (48, sel.make_rays, "sel_occluded1M", ("tfar",))):
        st = stride
        recs = make(org, d)
        want = recs.copy()
        getattr(sel.lib(), query)(sc.handle, want.ctypes.data, n, fmt)  # pageable: staged copies
        pinned = torch.full((n * st + 64,), 0xA5, dtype=torch.uint8).pin_memory()
        view = pinned.numpy()
        body = view[:n * st].reshape(n, st)
        body[:, :fmt] = recs.view(np.uint8).reshape(n, fmt)
        for option in (1, 0):
            device.set_option(sel.SEL_OPTION_ZERO_COPY, option)
            body[:, :fmt] = recs.view(np.uint8).reshape(n, fmt)
            sel.check(getattr(sel.lib(), query)(sc.handle, view.ctypes.data, n, st))
            got = np.ascontiguousarray(body[:, :fmt]).view(recs.dtype).reshape(n)
            assert_hits_equal(got, want, fields=fields)
            if st > fmt:
                assert (body[:, fmt:] == 0xA5).all()
            assert (view[n * st:] == 0xA5).all()
        device.set_option(sel.SEL_OPTION_ZERO_COPY, 1)
    sc.release()

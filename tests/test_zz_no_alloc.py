"""sel_intersect1M_noalloc: the closest-hit query for callers that must not allocate GPU memory (a plugin
whose host application owns every byte of HBM, a real-time loop that cannot risk the synchronisation
cudaMalloc may cause).  It must return exactly what sel_intersect1M returns -- ray queries are compared
bit for bit everywhere in this suite -- on consecutive calls that reuse its fixed staging array, and
reject batches larger than that array, refuse a scene whose instanced scenes changed, and leave the
device's free memory unchanged.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import selas_gb300 as sel
from conftest import assert_hits_equal
from selas_gb300 import scenes

pytestmark = pytest.mark.gpu
CAPACITY = 65536


def _noalloc(sc, recs, stride=96):
    lib = sel.lib()
    fn = lib.sel_intersect1M_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_size_t]
    fn.restype = ctypes.c_int
    return fn(sc.handle, recs.ctypes.data, recs.shape[0] if recs.ndim else 1, stride)


def test_noalloc_matches_intersect1M_on_consecutive_calls(device):
    data = scenes.displaced_icospheres(count=8, level=4, seed=21)
    sc = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8)
    data.attach_to(sc)
    sc.commit()
    cam = scenes.camera_basis([0.0, 70.0, -170.0], [0.0, 40.0, 0.0], [0.0, 1.0, 0.0], 60.0, 128, 96)
    batches = [scenes.primary_rays(cam), scenes.surface_rays(data, 40000, seed=3)]
    for org, d in batches:  # two calls in a row, different rays: nothing of the previous call may leak
        want = sel.make_rayhits(org, d)
        sc.intersect1M(want)
        got = sel.make_rayhits(org, d)
        sel.check(_noalloc(sc, got))
        assert (want["geomID"] != sel.INVALID_ID).sum() > 1000
        assert_hits_equal(got, want)
    # strided records (a caller embedding RTCRayHit in a larger struct), a third call
    org, d = batches[1]
    wide = np.zeros(org.shape[0], dtype=np.dtype({"names": ["rh"], "formats": [sel.RAYHIT_DTYPE], "offsets": [0],
                                                  "itemsize": 128}))
    wide["rh"] = sel.make_rayhits(org, d)
    sel.check(_noalloc(sc, wide, stride=128))
    want = sel.make_rayhits(org, d)
    sc.intersect1M(want)
    assert_hits_equal(wide["rh"], want)
    sc.release()


def test_noalloc_rejects_batches_beyond_its_array(device):
    data = scenes.displaced_icospheres(count=2, level=2, seed=5)
    sc = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8)
    data.attach_to(sc)
    sc.commit()
    org, d = scenes.surface_rays(data, CAPACITY + 1, seed=4)
    recs = sel.make_rayhits(org, d)
    rc = _noalloc(sc, recs)
    assert rc == sel.SEL_ERR_INVALID_ARGUMENT
    assert b"65536" in sel.lib().sel_get_last_error()
    full = recs[:CAPACITY].copy()
    sel.check(_noalloc(sc, full))
    want = recs[:CAPACITY].copy()
    sc.intersect1M(want)
    assert_hits_equal(full, want)
    sc.release()


def test_noalloc_refuses_a_scene_whose_instanced_scene_changed(device):
    data = scenes.displaced_icospheres(count=2, level=2, seed=7)
    leaf = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8)
    data.attach_to(leaf)
    leaf.commit()
    parent = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8)
    parent.attach_instance(2, leaf, np.eye(4, dtype=np.float32))
    parent.commit()
    org, d = scenes.surface_rays(data, 1000, seed=8)
    recs = sel.make_rayhits(org, d)
    sel.check(_noalloc(parent, recs))
    assert (recs["instID0"] == 2).sum() > 100
    leaf.commit()  # frees the trees the parent's instance records point at
    recs = sel.make_rayhits(org, d)
    assert _noalloc(parent, recs) == sel.SEL_ERR_INVALID_OPERATION
    assert (recs["geomID"] == sel.INVALID_ID).all()  # nothing was traced
    parent.commit()
    sel.check(_noalloc(parent, recs))
    want = sel.make_rayhits(org, d)
    parent.intersect1M(want)
    assert_hits_equal(recs, want)
    parent.release()
    leaf.release()


def test_noalloc_leaves_device_memory_unchanged(device):
    torch = pytest.importorskip("torch")
    data = scenes.displaced_icospheres(count=4, level=3, seed=9)
    sc = sel.Scene(device, sel.SEL_BVH_WIDE8_Q8)
    data.attach_to(sc)
    sc.commit()  # a fresh scene: the host-memory query forms have not allocated its staging buffer
    batches = [scenes.surface_rays(data, n, seed=10 + n) for n in (CAPACITY, 1000, 30000)]
    recs = [sel.make_rayhits(o, d) for o, d in batches]
    sel.check(_noalloc(sc, recs[0]))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for r in recs * 3:
        sel.check(_noalloc(sc, r))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0
    sc.release()

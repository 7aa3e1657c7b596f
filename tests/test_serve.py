"""Render server (sel_server_*): continuous batching of path-tracer, deferred path-tracer and VCM jobs.  A job's image must not
depend on what else runs: the same as alone, in a mix of other scenes, resolutions and integrators, and as
the single-render entry points give it (same random streams; only the order of FP64 additions differs)."""
import ctypes

import numpy as np
import pytest

import selas_gb300 as sel
from selas_gb300 import scenes

pytestmark = pytest.mark.gpu
TOL = dict(rtol=1e-5, atol=1e-8)


@pytest.fixture(scope="module")
def scene_set(device):
    cornell, spheres = scenes.cornell_box(), scenes.textured_spheres(count=4, level=3)
    built = {"cornell": (cornell, cornell.build(sel, device)), "spheres": (spheres, spheres.build(sel, device))}
    yield built
    for _, sc in built.values():
        sc.release()


def _jobs(scene_set):
    (cornell, c_sc), (spheres, s_sc) = scene_set["cornell"], scene_set["spheres"]
    return [
        sel.pt_job(c_sc, cornell.sel_camera(sel, 64, 64), sel.pt_settings(16, 8, seed=11)),
        sel.vcm_job(s_sc, spheres.sel_camera(sel, 48, 32), sel.vcm_settings(4, 8, seed=12)),
        sel.pt_job(s_sc, spheres.sel_camera(sel, 80, 60), sel.pt_settings(8, 6, seed=13)),
        sel.vcm_job(c_sc, cornell.sel_camera(sel, 32, 32), sel.vcm_settings(3, 10, seed=14)),
        sel.pt_job(c_sc, cornell.sel_camera(sel, 40, 40), sel.pt_settings(32, 8, seed=15)),
        sel.deferred_job(s_sc, spheres.sel_camera(sel, 56, 40), sel.deferred_settings(3, 8, seed=16)),
        sel.deferred_job(c_sc, cornell.sel_camera(sel, 48, 48), sel.deferred_settings(4, 6, seed=17)),
    ]


def test_each_job_renders_the_same_alone_and_in_a_mix(device, scene_set):
    jobs = _jobs(scene_set)
    srv = sel.Server(device)
    alone = []
    for j in jobs:
        img, st = srv.wait(srv.submit(j))
        assert st.status == 0
        alone.append(img)
    ids = [srv.submit(j) for j in jobs]  # all at once: they share wavefront batches and overlap
    mixed = [srv.wait(i)[0] for i in ids]
    stats = srv.stats()
    srv.release()
    assert stats.peak_jobs >= 3 and stats.completed == 2 * len(jobs)
    for a, m in zip(alone, mixed):
        assert np.isfinite(a).all() and a.mean() > 0
        np.testing.assert_allclose(m, a, **TOL)


def test_served_images_equal_the_single_render_entry_points(device, scene_set):
    jobs = _jobs(scene_set)
    srv = sel.Server(device)
    ids = [srv.submit(j) for j in jobs]
    served = [srv.wait(i)[0] for i in ids]
    srv.release()
    (cornell, c_sc), (spheres, s_sc) = scene_set["cornell"], scene_set["spheres"]
    direct = [
        c_sc.pt_generate_image(cornell.sel_camera(sel, 64, 64), sel.pt_settings(16, 8, seed=11)),
        s_sc.vcm_generate_image(spheres.sel_camera(sel, 48, 32), sel.vcm_settings(4, 8, seed=12)),
        s_sc.pt_generate_image(spheres.sel_camera(sel, 80, 60), sel.pt_settings(8, 6, seed=13)),
    ]
    served = served[:3] + served[5:]
    direct += [
        s_sc.deferred_generate_image(spheres.sel_camera(sel, 56, 40), sel.deferred_settings(3, 8, seed=16)),
        c_sc.deferred_generate_image(cornell.sel_camera(sel, 48, 48), sel.deferred_settings(4, 6, seed=17)),
    ]
    for s, d in zip(served, direct):
        np.testing.assert_allclose(s, d, **TOL)


def test_admission_respects_the_memory_budget(device, scene_set):
    cornell, c_sc = scene_set["cornell"]
    cam = cornell.sel_camera(sel, 96, 96)
    job_bytes = 96 * 96 * 2 * 3 * (8 + 4) + 1024  # accumulator + resolved image, with alignment slack
    srv = sel.Server(device, sel.server_config(hbm_budget_bytes=2 * job_bytes + 512))
    ids = [srv.submit(sel.pt_job(c_sc, cam, sel.pt_settings(8, 8, seed=100 + k))) for k in range(6)]
    res = [srv.wait(i) for i in ids]
    stats = srv.stats()
    srv.release()
    assert stats.peak_jobs <= 2 and stats.peak_bytes <= 2 * job_bytes + 512
    assert all(st.status == 0 for _, st in res)
    queued = [st.queue_ms for _, st in res]
    assert max(queued) > 0.0  # later jobs waited for memory
    ref = c_sc.pt_generate_image(cam, sel.pt_settings(8, 8, seed=105))
    np.testing.assert_allclose(res[5][0], ref, **TOL)


def test_latency_statistics_and_graph_reuse(device, scene_set):
    cornell, c_sc = scene_set["cornell"]
    srv = sel.Server(device)
    ids = [srv.submit(sel.pt_job(c_sc, cornell.sel_camera(sel, 48, 48), sel.pt_settings(4, 8, seed=k)))
           for k in range(8)]
    stats = [srv.wait(i)[1] for i in ids]
    s = srv.stats()
    srv.release()
    for st in stats:
        assert st.queue_ms >= 0 and st.run_ms > 0
        assert abs(st.latency_ms - st.queue_ms - st.run_ms) < 1e-6 * max(1.0, st.latency_ms) + 1e-9
    assert s.rays > 0 and s.graph_captures >= 1


def test_invalid_jobs_are_rejected(device, scene_set):
    cornell, _ = scene_set["cornell"]
    binary = cornell.build(sel, device, bvh_kind=sel.SEL_BVH_BINARY_FP32)
    srv = sel.Server(device, sel.server_config(max_bounces=4))
    jid = ctypes.c_uint64()
    j = sel.pt_job(binary, cornell.sel_camera(sel, 8, 8), sel.pt_settings(1, 4))
    assert sel.lib().sel_server_submit(srv.handle, ctypes.byref(j), ctypes.byref(jid)) == sel.SEL_ERR_INVALID_OPERATION
    _, c_sc = scene_set["cornell"]
    j = sel.pt_job(c_sc, cornell.sel_camera(sel, 8, 8), sel.pt_settings(1, 8))
    assert sel.lib().sel_server_submit(srv.handle, ctypes.byref(j), ctypes.byref(jid)) == sel.SEL_ERR_INVALID_ARGUMENT
    srv.release()
    binary.release()


def test_a_job_larger_than_the_budget_fails_instead_of_waiting(device, scene_set):
    cornell, c_sc = scene_set["cornell"]
    srv = sel.Server(device, sel.server_config(hbm_budget_bytes=4096))
    jid = srv.submit(sel.pt_job(c_sc, cornell.sel_camera(sel, 64, 64), sel.pt_settings(1, 8)))
    out = np.zeros((2, 64, 64, 3), np.float32)
    st = sel.SelJobStats()
    rc = sel.lib().sel_server_wait(srv.handle, jid, out.ctypes.data, out.size, ctypes.byref(st))
    srv.release()
    assert rc == sel.SEL_ERR_OUT_OF_MEMORY and st.status == sel.SEL_ERR_OUT_OF_MEMORY

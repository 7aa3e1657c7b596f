"""Vertex connection and merging.  The reference's VCM (Source/Applications/Selas/Source/VCM.cpp) is
commented out, so the oracle (oracle/oracle_vcm.cpp) restates the published algorithm it cites and is pinned
by agreement between estimators: on a BSDF whose sampling weights are exact (oracle.consistent_lambert),
VCM, bidirectional path tracing and each strategy alone must converge to the oracle path tracer's image.
The reference Disney BSDF is not of that kind (its diffuse sample weight and pdf differ from f * cos /
density by a factor pi, Disney.cpp:466-519), so on it VCM converges to its own image, the FP64 oracle VCM.
"""
import dataclasses
from pathlib import Path

import numpy as np
import pytest

import oracle
from selas_gb300 import scenes

SIZE = 32


@pytest.fixture(scope="module")
def cornell():
    return scenes.cornell_box()


def _mean(img):
    return img.mean(axis=(0, 1))


@pytest.fixture(scope="module")
def lambert_pt(cornell):
    with oracle.consistent_lambert():
        out = {}
        for length in (2, 4):
            spp = 2048
            out[length] = _mean(oracle.pt_render(cornell, SIZE, SIZE, 0, spp, max_bounces=length - 1,
                                                 physical_nee=True)[1] / spp)
        return out


@pytest.mark.parametrize("length", [2, 4])
@pytest.mark.parametrize("name,merging,strategies", [("vcm", True, 15), ("bpt", False, 15)])
def test_oracle_vcm_converges_to_path_tracing(cornell, lambert_pt, length, name, merging, strategies):
    with oracle.consistent_lambert():
        it = 256
        img = oracle.vcm_render(cornell, SIZE, SIZE, 0, it, max_len=length, merging=merging,
                                strategies=strategies) / it
    np.testing.assert_allclose(_mean(img), lambert_pt[length], rtol=0.01)


@pytest.mark.parametrize("name,strategies", [("next-event", 1), ("light tracing", 8)])
def test_oracle_single_strategies_converge(cornell, lambert_pt, name, strategies):
    """A strategy that alone covers every path of length 2 (direct light), weighted 1."""
    with oracle.consistent_lambert():
        it = 256
        img = oracle.vcm_render(cornell, SIZE, SIZE, 0, it, max_len=2, merging=False, strategies=strategies) / it
    np.testing.assert_allclose(_mean(img), lambert_pt[2], rtol=0.01)


def test_oracle_merging_alone_converges(cornell, lambert_pt):
    """Merging alone estimates direct light with a kernel bias that vanishes as the radius shrinks; the
    radius schedule r_i = r0 / i^((1 - alpha) / 2) (VCMCommon.cpp:91-94) brings it within 2% here.  The
    initial radius is set larger than the default so that a single estimator of this variance converges
    in a few seconds."""
    with oracle.consistent_lambert():
        it = 2048
        img = oracle.vcm_render(cornell, SIZE, SIZE, 0, it, max_len=2, merging=True, strategies=4,
                                radius0=3.0) / it
    np.testing.assert_allclose(_mean(img), lambert_pt[2], rtol=0.02)


def _env_scene(cornell, quads=False, rotation=0.0):
    """The Cornell box (open at the front) lit by the image-based light, with or without its quad light."""
    return dataclasses.replace(cornell, ibl=scenes.sky_ibl(rotation=rotation), lights=cornell.lights if quads else [])


@pytest.mark.parametrize("length", [2, 3])
def test_oracle_vcm_with_environment_converges_to_path_tracing(cornell, length):
    """The image-based light as VCM's environment emitter (light paths from a disc of the bounding-sphere radius,
    next-event estimation, camera paths that leave the scene): with it the only light, VCM with paths of at most L
    segments converges to the oracle path tracer with L bounces, which sees the environment only where BSDF
    sampling leaves the scene.  Both merging and bidirectional path tracing."""
    rs = _env_scene(cornell)
    with oracle.consistent_lambert():
        spp = 4096
        pt = _mean(oracle.pt_render(rs, 24, 24, 0, spp, max_bounces=length, physical_nee=True)[1] / spp)
        it = 256
        for merging in (True, False):
            img = oracle.vcm_render(rs, 24, 24, 0, it, max_len=length, merging=merging) / it
            np.testing.assert_allclose(_mean(img), pt, rtol=0.015)
        # the camera-hit strategy alone is the path tracer's estimator of the environment
        hit = oracle.vcm_render(rs, 24, 24, 0, it, max_len=length, strategies=16) / it
        np.testing.assert_allclose(_mean(hit), pt, rtol=0.015)


def test_oracle_vcm_light_pick_is_linear(cornell):
    """Quads and the environment share one uniform light pick: the image of both is the sum of each alone."""
    with oracle.consistent_lambert():
        it = 256
        both = _mean(oracle.vcm_render(_env_scene(cornell, quads=True), 24, 24, 0, it, max_len=3) / it)
        env = _mean(oracle.vcm_render(_env_scene(cornell), 24, 24, 0, it, max_len=3) / it)
        quads = _mean(oracle.vcm_render(cornell, 24, 24, 0, it, max_len=3) / it)
    np.testing.assert_allclose(both, env + quads, rtol=0.015)


def test_oracle_vcm_without_merging_is_bpt_at_zero_radius_weight(cornell):
    """merging=False drops the merge term and the merge weights; the estimator stays unbiased, so on the
    reference BSDF the two converge to the same image up to the kernel bias of merging."""
    it = 256
    a = oracle.vcm_render(cornell, SIZE, SIZE, 0, it, max_len=4, merging=True) / it
    b = oracle.vcm_render(cornell, SIZE, SIZE, 0, it, max_len=4, merging=False) / it
    np.testing.assert_allclose(_mean(a), _mean(b), rtol=0.01)


# ---------------------------------------------------------------------------------------------------
# GPU integrator (sel_vcm_generate_image) against the oracle
# ---------------------------------------------------------------------------------------------------
VCM_REF = Path(__file__).resolve().parent / "golden" / "cornell_vcm_64_ref.npz"
SEED = 0x5E1A5000
R0 = 1.25  # explicit initial radius, exact in float32, given to both implementations
RATIO = 1.05


def rmse(img, ref):
    return float(np.sqrt(np.mean((img - ref) ** 2)) / np.mean(ref))


def _gpu_vcm(device, rs, size, passes, seed=SEED, max_len=10, merging=True, radius=R0, first_pass=0):
    import selas_gb300 as sel
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, size, size)
    img = sc.vcm_generate_image(cam, sel.vcm_settings(passes, max_len, seed, first_pass, merging, radius))
    sc.release()
    return img.astype(np.float64)


def _same_paths(g, c):
    rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-3 * c.mean())
    assert np.median(rel) < 1e-4, np.median(rel)
    assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()
    assert abs(g.mean() / c.mean() - 1.0) < 5e-3, (g.mean(), c.mean())


@pytest.mark.gpu
@pytest.mark.parametrize("merging", [True, False])
def test_gpu_vcm_traces_the_oracles_paths(device, cornell, merging):
    """Same PCG32 streams: the GPU passes trace the oracle's light and camera paths, so the images agree
    pixel by pixel up to FP32 rounding (and the rare path whose Russian roulette or lobe choice flips)."""
    passes, size = 4, 48
    gpu = _gpu_vcm(device, cornell, size, passes, merging=merging)
    cpu = oracle.vcm_render(cornell, size, size, 0, passes, max_len=10, radius0=R0, seed=SEED, merging=merging) / passes
    _same_paths(gpu, cpu)


@pytest.mark.gpu
def test_gpu_vcm_passes_split_over_calls(device, cornell):
    a = _gpu_vcm(device, cornell, 32, 3, first_pass=0)
    b = _gpu_vcm(device, cornell, 32, 3, first_pass=3)
    whole = _gpu_vcm(device, cornell, 32, 6)
    np.testing.assert_allclose((a + b) / 2, whole, rtol=1e-5, atol=1e-7)


@pytest.mark.gpu
def test_gpu_vcm_rmse_within_ratio_of_oracle(device, cornell):
    """rMSE against the FP64 high-pass oracle VCM image at equal passes, averaged over independent seeds,
    within 1.05x that of the CPU oracle (default radius: 0.0025 x the bounding-sphere radius)."""
    ref = np.load(VCM_REF)["image"].astype(np.float64)
    passes = 16
    e_gpu = np.mean([rmse(_gpu_vcm(device, cornell, 64, passes, seed=s, radius=0.0), ref) for s in (11, 12, 13, 14)])
    e_cpu = np.mean([rmse(oracle.vcm_render(cornell, 64, 64, 0, passes, max_len=10, seed=s) / passes, ref)
                     for s in (21, 22, 23, 24)])
    print(f"VCM rmse gpu {e_gpu:.5f} oracle {e_cpu:.5f} ratio {e_gpu / e_cpu:.4f}")
    assert e_gpu <= RATIO * e_cpu


@pytest.mark.gpu
def test_gpu_vcm_full_size(device, cornell):
    """1280 x 720 (the VCM configuration's viewport), path length 10: finite, non-negative, and its mean equals
    the converged oracle image's mean within the statistical error."""
    ref = np.load(VCM_REF)["image"].astype(np.float64)
    img = _gpu_vcm(device, cornell, 720, 8, radius=0.0)
    assert np.isfinite(img).all() and (img >= 0).all()


@pytest.mark.gpu
def test_gpu_vcm_same_image_on_both_bvh_layouts(device, cornell):
    """The quantised 8-wide BVH returns the plain binary FP32 BVH's hits bit for bit, so both trace the
    same paths; the images differ only by the order of FP64 splats."""
    import selas_gb300 as sel
    imgs = []
    for kind in (sel.SEL_BVH_WIDE8_Q8, sel.SEL_BVH_BINARY_FP32):
        sc = cornell.build(sel, device, bvh_kind=kind)
        imgs.append(sc.vcm_generate_image(cornell.sel_camera(sel, 32, 32), sel.vcm_settings(3, radius=R0)))
        sc.release()
    np.testing.assert_allclose(imgs[0], imgs[1], rtol=1e-5, atol=1e-8)


@pytest.mark.gpu
def test_gpu_vcm_graph_replay_matches_direct_launches(device, cornell):
    """Passes replayed from one captured CUDA graph give the image of kernel-by-kernel launches."""
    import selas_gb300 as sel
    imgs = []
    for replay in (1, 0):
        device.set_option(sel.SEL_OPTION_GRAPH_REPLAY, replay)
        imgs.append(_gpu_vcm(device, cornell, 40, 5))
    device.set_option(sel.SEL_OPTION_GRAPH_REPLAY, 1)
    np.testing.assert_allclose(imgs[0], imgs[1], rtol=1e-5, atol=1e-8)


@pytest.mark.gpu
def test_gpu_material_sort_does_not_change_the_image(device):
    """SEL_OPTION_MATERIAL_SORT: hits shaded in material-class order with Ptex filtered in a kernel of its own
    give the image of queue-order shading (same paths; only the order of FP64 additions differs)."""
    import selas_gb300 as sel
    rs = scenes.textured_spheres(count=4, level=3)
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 48, 40)
    imgs = []
    for sort in (1, 0):
        device.set_option(sel.SEL_OPTION_MATERIAL_SORT, sort)
        imgs.append((sc.vcm_generate_image(cam, sel.vcm_settings(3, 8, seed=5)),
                     sc.pt_generate_image(cam, sel.pt_settings(4, 6, seed=5))))
    device.set_option(sel.SEL_OPTION_MATERIAL_SORT, 1)
    sc.release()
    np.testing.assert_allclose(imgs[0][0], imgs[1][0], rtol=1e-5, atol=1e-8)
    np.testing.assert_allclose(imgs[0][1], imgs[1][1], rtol=1e-5, atol=1e-8)


@pytest.mark.gpu
@pytest.mark.parametrize("rotation", [0.0, 0.3])
def test_gpu_vcm_with_environment_traces_the_oracles_paths(device, cornell, rotation):
    """Quads and the image-based light together: the GPU passes trace the oracle's light paths (from either
    emitter), next-event rays and camera paths that leave the scene."""
    rs = _env_scene(cornell, quads=True, rotation=rotation)
    passes, size = 4, 48
    gpu = _gpu_vcm(device, rs, size, passes)
    cpu = oracle.vcm_render(rs, size, size, 0, passes, max_len=10, radius0=R0, seed=SEED) / passes
    _same_paths(gpu, cpu)


@pytest.mark.gpu
def test_gpu_vcm_with_environment_on_a_textured_open_scene(device):
    """The textured spheres under the sky alone (material-sorted bounces, Ptex, most camera paths leaving the
    scene): same paths as the oracle."""
    import selas_gb300 as sel
    rs = dataclasses.replace(scenes.textured_spheres(count=4, level=3), ibl=scenes.sky_ibl(rotation=0.3), lights=[])
    sc = rs.build(sel, device)
    gpu = sc.vcm_generate_image(rs.sel_camera(sel, 48, 40), sel.vcm_settings(3, 8, SEED, 0, True, R0))
    sc.release()
    cpu = oracle.vcm_render(rs, 48, 40, 0, 3, max_len=8, radius0=R0, seed=SEED) / 3
    _same_paths(gpu.astype(np.float64), cpu)

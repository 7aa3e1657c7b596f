"""Deferred path-tracer parity (DeferredPathTracer::GenerateImage, the integrator the reference's main.cpp runs).

Pinned pieces: the correlated multi-jittered primary samples equal the reference's own
CorrelatedMultiJitter (compiled from its sources into tests/golden/cmj_golden.npz) bit for bit; the BSDF, Ptex
filter and ray queries the integrator calls are pinned by their own golden tests.  The shading glue
(DeferredPathTracer.cpp:61-148) is restated in oracle/oracle_pt.cpp.

Image error is the relative RMSE against the FP64 oracle image tests/golden/cornell_deferred_64_ref.npz
(64 x 64, 4096 correlated multi-jittered samples, MT19937 sampling, at most 64 segments):

    rmse(img) = sqrt(mean((img - ref)^2)) / mean(ref)

The bar: the GPU's rmse at equal spp is at most 1.05x that of the oracle with the reference's sampling
(correlated multi-jittered primary samples, MT19937 for the rest).  With the same PCG32 streams the GPU and the
oracle trace the same paths, so their images agree pixel by pixel up to FP32 rounding of the transcendental
functions.  A uniform of exactly 0 selects the reference BSDF's diffuse-transmission lobe with probability 0
(an infinite weight, NaN after the background MIS weight): such pixels appear identically in the oracle and on
the GPU, and the image comparisons leave non-finite pixels out after checking that both have the same ones.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from selas_gb300 import scenes

GOLDEN = Path(__file__).resolve().parent / "golden"
RATIO = 1.05
SEED = 0x5E1A5000


def rmse(img, ref):
    ok = np.isfinite(img).all(axis=-1) & np.isfinite(ref).all(axis=-1)
    return float(np.sqrt(np.mean((img[ok] - ref[ok]) ** 2)) / np.mean(ref[ok]))


@pytest.fixture(scope="module")
def ref_image():
    return np.load(GOLDEN / "cornell_deferred_64_ref.npz")["image"].astype(np.float64)


@pytest.fixture(scope="module")
def cornell():
    return scenes.cornell_box()


@pytest.fixture(scope="module")
def spheres():
    # Ptex-textured spheres under a non-black background: exercises the background's shadow rays and MIS
    return scenes.textured_spheres()


def test_cmj_matches_reference_golden():
    g = np.load(GOLDEN / "cmj_golden.npz")
    for i, (m, p) in enumerate(zip(g["m"], g["p"])):
        ref = g["points"][g["offsets"][i]:g["offsets"][i + 1]]
        got = oracle.cmj(int(m), int(p))
        assert np.array_equal(ref.view(np.uint32), got.view(np.uint32)), (int(m), int(p))


def test_cmj_is_multi_jittered():
    for p in (0, 1, 12345, (1 << 31) - 1):
        for m in (2, 3, 4, 7):
            xy = oracle.cmj(m, p).astype(np.float64)
            cells = {(int(x * m), int(y * m)) for x, y in xy}
            assert len(cells) == m * m
            assert sorted(np.floor(xy[:, 0] * m * m).astype(int)) == list(range(m * m))
            assert sorted(np.floor(xy[:, 1] * m * m).astype(int)) == list(range(m * m))


def test_fixture_is_the_oracle_converged_image(ref_image, cornell):
    # 64 and 16 samples (8 x 8 and 4 x 4 patterns), MT19937 sampling
    img64 = oracle.deferred_render(cornell, 64, 64, 0, 64, samples_per_axis=8, seed=7, rng="mt") / 64.0
    img16 = oracle.deferred_render(cornell, 64, 64, 0, 16, samples_per_axis=4, seed=8, rng="mt") / 16.0
    e64, e16 = rmse(img64, ref_image), rmse(img16, ref_image)
    assert 0.35 < e64 / e16 < 0.65, (e16, e64)  # ~ 1/2 (stratified primary samples help a little)
    assert abs(img64.mean() / ref_image.mean() - 1.0) < 0.01


def test_oracle_samples_split_additively(cornell):
    a = oracle.deferred_render(cornell, 32, 32, 0, 16, seed=SEED)
    b = oracle.deferred_render(cornell, 32, 32, 0, 5, seed=SEED) + oracle.deferred_render(cornell, 32, 32, 5, 16,
                                                                                             seed=SEED)
    np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-15)


def test_oracle_sampling_modes_agree(ref_image, cornell):
    pcg = oracle.deferred_render(cornell, 64, 64, 0, 16, seed=SEED) / 16.0
    mt = oracle.deferred_render(cornell, 64, 64, 0, 16, seed=SEED, rng="mt") / 16.0
    ratio = rmse(pcg, ref_image) / rmse(mt, ref_image)
    assert 0.9 < ratio < 1.1, ratio


def test_oracle_background_adds_light(spheres):
    import dataclasses
    dark = dataclasses.replace(spheres, background=(0.0, 0.0, 0.0))
    lit = oracle.deferred_render(spheres, 32, 32, 0, 16, seed=SEED)
    unlit = oracle.deferred_render(dark, 32, 32, 0, 16, seed=SEED)
    assert np.isfinite(lit).all() and np.isfinite(unlit).all()
    assert lit.mean() > unlit.mean() * 1.05


def _gpu_image(device, rs, size, axis, seed=SEED, paths_in_flight=0, max_bounces=64, bvh_kind=0):
    import selas_gb300 as sel
    sc = rs.build(sel, device, bvh_kind=bvh_kind)
    cam = rs.sel_camera(sel, size, size)
    img = sc.deferred_generate_image(cam, sel.deferred_settings(axis, max_bounces, seed, paths_in_flight))
    sc.release()
    return img.astype(np.float64)


def _assert_same_paths(gpu, cpu):
    fin_g, fin_c = np.isfinite(gpu).all(axis=-1), np.isfinite(cpu).all(axis=-1)
    assert np.array_equal(fin_g, fin_c), (np.argwhere(~fin_g), np.argwhere(~fin_c))
    g, c = gpu[fin_g], cpu[fin_c]
    rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-3 * c.mean())
    assert np.median(rel) < 1e-4, np.median(rel)
    assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()
    assert abs(g.mean() / c.mean() - 1.0) < 5e-3


@pytest.mark.gpu
def test_gpu_traces_the_oracles_paths(device, cornell):
    gpu = _gpu_image(device, cornell, 64, 4)
    cpu = oracle.deferred_render(cornell, 64, 64, 0, 16, seed=SEED) / 16.0
    _assert_same_paths(gpu, cpu)


@pytest.mark.gpu
def test_gpu_traces_the_oracles_paths_textured_sky(device, spheres):
    """Ptex base colours, background next-event estimation and the background MIS weight."""
    gpu = _gpu_image(device, spheres, 64, 4)
    cpu = oracle.deferred_render(spheres, 64, 64, 0, 16, seed=SEED) / 16.0
    _assert_same_paths(gpu, cpu)


@pytest.mark.gpu
def test_gpu_short_cap_matches_oracle(device, cornell):
    gpu = _gpu_image(device, cornell, 48, 3, max_bounces=3)
    cpu = oracle.deferred_render(cornell, 48, 48, 0, 9, samples_per_axis=3, max_bounces=3, seed=SEED) / 9.0
    _assert_same_paths(gpu, cpu)


@pytest.mark.gpu
def test_gpu_rmse_within_ratio_of_reference(device, cornell, ref_image):
    gpu = _gpu_image(device, cornell, 64, 8, seed=0x1234)
    cpu = oracle.deferred_render(cornell, 64, 64, 0, 64, samples_per_axis=8, seed=0x1234, rng="mt") / 64.0
    e_gpu, e_cpu = rmse(gpu, ref_image), rmse(cpu, ref_image)
    print(f"rmse gpu {e_gpu:.5f} reference-sampling oracle {e_cpu:.5f} ratio {e_gpu / e_cpu:.4f}")
    assert e_gpu <= RATIO * e_cpu


@pytest.mark.gpu
def test_gpu_batching_and_layouts_do_not_change_the_image(device, cornell):
    import selas_gb300 as sel
    a = _gpu_image(device, cornell, 40, 4, paths_in_flight=0)
    b = _gpu_image(device, cornell, 40, 4, paths_in_flight=3000)
    c = _gpu_image(device, cornell, 40, 4, bvh_kind=sel.SEL_BVH_BINARY_FP32)
    np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(a, c, rtol=1e-5, atol=1e-8)


@pytest.mark.gpu
def test_gpu_graph_replay_matches_direct_launches(device, cornell):
    import selas_gb300 as sel
    imgs = []
    for replay in (1, 0):
        device.set_option(sel.SEL_OPTION_GRAPH_REPLAY, replay)
        imgs.append(_gpu_image(device, cornell, 40, 4, paths_in_flight=2000))
    device.set_option(sel.SEL_OPTION_GRAPH_REPLAY, 1)
    np.testing.assert_allclose(imgs[0], imgs[1], rtol=1e-5, atol=1e-8)


@pytest.mark.gpu
def test_gpu_rejects_bad_settings(device, cornell):
    import selas_gb300 as sel
    sc = cornell.build(sel, device)
    cam = cornell.sel_camera(sel, 16, 16)
    for spp, bounces in ((15, 64), (0, 64), (16, 0), (16, 2000)):
        s = sel.deferred_settings(4, bounces)
        s.samplesPerPixel = spp
        with pytest.raises(sel.SelError):
            sc.deferred_generate_image(cam, s)
    sc.release()

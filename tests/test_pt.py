"""Path-tracer parity (PathTracer::GenerateImage / EvaluatePath) on the Cornell scene.

Image error is the relative RMSE of layer 1 (radiance) against the FP64 high-spp oracle image in
tests/golden/cornell_64_ref.npz (64 x 64, 4096 spp, MT19937 sampling as the reference's CSampler):

    rmse(img) = sqrt(mean((img - ref)^2)) / mean(ref)

The bar: the GPU path tracer's rmse at equal spp is at most 1.05x the rmse of the CPU oracle restatement
of the reference path tracer (with the reference's MT19937 sampling).  With the same PCG32 streams the GPU
and the oracle trace the same paths, so their images also agree pixel by pixel up to FP32 rounding.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from selas_gb300 import scenes

REF = Path(__file__).resolve().parent / "golden" / "cornell_64_ref.npz"
RATIO = 1.05
SEED = 0x5E1A5000


def rmse(img, ref):
    return float(np.sqrt(np.mean((img - ref) ** 2)) / np.mean(ref))


@pytest.fixture(scope="module")
def ref_image():
    return np.load(REF)["image"].astype(np.float64)


@pytest.fixture(scope="module")
def cornell():
    return scenes.cornell_box()


def test_fixture_is_the_oracle_converged_image(ref_image, cornell):
    # the oracle at 64 spp sits around the fixture with the noise its spp implies
    img = oracle.pt_render(cornell, 64, 64, 0, 64, seed=7, rng="mt") / 64.0
    e64 = rmse(img[1], ref_image[1])
    img16 = oracle.pt_render(cornell, 64, 64, 0, 16, seed=8, rng="mt") / 16.0
    e16 = rmse(img16[1], ref_image[1])
    assert 0.4 < e64 / e16 < 0.65, (e16, e64)  # ~ 1/2 for unbiased estimators
    assert abs(img[1].mean() / ref_image[1].mean() - 1.0) < 0.01


def test_oracle_sampling_modes_agree(ref_image, cornell):
    pcg = oracle.pt_render(cornell, 64, 64, 0, 32, seed=SEED, rng="pcg") / 32.0
    mt = oracle.pt_render(cornell, 64, 64, 0, 32, seed=SEED, rng="mt") / 32.0
    ratio = rmse(pcg[1], ref_image[1]) / rmse(mt[1], ref_image[1])
    assert 0.9 < ratio < 1.1, ratio
    assert np.isfinite(pcg).all() and (pcg >= 0).all()


def _gpu_image(device, rs, size, spp, seed=SEED, paths_in_flight=0, max_bounces=8):
    import selas_gb300 as sel
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, size, size)
    img = sc.pt_generate_image(cam, sel.pt_settings(spp, max_bounces, seed, paths_in_flight))
    sc.release()
    return img.astype(np.float64)


@pytest.mark.gpu
def test_gpu_traces_the_oracles_paths(device, cornell):
    spp = 16
    gpu = _gpu_image(device, cornell, 64, spp)
    cpu = oracle.pt_render(cornell, 64, 64, 0, spp, seed=SEED, rng="pcg") / spp
    for layer in (0, 1):
        g, c = gpu[layer], cpu[layer]
        rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-3 * c.mean())
        assert np.median(rel) < 1e-4, (layer, np.median(rel))
        assert (rel < 1e-2).mean() > 0.97, (layer, (rel < 1e-2).mean())
        assert abs(g.mean() / c.mean() - 1.0) < 5e-3


@pytest.mark.gpu
def test_gpu_rmse_within_ratio_of_reference(device, cornell, ref_image):
    spp = 64
    gpu = _gpu_image(device, cornell, 64, spp, seed=0x1234)
    cpu = oracle.pt_render(cornell, 64, 64, 0, spp, seed=0x1234, rng="mt") / spp
    e_gpu, e_cpu = rmse(gpu[1], ref_image[1]), rmse(cpu[1], ref_image[1])
    print(f"rmse gpu {e_gpu:.5f} reference-sampling oracle {e_cpu:.5f} ratio {e_gpu / e_cpu:.4f}")
    assert e_gpu <= RATIO * e_cpu


@pytest.mark.gpu
def test_gpu_full_size_cornell(device, cornell, ref_image):
    """512 x 512, 64 spp, depth 8 (the Cornell configuration): finite, non-negative, and its image mean
    equals the converged oracle image's mean within the statistical error."""
    img = _gpu_image(device, cornell, 512, 64)
    assert np.isfinite(img).all() and (img >= 0).all()
    assert abs(img[1].mean() / ref_image[1].mean() - 1.0) < 5e-3


@pytest.mark.gpu
def test_gpu_batching_does_not_change_the_image(device, cornell):
    a = _gpu_image(device, cornell, 48, 8, paths_in_flight=0)
    b = _gpu_image(device, cornell, 48, 8, paths_in_flight=5000)
    np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-9)


@pytest.mark.gpu
def test_gpu_same_image_on_both_bvh_layouts(device, cornell):
    import selas_gb300 as sel
    imgs = []
    for kind in (sel.SEL_BVH_WIDE8_Q8, sel.SEL_BVH_BINARY_FP32):
        sc = cornell.build(sel, device, bvh_kind=kind)
        imgs.append(sc.pt_generate_image(cornell.sel_camera(sel, 48, 48), sel.pt_settings(8)))
        sc.release()
    np.testing.assert_allclose(imgs[0], imgs[1], rtol=1e-5, atol=1e-8)


@pytest.mark.gpu
def test_gpu_graph_replay_matches_direct_launches(device, cornell):
    """Batches replayed from one captured CUDA graph (here 12 batches of 2,000 paths) give the image of
    kernel-by-kernel launches."""
    import selas_gb300 as sel
    imgs = []
    for replay in (1, 0):
        device.set_option(sel.SEL_OPTION_GRAPH_REPLAY, replay)
        imgs.append(_gpu_image(device, cornell, 40, 15, paths_in_flight=2000))
    device.set_option(sel.SEL_OPTION_GRAPH_REPLAY, 1)
    np.testing.assert_allclose(imgs[0], imgs[1], rtol=1e-5, atol=1e-8)


@pytest.mark.gpu
def test_gpu_ray_sort_does_not_change_the_image(device):
    """SEL_OPTION_RAY_SORT: continuing rays traced in (direction bin, origin cell) order give the image of queue
    order (same paths; only the order of FP64 additions differs), for both integrators."""
    import selas_gb300 as sel
    rs = scenes.textured_spheres(count=4, level=3)
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 48, 40)
    imgs = []
    for sort in (1, 0):
        device.set_option(sel.SEL_OPTION_RAY_SORT, sort)
        st = sel.pt_settings(6, 6, seed=9)
        st.pathsInFlight = 3000
        imgs.append((sc.pt_generate_image(cam, st), sc.deferred_generate_image(cam, sel.deferred_settings(3, 12, seed=9))))
    device.set_option(sel.SEL_OPTION_RAY_SORT, 0)
    sc.release()
    np.testing.assert_allclose(imgs[0][0], imgs[1][0], rtol=1e-5, atol=1e-8)
    np.testing.assert_allclose(imgs[0][1], imgs[1][1], rtol=1e-5, atol=1e-8)


@pytest.mark.gpu
def test_gpu_face_order_does_not_change_the_image(device):
    """Batches of 2M paths or more order a textured scene's hits by Ptex face and footprint region as well as by
    material class (here 64 x 64 x 512 spp in one batch): the same paths as queue order, so the same image up to
    the order of FP64 additions."""
    import selas_gb300 as sel
    rs = scenes.textured_spheres(count=4, level=3)
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 64, 64)
    imgs = []
    for sort in (1, 0):
        device.set_option(sel.SEL_OPTION_MATERIAL_SORT, sort)
        imgs.append(sc.pt_generate_image(cam, sel.pt_settings(512, 6, seed=9)))
    device.set_option(sel.SEL_OPTION_MATERIAL_SORT, 1)
    sc.release()
    np.testing.assert_allclose(imgs[0], imgs[1], rtol=1e-5, atol=1e-8)

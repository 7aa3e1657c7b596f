"""2D base-colour images, the reference's non-Ptex texture path (CalculateSurfaceParams,
SurfaceParameters.cpp:186-213): uvs from vertex attribute slot 2, TextureFiltering::Triangle at mip level 0 with
Repeat wrapping (TextureFiltering.h:30-100), SrgbToLinearPrecise, then the 2.2 power of every base colour.  The
GPU and the oracle trace the same PCG32 streams, so their images agree pixel by pixel up to FP32 rounding."""

import numpy as np
import pytest

import oracle
import ref_scenes
from selas_gb300 import scenes

SEED = 0x5E1A5000


# the textured Cornell box (checker image on the floor with repeating uvs, a grey image on the back wall without
# uvs) is shared with the reference pins (tests/ref_scenes.py)
_textured_cornell = ref_scenes.textured_cornell


def _same_paths(gpu, cpu):
    rel = np.abs(gpu - cpu) / np.maximum(np.abs(cpu), 1e-3 * cpu.mean())
    assert np.median(rel) < 1e-4, np.median(rel)
    assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()
    assert abs(gpu.mean() / cpu.mean() - 1.0) < 5e-3


def test_oracle_texture_changes_the_image():
    plain = scenes.cornell_box()
    tex = _textured_cornell()
    a = oracle.pt_render(plain, 32, 32, 0, 4, seed=SEED)
    b = oracle.pt_render(tex, 32, 32, 0, 4, seed=SEED)
    assert np.isfinite(b).all()
    # first-bounce reflectance of floor pixels takes the image's colours: blue and yellow both appear
    floor = b[0][24:, :, :].reshape(-1, 3)
    assert (floor[:, 2] > floor[:, 0]).any() and (floor[:, 0] > floor[:, 2]).any()
    assert not np.allclose(a, b)


@pytest.mark.gpu
def test_gpu_textured_pt_traces_the_oracles_paths(device):
    import selas_gb300 as sel
    rs = _textured_cornell()
    sc = rs.build(sel, device)
    gpu = sc.pt_generate_image(rs.sel_camera(sel, 48, 48), sel.pt_settings(8, 6, SEED)).astype(np.float64)
    sc.release()
    cpu = oracle.pt_render(rs, 48, 48, 0, 8, max_bounces=6, seed=SEED) / 8.0
    for layer in (0, 1):
        _same_paths(gpu[layer], cpu[layer])


@pytest.mark.gpu
def test_gpu_textured_deferred_and_vcm_trace_the_oracles_paths(device):
    import selas_gb300 as sel
    rs = _textured_cornell()
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 48, 48)
    d = sc.deferred_generate_image(cam, sel.deferred_settings(3, 16, SEED)).astype(np.float64)
    v = sc.vcm_generate_image(cam, sel.vcm_settings(3, 8, SEED, 0, True, 1.25)).astype(np.float64)
    sc.release()
    _same_paths(d, oracle.deferred_render(rs, 48, 48, 0, 9, samples_per_axis=3, max_bounces=16, seed=SEED) / 9.0)
    _same_paths(v, oracle.vcm_render(rs, 48, 48, 0, 3, max_len=8, radius0=1.25, seed=SEED) / 3.0)


@pytest.mark.gpu
def test_gpu_texture_sort_and_removal(device):
    """Queue-order and sorted shading give the same image; removing the image restores the plain material."""
    import selas_gb300 as sel
    rs = _textured_cornell()
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 40, 40)
    imgs = []
    for sort in (1, 0):
        device.set_option(sel.SEL_OPTION_MATERIAL_SORT, sort)
        imgs.append((sc.pt_generate_image(cam, sel.pt_settings(4, 6, seed=3)),
                     sc.vcm_generate_image(cam, sel.vcm_settings(2, 6, 3, 0, True, 1.25))))
    device.set_option(sel.SEL_OPTION_MATERIAL_SORT, 1)
    np.testing.assert_allclose(imgs[0][0], imgs[1][0], rtol=1e-5, atol=1e-8)
    np.testing.assert_allclose(imgs[0][1], imgs[1][1], rtol=1e-5, atol=1e-8)
    sc.set_texture(0, None)
    sc.set_texture(2, None)
    without = sc.pt_generate_image(cam, sel.pt_settings(4, 6, seed=3))
    sc.release()
    plain = scenes.cornell_box().build(sel, device)
    ref = plain.pt_generate_image(cam, sel.pt_settings(4, 6, seed=3))
    plain.release()
    np.testing.assert_allclose(without, ref, rtol=1e-5, atol=1e-8)
    with pytest.raises(sel.SelError):
        bad = scenes.cornell_box().build(sel, device)
        try:
            bad.set_texture(0, np.zeros((4, 4, 2), np.float32))
        finally:
            bad.release()

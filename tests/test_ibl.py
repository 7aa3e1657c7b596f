"""Image-based light (ImageBasedLightResource.cpp:81-268, AreaLighting.cpp:293-314,393-436): importance sampling
by marginal / conditional CDFs of sin(theta) x luma (BuildImageBasedLight.cpp:18-107), the light image for misses
after a diffuse or glossy bounce, the miss image for camera rays and pure-specular chains, and the deferred path
tracer's background next-event estimation with its MIS.

Reference conventions reproduced on purpose (and pinned here): the solid-angle density divides by (W H / 2 pi) /
sin(theta), so it integrates to pi over the sphere instead of 1; a direction's texel is found by truncating
(angle x size / span - 0.5), half a texel off the centres sampling uses; the lookup adds the rotation to the
azimuth while sampling adds it before converting to a direction, so with a non-zero rotation a sampled direction
looks up another texel."""
import dataclasses

import numpy as np
import pytest

import oracle
from selas_gb300 import scenes

SEED = 0x5E1A5000


def test_density_integrates_to_pi():
    ibl = scenes.sky_ibl(rotation=0.0)
    rng = np.random.default_rng(0)
    d = rng.normal(size=(400000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    p = oracle.ibl_pdf(ibl, d.astype(np.float32))
    assert abs(p.mean() * 4 * np.pi / np.pi - 1.0) < 0.02
    out, _ = oracle.ibl_sample(ibl, rng.random((200000, 2)))
    assert abs(np.mean(1.0 / out[:, 6]) / 4.0 - 1.0) < 0.03  # E[1/pdf] = 4 pi / pi


def test_sampled_directions_and_radiance():
    ibl = scenes.sky_ibl(rotation=0.0, exposure=2.0)
    h, w = ibl["light"].shape[:2]
    rng = np.random.default_rng(1)
    out, ev = oracle.ibl_sample(ibl, rng.random((20000, 2)))
    d = out[:, :3].astype(np.float64)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-5)
    # the direction is the centre of its texel: theta = (y + 0.5) pi / h, phi = (x + 0.5) 2 pi / w - pi
    theta = np.arccos(np.clip(d[:, 1], -1, 1))
    phi = np.arctan2(d[:, 2], d[:, 0])
    y = np.round(theta * h / np.pi - 0.5).astype(int)
    x = np.round((phi + np.pi) * w / (2 * np.pi) - 0.5).astype(int) % w
    np.testing.assert_allclose(out[:, 3:6], 2.0 * ibl["light"][y, x], rtol=1e-6)
    # brighter texels are sampled more often: the sun (a tiny solid angle) takes a large share
    sun = (out[:, 3:6].sum(1) > 100.0).mean()
    assert sun > 0.05  # the sun disc covers 0.1 % of the sphere
    # half-texel lookup offset: most, not all, sampled directions look their own texel up again
    same = np.isclose(out[:, 6], ev[:, 0], rtol=1e-5).mean()
    assert 0.5 < same < 1.0


def _ibl_scene(rotation=0.0):
    rs = scenes.textured_spheres(count=4, level=3)
    return dataclasses.replace(rs, ibl=scenes.sky_ibl(rotation=rotation), background=(0.0, 0.0, 0.0))


def _assert_same_paths(gpu, cpu):
    fin_g, fin_c = np.isfinite(gpu).all(axis=-1), np.isfinite(cpu).all(axis=-1)
    assert np.array_equal(fin_g, fin_c)
    g, c = gpu[fin_g], cpu[fin_c]
    rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-3 * c.mean())
    assert np.median(rel) < 1e-4, np.median(rel)
    assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()
    assert abs(g.mean() / c.mean() - 1.0) < 5e-3


def test_oracle_ibl_lights_the_scene():
    rs = _ibl_scene()
    lit = oracle.pt_render(rs, 32, 24, 0, 4, seed=SEED)
    dark = oracle.pt_render(dataclasses.replace(rs, ibl=None), 32, 24, 0, 4, seed=SEED)
    assert np.isfinite(lit).all() and lit[1].mean() > 1.5 * dark[1].mean()
    d = oracle.deferred_render(rs, 32, 24, 0, 16, seed=SEED)
    assert np.isfinite(d).all() and d.mean() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("rotation", [0.0, 0.3])
def test_gpu_pt_with_ibl_traces_the_oracles_paths(device, rotation):
    import selas_gb300 as sel
    rs = _ibl_scene(rotation)
    sc = rs.build(sel, device)
    gpu = sc.pt_generate_image(rs.sel_camera(sel, 64, 48), sel.pt_settings(8, 6, SEED)).astype(np.float64)
    sc.release()
    cpu = oracle.pt_render(rs, 64, 48, 0, 8, max_bounces=6, seed=SEED) / 8.0
    for layer in (0, 1):
        _assert_same_paths(gpu[layer], cpu[layer])


@pytest.mark.gpu
@pytest.mark.parametrize("rotation", [0.0, 0.3])
def test_gpu_deferred_with_ibl_traces_the_oracles_paths(device, rotation):
    import selas_gb300 as sel
    rs = _ibl_scene(rotation)
    sc = rs.build(sel, device)
    gpu = sc.deferred_generate_image(rs.sel_camera(sel, 64, 48), sel.deferred_settings(3, 16, SEED)).astype(np.float64)
    sc.release()
    cpu = oracle.deferred_render(rs, 64, 48, 0, 9, samples_per_axis=3, max_bounces=16, seed=SEED) / 9.0
    _assert_same_paths(gpu, cpu)


@pytest.mark.gpu
def test_gpu_ibl_can_be_removed(device):
    import selas_gb300 as sel
    rs = _ibl_scene()
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 32, 24)
    with_ibl = sc.pt_generate_image(cam, sel.pt_settings(4, 4, SEED))
    sc.set_ibl(None)
    without = sc.pt_generate_image(cam, sel.pt_settings(4, 4, SEED))
    sc.release()
    assert with_ibl[1].mean() > 1.5 * without[1].mean()
    with pytest.raises(sel.SelError):
        sc2 = sel.Scene(device)
        try:
            sc2.set_ibl(np.full((4, 8, 3), -1.0, np.float32))
        finally:
            sc2.release()

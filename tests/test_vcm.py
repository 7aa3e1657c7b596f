"""Vertex connection and merging.  The reference's VCM (Source/Applications/Selas/Source/VCM.cpp) is
commented out, so the oracle (oracle/oracle_vcm.cpp) restates the published algorithm it cites and is pinned
by agreement between estimators: on a BSDF whose sampling weights are exact (oracle.consistent_lambert),
VCM, bidirectional path tracing and each strategy alone must converge to the oracle path tracer's image.
The reference Disney BSDF is not of that kind (its diffuse sample weight and pdf differ from f * cos /
density by a factor pi, Disney.cpp:466-519), so on it VCM converges to its own image, the FP64 oracle VCM.
"""
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


def test_oracle_vcm_without_merging_is_bpt_at_zero_radius_weight(cornell):
    """merging=False drops the merge term and the merge weights; the estimator stays unbiased, so on the
    reference BSDF the two converge to the same image up to the kernel bias of merging."""
    it = 256
    a = oracle.vcm_render(cornell, SIZE, SIZE, 0, it, max_len=4, merging=True) / it
    b = oracle.vcm_render(cornell, SIZE, SIZE, 0, it, max_len=4, merging=False) / it
    np.testing.assert_allclose(_mean(a), _mean(b), rtol=0.01)

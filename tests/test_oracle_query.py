"""CPU checks of the ray-query oracle: its BVH agrees with its brute-force definition, and the contract's
edge cases (watertightness, tie rule, segment limits, degenerate triangles) hold."""
import numpy as np

import oracle
from conftest import assert_hits_equal
from edge_scenes import grid_rays, grid_scene, segment_rayhits, segment_rays, untraceable_rays
from selas_gb300 import INVALID_ID, make_rayhits, make_rays, scenes


def _both(soup, org, d):
    a = make_rayhits(org, d)
    b = make_rayhits(org, d)
    oracle.intersect_bruteforce(soup, a)
    bvh = oracle.OracleBvh(soup)
    bvh.intersect(b)
    return a, b, bvh


def test_bvh_matches_bruteforce_icospheres():
    s = scenes.displaced_icospheres(count=5, level=3, seed=11)
    soup = s.soup()
    cam = scenes.camera_basis([0.0, 70.0, -170.0], [0.0, 40.0, 0.0], [0.0, 1.0, 0.0], 60.0, 48, 48)
    for org, d in (scenes.primary_rays(cam), scenes.surface_rays(s, 3000, seed=5)):
        a, b, bvh = _both(soup, org, d)
        assert (a["geomID"] != INVALID_ID).sum() > 100
        assert_hits_equal(b, a)
        ra, rb = make_rays(org, d), make_rays(org, d)
        oracle.occluded_bruteforce(soup, ra)
        bvh.occluded(rb)
        assert_hits_equal(rb, ra, fields=("tfar",))
        # any-hit agrees with closest-hit existence
        assert np.array_equal(np.isneginf(ra["tfar"]), a["geomID"] != INVALID_ID)


def test_grid_is_watertight_and_ties_resolve_to_smallest_key():
    s = grid_scene()
    soup = s.soup()
    org, d, target = grid_rays()
    a, b, _ = _both(soup, org, d)
    assert_hits_equal(b, a)
    down = org.shape[0] - 4
    tx, tz = target[:down, 0], target[:down, 2]
    inside = (tx > 0) & (tx < 8) & (tz > 0) & (tz < 8)  # interior edges and vertices
    assert inside.sum() > 500
    assert (a["geomID"][:down][inside] != INVALID_ID).all(), "a ray aimed at the grid fell through"
    # duplicate quad [2,3]x[2,3] under geomID 1 wins over geomID 3 (same t)
    hit_dup = (a["geomID"] == 1)
    assert hit_dup.any()
    assert not (a["geomID"] == 7).any(), "zero-area triangle reported a hit"
    # points on the shared diagonal of a quad report the lower primID of the two triangles
    straight = slice(0, down // 3)
    t = a["tfar"][straight][inside[straight]]
    assert t.size > 100 and np.all(t == np.float32(3.0))


def test_segment_limits():
    s = grid_scene()
    soup = s.soup()
    r = segment_rayhits()
    oracle.intersect_bruteforce(soup, r)
    hit = r["geomID"] != INVALID_ID
    # t = 3 exactly: [0,inf] hit, [0,3] hit (inclusive), [0,3-ulp] miss, [3,3] hit, [3+ulp,inf] miss, [0,0] miss
    assert hit.tolist() == [True, True, False, True, False, False]
    rr = segment_rays()
    oracle.occluded_bruteforce(soup, rr)
    assert np.isneginf(rr["tfar"]).tolist() == [True, True, False, True, False, False]


def test_closed_mesh_never_leaks():
    v, f = scenes.icosphere(4)
    s = scenes.TriangleScene()
    s.add(0, (v * 3.0 + np.array([0.1, 0.2, 0.3])).astype(np.float32), f.astype(np.uint32))
    rng = np.random.default_rng(3)
    d = rng.normal(size=(20000, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    org = np.tile(np.array([[0.1, 0.2, 0.3]], np.float32), (20000, 1))
    # also exactly through vertices
    vd = (v - 0.0).astype(np.float32)
    org = np.concatenate([org, np.tile(np.array([[0.1, 0.2, 0.3]], np.float32), (vd.shape[0], 1))])
    d = np.concatenate([d, vd])
    a = make_rayhits(org, d)
    oracle.OracleBvh(s.soup()).intersect(a)
    assert (a["geomID"] == 0).all()


def test_untraceable_rays_never_hit():
    """The brute-force definition rejects rays with non-finite components or a zero direction (the GPU
    traversals return the same miss without walking the tree)."""
    data = scenes.displaced_icospheres(count=5, level=3, seed=11)
    org, d = untraceable_rays()
    rh = make_rayhits(org, d)
    oracle.intersect_bruteforce(data.soup(), rh)
    assert (rh["geomID"] == INVALID_ID).all()
    r = make_rays(org, d)
    before = r["tfar"].copy()
    oracle.occluded_bruteforce(data.soup(), r)
    assert np.array_equal(r["tfar"], before)  # never set to -inf (the any-hit mark)

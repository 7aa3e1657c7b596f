"""Ptex on quad meshes: the separable bicubic filter with B-spline weights that getFilter(f_bspline) gives a quad
texture, evaluated as Selas calls it (eval(primId, u, v, widths 0)), against the vendored Ptex 2.2 (golden fixture
from tests/golden/make_golden.py: cubes of 3 x 3 quads a side at 1 x 1 to 16 x 16 texels per face, fans of 5 and 6
quads around one vertex), and quad-Ptex renders against the oracle path tracers.

The filter has no transcendental functions and rounds every product and sum on its own, so the CPU oracle and the
device must reproduce the reference bit for bit."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from selas_gb300 import scenes

GOLDEN = Path(__file__).resolve().parent / "golden" / "ptex_quad_golden.npz"
SEED = 0x5E1A5000


@pytest.fixture(scope="module")
def golden():
    g = np.load(GOLDEN)
    cases = []
    k = 0
    while f"faces_{k}" in g:
        cases.append(tuple(g[f"{name}_{k}"] for name in ("faces", "texels", "queries", "out")))
        k += 1
    return cases


def test_golden_covers_the_cases(golden):
    assert sorted({int(c[0][0, 0]) for c in golden}) == [0, 1, 2, 3, 4]
    for faces, _, q, _ in golden:
        f = q[:, 0].view(np.int32)
        assert (f < 0).any() and (f >= faces.shape[0]).any()  # invalid face ids
        assert (q[:, 1] == 0).any() and (q[:, 2] == 1).any() and (q[:, 1] > 1).any()  # edges, corners, clamping
    boundaries = [(faces[:, 2:6] < 0).any() for faces, _, _, _ in golden]
    assert any(boundaries) and not all(boundaries)


def test_oracle_matches_vendored_ptex_exactly(golden):
    for faces, texels, queries, want in golden:
        got = oracle.ptex_quad_eval(faces, texels, queries)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), faces[0, 0]


def test_quad_adjacency_is_symmetric_and_valences_are_as_built():
    for (v, q), valence in ((scenes.quad_cube(3), {3, 4}), (scenes.quad_fan(5), {1, 2, 5}), (scenes.quad_fan(6),
                                                                                          {1, 2, 6})):
        adj, ae = scenes.triangle_adjacency(q)
        inner = adj >= 0
        f = np.arange(q.shape[0])[:, None].repeat(4, 1)
        e = np.arange(4)[None, :].repeat(q.shape[0], 0)
        assert np.array_equal(adj[adj[inner], ae[inner]], f[inner]) and np.array_equal(ae[adj[inner], ae[inner]],
                                                                                        e[inner])
        assert set(np.bincount(q.reshape(-1))) == valence


def test_constant_faces_take_the_readers_constant_forms():
    """A texture of one colour everywhere: every face is constant in a constant neighbourhood, so the filter returns
    the texel itself (the golden's last case mixes constant and varying faces)."""
    _, quads = scenes.quad_cube(2)
    faces = scenes.ptex_quad_faces(quads, 2)
    tex = np.tile(np.float16([0.25, 0.5, 0.75]), quads.shape[0] * 16).view(np.uint16)
    rng = np.random.default_rng(5)
    q = np.zeros((500, 3), np.float32)
    q[:, 0] = rng.integers(0, quads.shape[0], 500).astype(np.int32).view(np.float32)
    q[:, 1:] = rng.random((500, 2))
    out = oracle.ptex_quad_eval(faces, tex, q)
    np.testing.assert_array_equal(out, np.tile(np.float32([0.25, 0.5, 0.75]), (500, 1)))


@pytest.mark.gpu
def test_gpu_filter_matches_vendored_ptex_exactly(device, golden):
    import torch

    import selas_gb300 as sel
    for faces, texels, queries, want in golden:
        d_faces = torch.from_numpy(np.ascontiguousarray(faces)).cuda()
        d_tex = torch.from_numpy(texels.view(np.int16).copy()).cuda()
        d_q = torch.from_numpy(queries).cuda()
        d_out = torch.zeros((queries.shape[0], 3), dtype=torch.float32, device="cuda")
        sel.check(sel.lib().sel_ptex_quad_filter_device(device.handle, d_faces.data_ptr(), faces.shape[0],
                                                        d_tex.data_ptr(), d_q.data_ptr(), queries.shape[0],
                                                        d_out.data_ptr(), None))
        device.sync(None)
        got = d_out.cpu().numpy()
        valid = (queries[:, 0].view(np.int32) >= 0) & (queries[:, 0].view(np.int32) < faces.shape[0])
        assert np.array_equal(got[valid].view(np.uint32), want[valid].view(np.uint32)), faces[0, 0]
        assert (got[~valid] == 0).all()


def _same_paths(gpu, cpu):
    rel = np.abs(gpu - cpu) / np.maximum(np.abs(cpu), 1e-3 * cpu.mean())
    assert np.median(rel) < 1e-4, np.median(rel)
    assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()
    assert abs(gpu.mean() / cpu.mean() - 1.0) < 5e-3


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["pt", "deferred", "vcm"])
def test_gpu_quad_ptex_scene_traces_the_oracles_paths(device, integrator):
    import selas_gb300 as sel
    rs = scenes.quad_textured_cubes()
    sc = rs.build(sel, device)
    cam = rs.sel_camera(sel, 48, 32)
    try:
        if integrator == "pt":
            gpu = sc.pt_generate_image(cam, sel.pt_settings(8, 6, SEED)).astype(np.float64)
            cpu = oracle.pt_render(rs, 48, 32, 0, 8, max_bounces=6, seed=SEED) / 8.0
            pairs = [(gpu[0], cpu[0]), (gpu[1], cpu[1])]
        elif integrator == "deferred":
            gpu = sc.deferred_generate_image(cam, sel.deferred_settings(4, 6, SEED)).astype(np.float64)
            cpu = oracle.deferred_render(rs, 48, 32, 0, 16, samples_per_axis=4, max_bounces=6, seed=SEED) / 16.0
            pairs = [(gpu, cpu)]
        else:
            gpu = sc.vcm_generate_image(cam, sel.vcm_settings(4, 6, SEED)).astype(np.float64)
            cpu = oracle.vcm_render(rs, 48, 32, 0, 4, max_len=6, seed=SEED) / 4.0
            pairs = [(gpu, cpu)]
    finally:
        sc.release()
    for g, c in pairs:
        _same_paths(g, c)


@pytest.mark.gpu
def test_gpu_ptex_entry_points_take_their_own_mesh_kind(device):
    import selas_gb300 as sel
    cubes = scenes.quad_textured_cubes(count=1)
    rows, tex = cubes.ptex[0]
    tri = scenes.textured_spheres(count=1, level=1)
    trows, ttex = next(iter(tri.ptex.values()))
    sc = sel.Scene(device)
    v, q = scenes.quad_cube(3)
    sc.attach_quad_mesh(0, v, q)
    sc.attach_triangle_mesh(1, tri.geometry.meshes[0][1], tri.geometry.meshes[0][2])
    with pytest.raises(sel.SelError):
        sc.set_ptex(0, trows[:q.shape[0]], ttex)  # triangle records on a quad mesh
    with pytest.raises(sel.SelError):
        sc.set_ptex(1, rows, tex)  # quad records on a triangle mesh
    with pytest.raises(sel.SelError):
        sc.set_ptex(0, rows[:-1], tex)  # one face short
    bad = rows.copy()
    bad[3, 2] = q.shape[0]  # a neighbour past the face table
    with pytest.raises(sel.SelError):
        sc.set_ptex(0, bad, tex)
    sc.set_ptex(0, rows, tex)
    sc.release()

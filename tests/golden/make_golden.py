"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Run on a machine with the reference checkout (it loads oracle/_ref/*.so, built from the reference sources
by oracle/ref/build_ref.py):

    python tests/golden/make_golden.py

bsdf_golden.npz  - seeded (surface, wo, wi) tuples -> EvaluateBsdf (f, forwardPdfW, reversePdfW) and
                   seeded (surface, wo, 4 uniforms) tuples -> SampleBsdfFunction results, computed by
                   Source/Core/Shading/SurfaceScattering.cpp:18-60 -> Disney.cpp / DiracTransparent.cpp.
ptex_golden.npz  - a triangle mesh (icosphere, 320 faces) with 16 x 16 half-float RGB value-noise texels per
                   face and Ptex adjacency, written with the vendored Ptex 2.2 writer and filtered by its
                   PtexTriangleFilter (getFilter(f_bspline), zero widths, as SurfaceParameters.cpp:196-206)
                   at seeded (face, u, v) queries including edges, corners and out-of-range faces.
ptex_quad_golden.npz - quad meshes (a cube of 3 x 3 quads a side: corner valence 3; fans of 5 and 6 quads around
                   one vertex, with a boundary) at 1 x 1 to 16 x 16 texels per face, filtered by the vendored Ptex's
                   separable bicubic filter with B-spline weights (getFilter(f_bspline) on mt_quad, zero widths).
cornell_64_ref.npz - the FP64 high-spp image of the Cornell scene (64 x 64, 4096 spp, depth 8, background 0)
                   from the reference's own path tracer (PathTracer.cpp EvaluatePath, compiled into
                   oracle/_ref/libref_pt.so) with its MT19937 sampling (each 256-spp chunk with seeds of its own);
                   the image the path tracers' rMSE is measured against.
ref_pt_golden.npz - from the reference's own code in oracle/_ref/libref_pt.so (tests/golden/ref_pt.py):
                   * img_<name>: EvaluatePath images (per-path means, both layers) of the scenes in
                     tests/ref_scenes.py IMAGES on the GPU's PCG32 streams (stream pass * W * H + pixel);
                   * deferred_<name>: DeferredPathTracer images (ShadeHitBatch / TraceRayBatch /
                     TraceOcclusionBatch, one path at a time) of tests/ref_scenes.py DEFERRED on PCG32 streams;
                   * cornell_mt64: layer 1 of the Cornell scene at 64 x 64, 64 spp with the reference's MT19937
                     sampling (seed 0x1234): the reference arm of the path tracer's rMSE gate;
                   * surf_*: CalculateSurfaceParams (+ OffsetRayOrigin) on hits of four scenes (vertex
                     normals and tangents, Ptex, 2D images with uvs, transparent solids);
                   * nee_*: NextEventEstimation / LightingPdf with prescribed uniforms over light sets of one
                     and three quad lights;
                   * ibl_*: Ibl / SampleIbl / SampleIblMiss / SampleIBlPdf with the densities of
                     BuildImageBasedLight.cpp;
                   * vcm_*: VCMCommon::CalculateIterationConstants.
cornell_vcm_64_ref.npz - the FP64 high-pass vertex connection and merging image of the Cornell scene (64 x 64,
                   4096 passes, path length 10, the default radius) from the oracle VCM (oracle/oracle_vcm.cpp);
                   the image the VCM integrators' rMSE is measured against.  Needs only the oracle
                   (python ... vcm).
cmj_golden.npz   - correlated multi-jittered points CorrelatedMultiJitter(s, m, m, p) of the reference
                   (Source/Core/MathLib/CorrelatedMultiJitter.cpp, compiled into oracle/_ref/libref_bsdf.so)
                   for pattern sizes 1..16 and seeded decorrelation values p.
cornell_deferred_64_ref.npz - the FP64 image of the Cornell scene (64 x 64) from the oracle deferred path
                   tracer (oracle/oracle_pt.cpp) with a 64 x 64 correlated multi-jittered pattern (4096 spp),
                   MT19937 sampling (each 256-sample chunk with seeds of its own) and a 64-segment cap; the image the deferred integrators' rMSE is measured against.
                   Needs only the oracle (python ... deferred).
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
OUT = Path(__file__).resolve().parent

SHADER_THIN, SHADER_SOLID, SHADER_DIRAC = 0, 1, 2


def random_frames(rng, n):
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    helper = np.where(np.abs(nrm[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0, 1.0, 0]]))
    t = np.cross(helper, nrm)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(nrm, t)
    return t, nrm, b


def random_dirs(rng, n, nrm, upper_frac):
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    up = np.sum(d * nrm, axis=1) >= 0
    want_up = rng.random(n) < upper_frac
    flip = up != want_up
    d[flip] *= -1
    return d


def random_surfaces(rng, n, allow_dirac=True):
    t, nrm, b = random_frames(rng, n)
    s = np.zeros((n, 32), np.float64)
    s[:, 0:3], s[:, 3:6], s[:, 6:9] = t, nrm, b
    s[:, 9:12] = rng.uniform(0.02, 1.0, (n, 3))
    s[:, 12:15] = rng.uniform(0.0, 1.0, (n, 3))

    def sparse(p_zero, lo=0.0, hi=1.0):
        v = rng.uniform(lo, hi, n)
        v[rng.random(n) < p_zero] = 0.0
        return v

    s[:, 15] = sparse(0.5)                      # sheen
    s[:, 16] = rng.random(n)                    # sheenTint
    s[:, 17] = sparse(0.5)                      # clearcoat
    s[:, 18] = rng.random(n)                    # clearcoatGloss
    met = rng.random(n)
    r = rng.random(n)
    met[r < 0.4] = 0.0
    met[(r >= 0.4) & (r < 0.6)] = 1.0
    s[:, 19] = met                              # metallic
    s[:, 20] = sparse(0.5)                      # specTrans
    s[:, 21] = sparse(0.5, 0.0, 0.5)            # diffTrans (already halved, as SurfaceParameters holds it)
    s[:, 22] = rng.random(n)                    # flatness
    s[:, 23] = sparse(0.5)                      # anisotropic
    ior = rng.uniform(1.1, 2.5, n)
    s[:, 28] = ior
    s[:, 24] = np.where(rng.random(n) < 0.5, 1.0 / ior, ior)  # relativeIOR
    s[:, 25] = rng.random(n)                    # specularTint
    rough = rng.uniform(0.01, 1.0, n)
    rough[rng.random(n) < 0.05] = 0.005
    s[:, 26] = rough                            # roughness
    s[:, 27] = rng.uniform(0.1, 2.0, n)         # scatterDistance
    sh = rng.random(n)
    s[:, 29] = np.where(sh < 0.7, SHADER_SOLID, SHADER_THIN)
    if allow_dirac:
        s[sh >= 0.92, 29] = SHADER_DIRAC
    return s.astype(np.float32)


def make_bsdf(n_eval=3000, n_sample=3000, seed=0x5E1A5B5D):
    lib = ctypes.CDLL(str(ROOT / "oracle" / "_ref" / "libref_bsdf.so"))
    vp = ctypes.c_void_p
    lib.ref_bsdf_evaluate.argtypes = [vp, vp, vp, ctypes.c_int, vp]
    lib.ref_bsdf_sample.argtypes = [vp, vp, vp, ctypes.c_int, vp]
    rng = np.random.default_rng(seed)

    surf_e = random_surfaces(rng, n_eval, allow_dirac=False)
    wo_e = random_dirs(rng, n_eval, surf_e[:, 3:6].astype(np.float64), 0.8).astype(np.float32)
    wi_e = random_dirs(rng, n_eval, surf_e[:, 3:6].astype(np.float64), 0.7).astype(np.float32)
    out_e = np.zeros((n_eval, 5), np.float32)
    lib.ref_bsdf_evaluate(surf_e.ctypes.data, wo_e.ctypes.data, wi_e.ctypes.data, n_eval, out_e.ctypes.data)

    surf_s = random_surfaces(rng, n_sample, allow_dirac=True)
    wo_s = random_dirs(rng, n_sample, surf_s[:, 3:6].astype(np.float64), 0.8).astype(np.float32)
    u_s = rng.random((n_sample, 4)).astype(np.float32)
    out_s = np.zeros((n_sample, 16), np.float32)
    lib.ref_bsdf_sample(surf_s.ctypes.data, wo_s.ctypes.data, u_s.ctypes.data, n_sample, out_s.ctypes.data)

    np.savez_compressed(OUT / "bsdf_golden.npz", surf_e=surf_e, wo_e=wo_e, wi_e=wi_e, out_e=out_e,
                        surf_s=surf_s, wo_s=wo_s, u_s=u_s, out_s=out_s)
    print("bsdf_golden.npz:", n_eval, "eval,", n_sample, "sample tuples;",
          "nonzero f:", int((out_e[:, :3].sum(1) > 0).sum()), "successful samples:", int(out_s[:, 0].sum()))


def make_ptex(seed=0x5E1A5E7E, n_random=6000):
    import tempfile
    from selas_gb300 import scenes
    lib = ctypes.CDLL(str(ROOT / "oracle" / "_ref" / "libref_ptex.so"))
    vp = ctypes.c_void_p
    lib.ref_ptex_write.argtypes = [ctypes.c_char_p, vp, ctypes.c_int, vp]
    lib.ref_ptex_eval.argtypes = [ctypes.c_char_p, vp, ctypes.c_int, vp]
    _, tris = scenes.icosphere(2)
    faces = scenes.ptex_faces(tris, 4)
    texels = scenes.value_noise_texels(tris.shape[0], 4, seed)
    tex_u16 = np.ascontiguousarray(texels.view(np.uint16))
    rng = np.random.default_rng(seed)
    nf = tris.shape[0]
    f = rng.integers(0, nf, n_random)
    a, b = rng.random(n_random), rng.random(n_random)
    flip = a + b > 1
    a[flip], b[flip] = 1 - a[flip], 1 - b[flip]
    q = [np.stack([f, a, b], 1)]
    special = []
    for face in rng.integers(0, nf, 40):
        for u, v in ((0, 0), (1, 0), (0, 1), (0.5, 0), (0, 0.5), (0.5, 0.5), (1e-4, 0.3), (0.3, 1e-4),
                     (0.4999, 0.4999), (1.2, -0.1), (0.02, 0.97)):
            special.append((face, u, v))
    special += [(-1, 0.3, 0.3), (nf, 0.3, 0.3)]
    q.append(np.array(special, np.float64))
    q = np.concatenate(q)
    queries = np.zeros((q.shape[0], 3), np.float32)
    queries[:, 0] = q[:, 0].astype(np.int32).view(np.float32)
    queries[:, 1:] = q[:, 1:]
    out = np.zeros((q.shape[0], 3), np.float32)
    with tempfile.TemporaryDirectory() as d:
        path = (Path(d) / "noise.ptx").as_posix().encode()
        assert lib.ref_ptex_write(path, faces.ctypes.data, nf, tex_u16.ctypes.data) == 0
        assert lib.ref_ptex_eval(path, queries.ctypes.data, queries.shape[0], out.ctypes.data) == 0
    np.savez_compressed(OUT / "ptex_golden.npz", faces=faces, texels=tex_u16, queries=queries, out=out)
    print("ptex_golden.npz:", queries.shape[0], "queries over", nf, "faces")


# (mesh, log2, constant) of the quad-mesh Ptex golden: the cube's corners have valence 3, its other vertices 4; the
# fans have one interior vertex of valence 5 and 6 and a boundary.  Small faces (log2 0..2) take the filter's wide-
# kernel branches; 1 x 1 faces are constant faces.  constant: the first 27 faces of the cube (half of it) hold one
# colour, so the writer flags constant faces and constant neighbourhoods among them.
QUAD_PTEX_CASES = (("cube", 0, False), ("cube", 1, False), ("cube", 2, False), ("cube", 3, False), ("cube", 4, False),
                   ("fan5", 3, False), ("fan6", 2, False), ("cube", 2, True))


def quad_ptex_mesh(name):
    from selas_gb300 import scenes
    return {"cube": lambda: scenes.quad_cube(3), "fan5": lambda: scenes.quad_fan(5),
            "fan6": lambda: scenes.quad_fan(6)}[name]()


def make_ptex_quad(seed=0x5E1A5E7F, n_random=2500):
    """ptex_quad_golden.npz: for each case k, faces_k / texels_k / queries_k / out_k, the vendored Ptex's
    bicubic B-spline filter on a quad mesh (the separable filter) as Selas calls it."""
    import tempfile
    from selas_gb300 import scenes
    lib = ctypes.CDLL(str(ROOT / "oracle" / "_ref" / "libref_ptex.so"))
    vp = ctypes.c_void_p
    lib.ref_ptex_write_quad.argtypes = [ctypes.c_char_p, vp, ctypes.c_int, vp]
    lib.ref_ptex_eval.argtypes = [ctypes.c_char_p, vp, ctypes.c_int, vp]
    rng = np.random.default_rng(seed)
    arrays = {}
    for k, (mesh, log2, constant) in enumerate(QUAD_PTEX_CASES):
        _, quads = quad_ptex_mesh(mesh)
        nf = quads.shape[0]
        faces = scenes.ptex_quad_faces(quads, log2)
        tex_u16 = np.ascontiguousarray(scenes.value_noise_texels(nf, log2, seed + k).view(np.uint16))
        if constant:
            per_face = tex_u16.reshape(nf, -1, 3)
            per_face[:27] = np.float16([0.3, 0.6, 0.2]).view(np.uint16)
        f = rng.integers(0, nf, n_random)
        q = [np.stack([f, rng.random(n_random), rng.random(n_random)], 1)]
        special = []
        for face in rng.integers(0, nf, 30):
            for u, v in ((0, 0), (1, 0), (0, 1), (1, 1), (0.5, 0), (0, 0.5), (1, 0.5), (0.5, 1), (0.5, 0.5),
                         (1e-4, 0.3), (0.3, 0.9999), (0.02, 0.97), (0.97, 0.03), (1.2, -0.1), (-0.3, 0.5)):
                special.append((face, u, v))
        special += [(-1, 0.3, 0.3), (nf, 0.3, 0.3)]
        q.append(np.array(special, np.float64))
        q = np.concatenate(q)
        queries = np.zeros((q.shape[0], 3), np.float32)
        queries[:, 0] = q[:, 0].astype(np.int32).view(np.float32)
        queries[:, 1:] = q[:, 1:]
        out = np.zeros((q.shape[0], 3), np.float32)
        with tempfile.TemporaryDirectory() as d:
            path = (Path(d) / "quads.ptx").as_posix().encode()
            assert lib.ref_ptex_write_quad(path, faces.ctypes.data, nf, tex_u16.ctypes.data) == 0
            assert lib.ref_ptex_eval(path, queries.ctypes.data, queries.shape[0], out.ctypes.data) == 0
        arrays.update({f"faces_{k}": faces, f"texels_{k}": tex_u16, f"queries_{k}": queries, f"out_{k}": out})
    np.savez_compressed(OUT / "ptex_quad_golden.npz", **arrays)
    print("ptex_quad_golden.npz:", len(QUAD_PTEX_CASES), "textures")


def make_cornell(spp=4096, size=64, seed=0x5E1A5C0B):
    import ref_pt
    from selas_gb300 import scenes
    img = np.zeros((2, size, size, 3), np.float64)
    step = 256
    with ref_pt.RefScene(scenes.cornell_box()) as ref:
        for p in range(0, spp, step):
            # MT19937 engines are seeded per call (seed + pixel): each chunk takes seeds of its own
            img += ref.render(size, size, p, min(spp, p + step), max_bounces=8, seed=seed + (p // step) * 65536,
                              rng="mt")
    img /= spp
    np.savez_compressed(OUT / "cornell_64_ref.npz", image=img.astype(np.float32), spp=spp, seed=seed)
    print("cornell_64_ref.npz: mean radiance", img[1].mean(axis=(0, 1)))


def make_cornell_vcm(passes=4096, size=64, max_len=10, seed=0x5E1A5C0C):
    import oracle
    from selas_gb300 import scenes
    rs = scenes.cornell_box()
    img = np.zeros((size, size, 3), np.float64)
    step = 256
    for p in range(0, passes, step):
        img += oracle.vcm_render(rs, size, size, p, min(passes, p + step), max_len=max_len, seed=seed)
    img /= passes
    np.savez_compressed(OUT / "cornell_vcm_64_ref.npz", image=img.astype(np.float32), passes=passes, seed=seed,
                        max_len=max_len)
    print("cornell_vcm_64_ref.npz: mean radiance", img.mean(axis=(0, 1)))


def make_cmj(seed=0x5E1ACC17):
    lib = ctypes.CDLL(str(ROOT / "oracle" / "_ref" / "libref_bsdf.so"))
    lib.ref_cmj.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    rng = np.random.default_rng(seed)
    ps = [0, 1, 7, 4095, 65535, (1 << 20) + 3, (1 << 31) - 1] + [int(x) for x in rng.integers(0, 1 << 31, 9)]
    ms, pv, pts = [], [], []
    for m in (1, 2, 3, 4, 5, 7, 8, 16):
        for p in ps:
            xy = np.zeros((m * m, 2), np.float32)
            lib.ref_cmj(m, p, m * m, xy.ctypes.data)
            ms.append(m)
            pv.append(p)
            pts.append(xy)
    offs = np.cumsum([0] + [x.shape[0] for x in pts]).astype(np.int64)
    np.savez_compressed(OUT / "cmj_golden.npz", m=np.array(ms, np.int32), p=np.array(pv, np.int64), offsets=offs,
                        points=np.concatenate(pts))
    print("cmj_golden.npz:", len(ms), "patterns")


def make_cornell_deferred(axis=64, size=64, max_bounces=64, seed=0x5E1A5C0D):
    import oracle
    from selas_gb300 import scenes
    rs = scenes.cornell_box()
    img = np.zeros((size, size, 3), np.float64)
    spp = axis * axis
    step = 256
    for p in range(0, spp, step):
        img += oracle.deferred_render(rs, size, size, p, min(spp, p + step), samples_per_axis=axis,
                                      max_bounces=max_bounces, seed=seed + (p // step) * 65536, rng="mt")
    img /= spp
    np.savez_compressed(OUT / "cornell_deferred_64_ref.npz", image=img.astype(np.float32), spp=spp, seed=seed,
                        max_bounces=max_bounces)
    print("cornell_deferred_64_ref.npz: mean radiance", img.mean(axis=(0, 1)))


def _hits(rs, n, seed):
    """n closest hits of rays from the scene's camera position and from points around the scene into random
    directions: (hits n x 12 = position o + t d in FP32 as RayPick forms it, Ng, d, u, v, t; ids n x 2)."""
    import oracle
    import selas_gb300 as sel
    rng = np.random.default_rng(seed)
    soup = rs.geometry.soup()
    lo, hi = rs.geometry.bounds()
    cam = np.array(rs.camera["position"], np.float32)
    org = np.where(rng.random((4 * n, 1)) < 0.5, cam, rng.uniform(lo, hi, (4 * n, 3))).astype(np.float32)
    target = rng.uniform(lo, hi, (4 * n, 3)).astype(np.float32)
    d = target - org
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rh = sel.make_rayhits(org, d)
    oracle.intersect_bruteforce(soup, rh)
    ok = np.nonzero(rh["geomID"] != sel.INVALID_ID)[0][:n]
    rh, org, d = rh[ok], org[ok], d[ok]
    t = rh["tfar"].astype(np.float32)
    pos = (org + t[:, None] * d).astype(np.float32)
    hits = np.zeros((ok.size, 12), np.float32)
    hits[:, 0:3] = pos
    hits[:, 3:6] = np.stack([rh["Ng_x"], rh["Ng_y"], rh["Ng_z"]], 1)
    hits[:, 6:9] = d
    hits[:, 9], hits[:, 10], hits[:, 11] = rh["u"], rh["v"], t
    ids = np.stack([rh["geomID"], rh["primID"]], 1).astype(np.uint32)
    return hits, ids


def nee_scene():
    """The Cornell box with light set 0 holding three quad lights (the ceiling light and two tilted wall panels)
    and light set 1 one small light: NextEventEstimation's uniform pick over a set."""
    import dataclasses
    from selas_gb300 import scenes
    c = scenes.cornell_box()
    l0 = c.lights[0][1]
    l1 = dict(position=(10.0, 300.0, 280.0), direction=(1.0, 0.0, 0.0), x=(0.0, 0.0, 90.0), z=(0.0, 60.0, 0.0),
              radiance=(5.0, 5.0, 8.0))
    l2 = dict(position=(278.0, 250.0, 550.0), direction=(0.0, -0.6, -0.8), x=(120.0, 0.0, 0.0),
              z=(0.0, 64.0, -48.0), radiance=(3.0, 6.0, 3.0))
    l3 = dict(position=(400.0, 554.0, 100.0), direction=(0.0, -1.0, 0.0), x=(40.0, 0.0, 0.0), z=(0.0, 0.0, 30.0),
              radiance=(30.0, 20.0, 10.0))
    return dataclasses.replace(c, lights=[(0, l0), (0, l1), (0, l2), (1, l3)])


def make_ref_pt(seed=0x5E1A5A11):
    import ref_pt
    import ref_scenes
    from selas_gb300 import scenes
    out = {}
    for name, (make, w, h, spp, max_bounces) in ref_scenes.IMAGES.items():
        with ref_pt.RefScene(make()) as ref:
            img = ref.render(w, h, 0, spp, max_bounces=max_bounces, seed=ref_scenes.SEED, rng="pcg") / spp
        out[f"img_{name}"] = img.astype(np.float32)
        print(f"img_{name}: {w}x{h} x {spp} spp, depth {max_bounces}, mean radiance {img[1].mean():.5f}")
    for name, (make, w, h, m, max_bounces) in ref_scenes.DEFERRED.items():
        with ref_pt.RefScene(make()) as ref:
            img = ref.deferred_render(w, h, m, 0, m * m, max_bounces=max_bounces, seed=ref_scenes.SEED) / (m * m)
        out[f"deferred_{name}"] = img.astype(np.float32)
        print(f"deferred_{name}: {w}x{h} x {m * m} samples, at most {max_bounces} segments, mean {img.mean():.5f}")
    with ref_pt.RefScene(scenes.cornell_box()) as ref:
        out["cornell_mt64"] = (ref.render(64, 64, 0, 64, max_bounces=8, seed=0x1234, rng="mt")[1] / 64).astype(np.float32)
    # CalculateSurfaceParams on hits of scenes that exercise each of its branches
    surf_scenes = {"smooth": scenes.smooth_spheres(), "ibl": ref_scenes.ibl_spheres(0.3),
                   "textured": ref_scenes.textured_cornell(), "media": ref_scenes.media_cornell()}
    for k, (name, rs) in enumerate(surf_scenes.items()):
        hits, ids = _hits(rs, 1000, seed + k)
        with ref_pt.RefScene(rs) as ref:
            out[f"surf_{name}_hits"], out[f"surf_{name}_ids"] = hits, ids
            out[f"surf_{name}_out"] = ref.surface_params(hits, ids)
        print(f"surf_{name}: {hits.shape[0]} hits")
    # NextEventEstimation + LightingPdf with prescribed uniforms
    rng = np.random.default_rng(seed + 10)
    rs = nee_scene()
    n = 2000
    q = np.zeros((n, 6), np.float32)
    q[:, 0:3] = rng.uniform([1, 1, 1], [555, 553, 555], (n, 3))
    nrm = rng.normal(size=(n, 3))
    q[:, 3:6] = nrm / np.linalg.norm(nrm, axis=1, keepdims=True)
    sets = rng.integers(0, 3, n).astype(np.uint32)  # set 2 does not exist: no sample
    u = rng.random((n, 3)).astype(np.float32)
    u[:16, 0] = np.linspace(0.0, 0.999999, 16)
    wi = rng.normal(size=(n, 3))
    wi = (wi / np.linalg.norm(wi, axis=1, keepdims=True)).astype(np.float32)
    with ref_pt.RefScene(rs) as ref:
        out["nee_q"], out["nee_sets"], out["nee_u"], out["nee_wi"] = q, sets, u, wi
        out["nee_out"] = ref.nee(q, sets, u, wi)
    # the image-based light
    ibl = scenes.sky_ibl(rotation=0.3, exposure=1.5)
    rs = ref_scenes.ibl_spheres(0.3)
    h, w = ibl["light"].shape[:2]
    r = rng.random((2000, 2)).astype(np.float32)
    r[:4] = [[0.0, 0.0], [0.999999, 0.999999], [0.5, 0.0], [0.0, 0.5]]
    dirs = rng.normal(size=(2000, 3))
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    with ref_pt.RefScene(rs) as ref:
        smp, rgb, ev, mdf, cdf = ref.ibl(r, dirs, w, h)
    out.update(ibl_r=r, ibl_sample=smp, ibl_rgb=rgb, ibl_dirs=dirs, ibl_eval=ev, ibl_mdf=mdf, ibl_cdf=cdf)
    # VCM iteration constants
    args = np.array([[921600, 1, 0.05, 0.75, 1], [921600, 1, 0.05, 0.75, 256], [4096, 1, 2.5, 0.75, 17],
                     [4096, 1, 2.5, 0.5, 3], [65536, 1, 0.003, 0.9, 1000]], np.float64)
    out["vcm_args"] = args
    out["vcm_out"] = np.stack([ref_pt.vcm_constants(int(a[0]), int(a[1]), a[2], a[3], a[4]) for a in args])
    np.savez_compressed(OUT / "ref_pt_golden.npz", **out)
    print("ref_pt_golden.npz:", len(out), "arrays")


if __name__ == "__main__":
    sys.path.insert(0, str(OUT))
    sys.path.insert(0, str(OUT.parent))
    what = sys.argv[1:] or ["bsdf", "ptex", "ptex_quad", "cornell", "vcm", "cmj", "deferred", "ref_pt"]
    if "bsdf" in what:
        make_bsdf()
    if "ptex" in what:
        make_ptex()
    if "ptex_quad" in what:
        make_ptex_quad()
    if "cornell" in what:
        make_cornell()
    if "vcm" in what:
        make_cornell_vcm()
    if "cmj" in what:
        make_cmj()
    if "deferred" in what:
        make_cornell_deferred()
    if "ref_pt" in what:
        make_ref_pt()

"""ORACLE - test infrastructure only.

ctypes view of oracle/liboracle.so (the CPU restatements in oracle/*.cpp).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this package, as the checker; the product
(selas_gb300) never does.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_lib = None
_vp, _i64, _i = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        from .build import build_oracle
        path = build_oracle()
        _lib = ctypes.CDLL(str(path))
        sig = {
            "oracle_intersect_bruteforce": ([_vp, _vp, _vp, _i64, _vp, _i64, _i], None),
            "oracle_occluded_bruteforce": ([_vp, _vp, _vp, _i64, _vp, _i64, _i], None),
            "oracle_bvh_build": ([_vp, _vp, _vp, _i64], _vp),
            "oracle_bvh_free": ([_vp], None),
            "oracle_intersect_bvh": ([_vp, _vp, _i64, _i], None),
            "oracle_occluded_bvh": ([_vp, _vp, _i64, _i], None),
            "oracle_bsdf_evaluate": ([_vp, _vp, _vp, _i64, _vp], None),
            "oracle_bsdf_sample": ([_vp, _vp, _vp, _i64, _vp], None),
            "oracle_ptex_eval": ([_vp, _i, _vp, _vp, _i64, _vp], None),
            "oracle_ptex_quad_eval": ([_vp, _i, _vp, _vp, _i64, _vp], None),
            "oracle_curve_hits": ([_vp, _vp, _i64, ctypes.c_uint32, _vp, _i64, _i], None),
            "oracle_set_quad_ptex": ([_i, _vp, _vp, _vp, _vp, _vp], None),
            "oracle_set_curves": ([_i, _vp, _vp, _vp, _vp, _vp], None),
            "oracle_pt_render": ([_vp, _vp, _vp, _i64, _vp, _i, _vp, _i, _vp, _i, _vp, _vp, ctypes.c_uint32,
                                  ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                  ctypes.c_uint64, _i, _i, _vp, _i, _vp, _i, _vp], None),
            "oracle_deferred_render": ([_vp, _vp, _vp, _i64, _vp, _i, _vp, _i, _vp, _i, _vp, _vp, ctypes.c_uint32,
                                        ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_uint32, ctypes.c_uint64, _i, _i, _vp, _i, _vp, _i, _vp], None),
            "oracle_cmj": ([_i, _i, _i, _vp], None),
            "oracle_set_ibl": ([_vp, ctypes.c_uint32, ctypes.c_uint32, _vp, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_float, ctypes.c_float], None),
            "oracle_ibl_sample": ([_vp, _i, _vp, _vp], None),
            "oracle_ibl_pdf": ([_vp, _i, _vp], None),
            "oracle_set_attributes": ([_i64, _vp, _vp, _vp, _vp], None),
            "oracle_set_textures": ([ctypes.c_int, _vp, _vp, _vp, _vp], None),
            "oracle_instanced_query": ([_i, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _i64, _i, _vp, _i64, _i, _i],
                                       None),
            "oracle_affine_inverse": ([_vp, _vp], _i),
            "oracle_graph_render": ([_i, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp,
                                     _vp, _vp, _i, _vp, _i, _vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, _i, _i, _i, ctypes.c_uint32, _vp],
                                    None),
            "oracle_graph_intersect": ([_i, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _i64, _i, _vp, _i64, _i], None),
            "oracle_vcm_render": ([_vp, _vp, _vp, _i64, _vp, _i, _vp, _i, _vp, ctypes.c_uint32, ctypes.c_uint32,
                                   ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_uint64, _i, _vp, _i, _vp, _i, _i, _vp], None),
            "oracle_vcm_graph_render": ([_i, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _i64, _i, _vp, _vp, _vp, _vp,
                                         _vp, _vp, _vp, _i, _vp, _vp, ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                         ctypes.c_float, ctypes.c_uint64, _i, _i, _i, _vp], None),
        }
        for name, (args, res) in sig.items():
            fn = getattr(_lib, name)
            fn.argtypes = args
            fn.restype = res
    return _lib


def threads() -> int:
    return int(os.environ.get("ORACLE_THREADS", os.cpu_count() or 1))


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def curve_hits(points, indices, geom_id: int, records: np.ndarray) -> None:
    """Brute-force round B-spline curve hits (oracle_curve.cpp) of one curve geometry, in place: RTCRayHit
    records (closest hit; a nearer curve hit replaces the record's) or RTCRay records (any hit)."""
    p = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
    i = np.ascontiguousarray(indices, np.uint32).reshape(-1)
    lib().oracle_curve_hits(_p(p), _p(i), i.size, geom_id, _p(records), records.shape[0], records.dtype.itemsize)


def intersect_bruteforce(soup, rayhits: np.ndarray, nthreads: int | None = None) -> None:
    v, p, g = soup
    lib().oracle_intersect_bruteforce(_p(v), _p(p), _p(g), v.shape[0], _p(rayhits), rayhits.shape[0],
                                      nthreads or threads())


def occluded_bruteforce(soup, rays: np.ndarray, nthreads: int | None = None) -> None:
    v, p, g = soup
    lib().oracle_occluded_bruteforce(_p(v), _p(p), _p(g), v.shape[0], _p(rays), rays.shape[0], nthreads or threads())


class OracleBvh:
    """The oracle's own binned-SAH binary BVH over a triangle soup."""

    def __init__(self, soup):
        v, p, g = soup
        self._keep = soup
        self.handle = lib().oracle_bvh_build(_p(v), _p(p), _p(g), v.shape[0])

    def intersect(self, rayhits: np.ndarray, nthreads: int | None = None) -> None:
        lib().oracle_intersect_bvh(self.handle, _p(rayhits), rayhits.shape[0], nthreads or threads())

    def occluded(self, rays: np.ndarray, nthreads: int | None = None) -> None:
        lib().oracle_occluded_bvh(self.handle, _p(rays), rays.shape[0], nthreads or threads())

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.oracle_bvh_free(self.handle)
            self.handle = None


def surface_records(surf: np.ndarray) -> np.ndarray:
    """Golden-fixture surfaces keep the shader as a float; SelSurface records hold it as int32 bits."""
    out = np.ascontiguousarray(surf, np.float32).copy()
    out[:, 29] = out[:, 29].astype(np.int32).view(np.float32)
    return out


def bsdf_evaluate(surf, wo, wi):
    s = surface_records(surf)
    wo, wi = np.ascontiguousarray(wo, np.float32), np.ascontiguousarray(wi, np.float32)
    out = np.zeros((s.shape[0], 5), np.float32)
    lib().oracle_bsdf_evaluate(_p(s), _p(wo), _p(wi), s.shape[0], _p(out))
    return out


def bsdf_sample(surf, wo, u):
    s = surface_records(surf)
    wo, u = np.ascontiguousarray(wo, np.float32), np.ascontiguousarray(u, np.float32)
    out = np.zeros((s.shape[0], 16), np.float32)
    lib().oracle_bsdf_sample(_p(s), _p(wo), _p(u), s.shape[0], _p(out))
    return out


class consistent_lambert:
    """Context manager: the oracle's BSDF is an opaque Lambert with exact sampling weights while inside
    (oracle_bsdf.cpp, g_consistent_lambert), for checking that the integrators' estimators agree."""

    def __enter__(self):
        lib().oracle_set_consistent_lambert(1)
        return self

    def __exit__(self, *exc):
        lib().oracle_set_consistent_lambert(0)
        return False


def set_ibl(ibl):
    """Image-based light of the following oracle renders (a RenderScene.ibl dict, or None)."""
    if not ibl:
        lib().oracle_set_ibl(None, 0, 0, None, 0, 0, 0.0, 1.0)
        return
    a = np.ascontiguousarray(ibl["light"], np.float32)
    m = ibl.get("miss")
    m = None if m is None else np.ascontiguousarray(m, np.float32)
    lib().oracle_set_ibl(_p(a), a.shape[1], a.shape[0], None if m is None else _p(m), 0 if m is None else m.shape[1],
                         0 if m is None else m.shape[0], float(ibl.get("rotation", 0.0)), float(ibl.get("exposure", 1.0)))


def set_attributes(parts):
    """Vertex attributes of the next oracle renders' soup: the RenderScenes whose meshes make it, in order."""
    soups = [p.attribute_soup() for p in parts]
    n = np.ascontiguousarray(np.concatenate([s[0] for s in soups]))
    t = np.ascontiguousarray(np.concatenate([s[1] for s in soups]))
    f = np.ascontiguousarray(np.concatenate([s[2] for s in soups]))
    uv = np.ascontiguousarray(np.concatenate([s[3] for s in soups]))
    if not f.any():
        lib().oracle_set_attributes(0, None, None, None, None)
    else:
        lib().oracle_set_attributes(f.shape[0], _p(n), _p(t), _p(f), _p(uv))
    set_textures(parts)


def set_textures(parts):
    """2D base-colour images of the next oracle renders: those of the RenderScenes `parts` (scene index = position),
    as RGBA (one channel: grey, three: alpha 1)."""
    keys, dims, offs, data, off = [], [], [], [], 0
    for si, p in enumerate(parts):
        for gid, img in sorted((getattr(p, "textures", None) or {}).items()):
            a = np.asarray(img, np.float32)
            a = a.reshape(a.shape[0], a.shape[1], -1)
            rgba = np.ones(a.shape[:2] + (4,), np.float32)
            rgba[..., :3] = a[..., :1] if a.shape[2] == 1 else a[..., :3]
            if a.shape[2] == 4:
                rgba[..., 3] = a[..., 3]
            keys += [si, gid]
            dims += [a.shape[1], a.shape[0]]
            offs.append(off)
            data.append(rgba.reshape(-1))
            off += rgba.size
    if not keys:
        lib().oracle_set_textures(0, None, None, None, None)
    else:
        k, d = np.asarray(keys, np.uint32), np.asarray(dims, np.uint32)
        o, r = np.asarray(offs, np.int64), np.ascontiguousarray(np.concatenate(data))
        lib().oracle_set_textures(len(offs), _p(k), _p(d), _p(o), _p(r))
    set_quad_ptex(parts)
    set_curves(parts)


def set_curves(parts):
    """Round B-spline curve geometries of the next oracle renders: those of the RenderScenes `parts` (scene index =
    position; RenderScene.curves, geomID -> (points (n, 4), segment first points)), traced beside each scene's
    triangles (oracle_curve.cpp)."""
    keys, pt_offs, pts, idx_offs, idx = [], [0], [], [0], []
    for si, p in enumerate(parts):
        for gid, (cp, ci) in sorted((getattr(p, "curves", None) or {}).items()):
            cp = np.ascontiguousarray(cp, np.float32).reshape(-1, 4)
            ci = np.ascontiguousarray(ci, np.uint32).reshape(-1)
            keys += [si, gid]
            pts.append(cp)
            pt_offs.append(pt_offs[-1] + cp.shape[0])
            idx.append(ci)
            idx_offs.append(idx_offs[-1] + ci.size)
    if not keys:
        lib().oracle_set_curves(0, None, None, None, None, None)
        return
    k = np.asarray(keys, np.uint32)
    po, io = np.asarray(pt_offs, np.int64), np.asarray(idx_offs, np.int64)
    P, I = np.ascontiguousarray(np.concatenate(pts)), np.ascontiguousarray(np.concatenate(idx))
    lib().oracle_set_curves(len(keys) // 2, _p(k), _p(po), _p(P), _p(io), _p(I))


def _material_count(render_scene, geom):
    """Material records a flat render needs: every geomID of its triangles, curves and materials."""
    ids = [int(geom.max()) if geom.size else 0] + list(render_scene.materials.keys())
    ids += list((getattr(render_scene, "curves", None) or {}).keys())
    return 1 + max(ids)


def set_quad_ptex(parts):
    """Quad-mesh Ptex textures of the next oracle renders: those of the RenderScenes `parts` (scene index =
    position), face rows (n, 10) and half texels each."""
    keys, row_offs, rows, tex_offs, texels = [], [0], [], [0], []
    for si, p in enumerate(parts):
        tables = p.quad_ptex_tables() if hasattr(p, "quad_ptex_tables") else []
        for gid, r, t in tables:
            keys += [si, gid]
            rows.append(r.reshape(-1))
            row_offs.append(row_offs[-1] + r.shape[0])
            texels.append(t.reshape(-1))
            tex_offs.append(tex_offs[-1] + t.size)
    if not keys:
        lib().oracle_set_quad_ptex(0, None, None, None, None, None)
        return
    k = np.asarray(keys, np.uint32)
    ro, to = np.asarray(row_offs, np.int64), np.asarray(tex_offs, np.int64)
    R, T = np.ascontiguousarray(np.concatenate(rows)), np.ascontiguousarray(np.concatenate(texels))
    lib().oracle_set_quad_ptex(len(keys) // 2, _p(k), _p(ro), _p(R), _p(to), _p(T))


def ibl_sample(ibl, r):
    """Oracle IBL sampling of (n, 2) uniforms: (n, 7) [dir, radiance, pdf] and (n, 7) [pdf, light rgb, miss rgb]
    looked up again for the sampled directions."""
    set_ibl(ibl)
    r = np.ascontiguousarray(r, np.float32)
    out = np.zeros((r.shape[0], 7), np.float32)
    ev = np.zeros((r.shape[0], 7), np.float32)
    lib().oracle_ibl_sample(_p(r), r.shape[0], _p(out), _p(ev))
    return out, ev


def ibl_pdf(ibl, dirs):
    set_ibl(ibl)
    d = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(d.shape[0], np.float32)
    lib().oracle_ibl_pdf(_p(d), d.shape[0], _p(out))
    return out


def pt_render(render_scene, width, height, pass_begin, pass_end, max_bounces=8, seed=0x5E1A5000, rng="pcg",
              nthreads=None, physical_nee=False):
    """CPU oracle path tracer (oracle_pt.cpp): FP64 per-pixel sums over passes [pass_begin, pass_end),
    shape (2, height, width, 3)."""
    from selas_gb300.scenes import light_records, material_records
    set_ibl(getattr(render_scene, "ibl", None))
    set_attributes([render_scene])
    verts, prim, geom = render_scene.geometry.soup()
    mats = material_records(render_scene.materials, _material_count(render_scene, geom))
    rows, texels = render_scene.ptex_tables(mats)
    lights, sets = light_records(render_scene.lights)
    bg = np.array(render_scene.background, np.float32)
    c = render_scene.camera
    cam = np.array(list(c["position"]) + list(c["look_at"]) + list(c["up"]) + [c["fov_degrees"]], np.float32)
    out = np.zeros((2, height, width, 3), np.float64)
    L = lib()
    L.oracle_pt_render(_p(verts), _p(prim), _p(geom), verts.shape[0], _p(mats), mats.shape[0], _p(lights),
                       lights.shape[0], _p(sets), sets.shape[0], _p(bg), _p(cam), width, height, pass_begin, pass_end,
                       max_bounces, seed, 0 if rng == "pcg" else 1, nthreads or threads(), _p(rows), rows.shape[0],
                       _p(texels), int(physical_nee), _p(out))
    return out


def deferred_render(render_scene, width, height, sample_begin, sample_end, samples_per_axis=4, max_bounces=64,
                    seed=0x5E1A5000, nthreads=None, physical_nee=False, rng="pcg"):
    """CPU oracle deferred path tracer (oracle_pt.cpp): FP64 per-pixel sums over correlated multi-jittered
    samples [sample_begin, sample_end) of samples_per_axis^2 per pixel, shape (height, width, 3).  rng "pcg":
    the GPU's streams; "mt": MT19937 per pixel as the reference's sampler."""
    from selas_gb300.scenes import light_records, material_records
    set_ibl(getattr(render_scene, "ibl", None))
    set_attributes([render_scene])
    verts, prim, geom = render_scene.geometry.soup()
    mats = material_records(render_scene.materials, _material_count(render_scene, geom))
    rows, texels = render_scene.ptex_tables(mats)
    lights, sets = light_records(render_scene.lights)
    bg = np.array(render_scene.background, np.float32)
    c = render_scene.camera
    cam = np.array(list(c["position"]) + list(c["look_at"]) + list(c["up"]) + [c["fov_degrees"]], np.float32)
    out = np.zeros((height, width, 3), np.float64)
    lib().oracle_deferred_render(_p(verts), _p(prim), _p(geom), verts.shape[0], _p(mats), mats.shape[0], _p(lights),
                                 lights.shape[0], _p(sets), sets.shape[0], _p(bg), _p(cam), width, height,
                                 samples_per_axis, sample_begin, sample_end, max_bounces, seed,
                                 0 if rng == "pcg" else 1, nthreads or threads(),
                                 _p(rows), rows.shape[0], _p(texels), int(physical_nee), _p(out))
    return out


def cmj(m, p, n=None):
    """Correlated multi-jittered points s = 0..n-1 (default m * m) of an m x m pattern decorrelated by p."""
    n = m * m if n is None else n
    xy = np.zeros((n, 2), np.float32)
    lib().oracle_cmj(m, p, n, _p(xy))
    return xy


def affine_inverse(l2w_rows):
    """World-to-local rows (3 x 4 float32) of a local-to-world affine (3 x 4 rows), as instances use them."""
    a = np.ascontiguousarray(np.asarray(l2w_rows, np.float32)[:3, :4])
    out = np.zeros((3, 4), np.float32)
    if not lib().oracle_affine_inverse(_p(a), _p(out)):
        raise ValueError("singular transform")
    return out


def _graph_arrays(scenes):
    """Flat arrays of an instanced scene graph: triangles (verts, prim, geom, owning scene) and instances
    (local-to-world rows, id, owning scene, instanced scene)."""
    verts, prim, geom, owner = [], [], [], []
    l2w, ids, holder, proto = [], [], [], []
    for si, sc in enumerate(scenes):
        for gid, v, idx in sc.get("meshes", []):
            v = np.asarray(v, np.float32).reshape(-1, 3)
            idx = np.asarray(idx, np.int64).reshape(-1, 3)
            verts.append(v[idx].reshape(-1, 9))
            prim.append(np.arange(idx.shape[0], dtype=np.uint32))
            geom.append(np.full(idx.shape[0], gid, np.uint32))
            owner.append(np.full(idx.shape[0], si, np.uint32))
        for iid, pi, m in sc.get("instances", []):
            l2w.append(np.asarray(m, np.float32)[:3, :4].reshape(12))
            ids.append(iid)
            holder.append(si)
            proto.append(pi)
    cat = lambda xs, dt, shape: np.ascontiguousarray(np.concatenate(xs).astype(dt)) if xs else np.zeros(shape, dt)
    return (cat(verts, np.float32, (0, 9)), cat(prim, np.uint32, 0), cat(geom, np.uint32, 0), cat(owner, np.uint32, 0),
            np.ascontiguousarray(np.array(l2w, np.float32).reshape(-1, 12)), np.array(ids, np.uint32),
            np.array(holder, np.uint32), np.array(proto, np.uint32))


def graph_intersect(scenes, top, rayhits, nthreads=None):
    """The render oracle's per-scene-BVH instanced traversal (closest hit; instIDs are not written)."""
    V, P, G, O, L, I, H, Q = _graph_arrays(scenes)
    set_curves([])  # triangles only: no curves left from an earlier render
    lib().oracle_graph_intersect(len(scenes), _p(V), _p(P), _p(G), _p(O), V.shape[0], _p(L), _p(I), _p(H), _p(Q),
                                 L.shape[0], top, _p(rayhits), rayhits.shape[0], nthreads or threads())


def graph_render(iscene, width, height, begin, end, max_bounces=8, seed=0x5E1A5000, deferred=False,
                 samples_per_axis=4, nthreads=None, physical_nee=False):
    """CPU oracle path tracer (deferred=False: shape (2, height, width, 3), passes [begin, end)) or deferred
    path tracer (shape (height, width, 3), samples [begin, end)) over an InstancedRenderScene, PCG32 sampling;
    FP64 sums."""
    from selas_gb300.scenes import light_records, material_records
    set_ibl(iscene.parts[0].ibl)
    set_attributes(iscene.parts)
    V, P, G, O, L, I, H, Q = _graph_arrays(iscene.graph())
    mats, mat_off, rows, row_off, texels, tex_off = [], [0], [], [0], [], [0]
    for part in iscene.parts:
        count = 1 + max([gid for gid, _, _ in part.geometry.meshes] + list(part.materials.keys()) +
                        list((getattr(part, "curves", None) or {}).keys()) + [0])
        m = material_records(part.materials, count)
        r, t = part.ptex_tables(m)
        mats.append(m)
        mat_off.append(mat_off[-1] + m.shape[0])
        rows.append(r)
        row_off.append(row_off[-1] + r.shape[0])
        tex = t if r.shape[0] else np.zeros(0, np.uint16)
        texels.append(tex)
        tex_off.append(tex_off[-1] + tex.size // 3)
    M = np.ascontiguousarray(np.concatenate(mats))
    R = np.ascontiguousarray(np.concatenate(rows).astype(np.int32)).reshape(-1, 8)
    T = np.ascontiguousarray(np.concatenate(texels + [np.zeros(3, np.uint16)]))
    MO, RO, TO = np.array(mat_off, np.int32), np.array(row_off, np.int32), np.array(tex_off, np.int64)
    top = iscene.parts[0]
    lights, sets = light_records(top.lights)
    bg = np.array(top.background, np.float32)
    c = top.camera
    cam = np.array(list(c["position"]) + list(c["look_at"]) + list(c["up"]) + [c["fov_degrees"]], np.float32)
    out = np.zeros((height, width, 3) if deferred else (2, height, width, 3), np.float64)
    lib().oracle_graph_render(len(iscene.parts), _p(V), _p(P), _p(G), _p(O), V.shape[0], _p(L), _p(I), _p(H), _p(Q),
                              L.shape[0], 0, _p(M), _p(MO), _p(R), _p(RO), _p(T), _p(TO), _p(lights), lights.shape[0],
                              _p(sets), sets.shape[0], _p(bg), _p(cam), width, height, begin, end, max_bounces, seed,
                              nthreads or threads(), int(physical_nee), int(deferred), samples_per_axis, _p(out))
    return out


def graph_vcm_render(iscene, width, height, iter_begin, iter_end, bounds, max_len=10, radius0=0.0, alpha=0.75,
                     seed=0x5E1A5000, nthreads=None, merging=True, strategies=15):
    """CPU oracle VCM (oracle_vcm.cpp) over an InstancedRenderScene: FP64 per-pixel sums over iterations
    [iter_begin, iter_end), shape (height, width, 3); bounds: the top scene's world box (lo, hi), the
    environment's emission disc; lights: the top scene's light set 0."""
    from selas_gb300.scenes import light_records, material_records
    set_ibl(iscene.parts[0].ibl)
    set_attributes(iscene.parts)
    V, P, G, O, L, I, H, Q = _graph_arrays(iscene.graph())
    mats, mat_off, rows, row_off, texels, tex_off = [], [0], [], [0], [], [0]
    for part in iscene.parts:
        count = 1 + max([gid for gid, _, _ in part.geometry.meshes] + list(part.materials.keys()) +
                        list((getattr(part, "curves", None) or {}).keys()) + [0])
        m = material_records(part.materials, count)
        r, t = part.ptex_tables(m)
        mats.append(m)
        mat_off.append(mat_off[-1] + m.shape[0])
        rows.append(r)
        row_off.append(row_off[-1] + r.shape[0])
        tex = t if r.shape[0] else np.zeros(0, np.uint16)
        texels.append(tex)
        tex_off.append(tex_off[-1] + tex.size // 3)
    M = np.ascontiguousarray(np.concatenate(mats))
    R = np.ascontiguousarray(np.concatenate(rows).astype(np.int32)).reshape(-1, 8)
    T = np.ascontiguousarray(np.concatenate(texels + [np.zeros(3, np.uint16)]))
    MO, RO, TO = np.array(mat_off, np.int32), np.array(row_off, np.int32), np.array(tex_off, np.int64)
    top = iscene.parts[0]
    lights, sets = light_records(top.lights)
    lights = lights[int(sets[0][0]):int(sets[0][0] + sets[0][1])] if sets.shape[0] else lights[:0]
    lights = np.ascontiguousarray(lights)
    B = np.ascontiguousarray(np.concatenate([np.asarray(bounds[0], np.float32), np.asarray(bounds[1], np.float32)]))
    c = top.camera
    cam = np.array(list(c["position"]) + list(c["look_at"]) + list(c["up"]) + [c["fov_degrees"]], np.float32)
    out = np.zeros((height, width, 3), np.float64)
    lib().oracle_vcm_graph_render(len(iscene.parts), _p(V), _p(P), _p(G), _p(O), V.shape[0], _p(L), _p(I), _p(H),
                                  _p(Q), L.shape[0], 0, _p(M), _p(MO), _p(R), _p(RO), _p(T), _p(TO), _p(lights),
                                  lights.shape[0], _p(B), _p(cam), width, height, iter_begin, iter_end, max_len,
                                  float(radius0), float(alpha), seed, nthreads or threads(), int(merging), strategies,
                                  _p(out))
    return out


def instanced_query(scenes, top, rays, any_hit=False, nthreads=None):
    """Brute-force queries of an instanced scene graph, in place.  scenes: list of dicts with "meshes"
    [(geom_id, vertices (n, 3), indices (m, 3))] and "instances" [(inst_id, scene index, local-to-world 3 x 4
    or 4 x 4)]; rays: SelRayHit records (closest hit) or SelRay records (any hit)."""
    verts, prim, geom, owner = [], [], [], []
    w2l, ids, holder, proto = [], [], [], []
    for si, sc in enumerate(scenes):
        for gid, v, idx in sc.get("meshes", []):
            v = np.asarray(v, np.float32).reshape(-1, 3)
            idx = np.asarray(idx, np.int64).reshape(-1, 3)
            verts.append(v[idx].reshape(-1, 9))
            prim.append(np.arange(idx.shape[0], dtype=np.uint32))
            geom.append(np.full(idx.shape[0], gid, np.uint32))
            owner.append(np.full(idx.shape[0], si, np.uint32))
        for iid, pi, m in sc.get("instances", []):
            w2l.append(affine_inverse(np.asarray(m, np.float32)[:3, :4]).reshape(12))
            ids.append(iid)
            holder.append(si)
            proto.append(pi)
    cat = lambda xs, dt, shape: np.ascontiguousarray(np.concatenate(xs).astype(dt)) if xs else np.zeros(shape, dt)
    V, P, G, O = cat(verts, np.float32, (0, 9)), cat(prim, np.uint32, 0), cat(geom, np.uint32, 0), cat(owner, np.uint32, 0)
    W = np.ascontiguousarray(np.array(w2l, np.float32).reshape(-1, 12))
    I = np.array(ids, np.uint32)
    H = np.array(holder, np.uint32)
    Q = np.array(proto, np.uint32)
    lib().oracle_instanced_query(len(scenes), _p(V), _p(P), _p(G), _p(O), V.shape[0], _p(W), _p(I), _p(H), _p(Q),
                                 W.shape[0], top, _p(rays), rays.shape[0], int(any_hit), nthreads or threads())


def ptex_quad_eval(faces, texels_u16, queries):
    """Oracle Ptex quad filter (oracle_ptex_quad.cpp): faces (n, 10), queries (m, 3) = (face bits, u, v) -> (m, 3)."""
    faces = np.ascontiguousarray(faces, np.int32)
    texels_u16 = np.ascontiguousarray(texels_u16, np.uint16)
    queries = np.ascontiguousarray(queries, np.float32)
    out = np.zeros((queries.shape[0], 3), np.float32)
    lib().oracle_ptex_quad_eval(_p(faces), faces.shape[0], _p(texels_u16), _p(queries), queries.shape[0], _p(out))
    return out


def ptex_eval(faces, texels_u16, queries):
    """Oracle Ptex triangle filter (oracle_ptex.cpp): queries (n, 3) = (face bits, u, v) -> (n, 3)."""
    faces = np.ascontiguousarray(faces, np.int32)
    texels_u16 = np.ascontiguousarray(texels_u16, np.uint16)
    queries = np.ascontiguousarray(queries, np.float32)
    out = np.zeros((queries.shape[0], 3), np.float32)
    lib().oracle_ptex_eval(_p(faces), faces.shape[0], _p(texels_u16), _p(queries), queries.shape[0], _p(out))
    return out


def vcm_render(render_scene, width, height, iter_begin, iter_end, max_len=10, radius0=None, alpha=0.75,
               seed=0x5E1A5000, nthreads=None, merging=True, strategies=15):
    """CPU oracle VCM (oracle_vcm.cpp): FP64 per-pixel sums over iterations [iter_begin, iter_end), shape
    (height, width, 3).  radius0 defaults to 0.0025 x the scene's bounding-sphere radius (VCM.cpp:778 with
    VcmRadiusFactor_ = 0.0025), the sphere taken about the bounding box (radius = half its diagonal).  The
    scene's image-based light, if any, is an environment emitter.  strategies: bit 0 next-event estimation,
    1 vertex connection, 2 vertex merging, 3 light tracing (15: all, MIS-weighted); a subset is unweighted,
    and bit 4 adds camera paths that hit the environment to it."""
    from selas_gb300.scenes import light_records, material_records
    set_attributes([render_scene])
    set_ibl(getattr(render_scene, "ibl", None))
    verts, prim, geom = render_scene.geometry.soup()
    mats = material_records(render_scene.materials, _material_count(render_scene, geom))
    rows, texels = render_scene.ptex_tables(mats)
    lights, sets = light_records(render_scene.lights)
    lights0 = np.ascontiguousarray(lights[sets[0, 0]:sets[0, 0] + sets[0, 1]]) if sets.shape[0] else lights[:0]
    if radius0 is None:
        lo, hi = render_scene.geometry.bounds()
        radius0 = 0.0025 * 0.5 * float(np.linalg.norm(hi - lo))
    c = render_scene.camera
    cam = np.array(list(c["position"]) + list(c["look_at"]) + list(c["up"]) + [c["fov_degrees"]], np.float32)
    out = np.zeros((height, width, 3), np.float64)
    lib().oracle_vcm_render(_p(verts), _p(prim), _p(geom), verts.shape[0], _p(mats), mats.shape[0], _p(lights0),
                            lights0.shape[0], _p(cam), width, height, iter_begin, iter_end, max_len, radius0, alpha,
                            seed, nthreads or threads(), _p(rows), rows.shape[0], _p(texels), int(merging), int(strategies), _p(out))
    return out

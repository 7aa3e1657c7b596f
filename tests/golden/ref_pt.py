"""ctypes view of oracle/_ref/libref_pt.so, the reference's own path tracer and surface / light / camera / IBL /
VCM-constant functions compiled from the reference checkout (oracle/ref/pt_harness.cpp, oracle/ref/build_ref.py).

Used by make_golden.py to generate tests/golden/ref_pt_golden.npz on a machine that has the reference checkout;
tests read only that fixture.
"""
from __future__ import annotations

import ctypes
import os
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
_vp = ctypes.c_void_p
_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(str(ROOT / "oracle" / "_ref" / "libref_pt.so"))
        u32, i32, f32, i64, u64 = ctypes.c_uint32, ctypes.c_int, ctypes.c_float, ctypes.c_int64, ctypes.c_uint64
        L.ref_scene_new.argtypes = [_vp, _vp, _vp, i64, _vp, i32, _vp, i32, _vp, i32, _vp, _vp, _vp, _vp, _vp, _vp,
                                    _vp, i32, _vp, _vp, u32, u32, _vp, u32, u32, f32, f32]
        L.ref_scene_new.restype = _vp
        L.ref_scene_release.argtypes = [_vp]
        L.ref_pt_render.argtypes = [_vp, _vp, u32, u32, u32, u32, u32, u64, i32, i32, _vp]
        L.ref_deferred_render.argtypes = [_vp, _vp, u32, u32, u32, u32, u32, u32, u64, i32, _vp]
        L.ref_surface_params.argtypes = [_vp, _vp, _vp, i32, _vp]
        L.ref_nee.argtypes = [_vp, _vp, _vp, _vp, _vp, i32, _vp]
        L.ref_camera_rays.argtypes = [_vp, u32, u32, _vp, i32, _vp, _vp]
        L.ref_ibl.argtypes = [_vp, _vp, i32, _vp, _vp, _vp, i32, _vp, _vp, _vp]
        L.ref_vcm_constants.argtypes = [u32, u32, f32, f32, f32, _vp]
        P = ctypes.CDLL(str(ROOT / "oracle" / "_ref" / "libref_ptex.so"))
        P.ref_ptex_write.argtypes = [ctypes.c_char_p, _vp, ctypes.c_int, _vp]
        L._ptex = P
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def camera_words(c):
    return np.array(list(c["position"]) + list(c["look_at"]) + list(c["up"]) + [c["fov_degrees"]], np.float32)


class RefScene:
    """A RenderScene (selas_gb300.scenes) in the reference's SceneResource / SubsceneResource / ModelResource
    structures, its Ptex textures written as .ptx files by the vendored Ptex writer."""

    def __init__(self, rs):
        from selas_gb300.scenes import light_records, material_records
        L = lib()
        self._keep = []
        verts, prim, geom = rs.geometry.soup()
        n_mat = int(geom.max()) + 1
        mats = material_records(rs.materials, n_mat)
        lights, sets = light_records(rs.lights)
        bg = np.array(rs.background, np.float32)
        nrm, tan, flags, uvs = rs.attribute_soup()
        has = flags.any()
        self._dir = tempfile.TemporaryDirectory()
        paths = (ctypes.c_char_p * n_mat)()
        for gid, (rows, texels) in sorted((rs.ptex or {}).items()):
            path = os.path.join(self._dir.name, f"g{gid}.ptx").encode()
            rows = np.ascontiguousarray(rows, np.int32)
            tex = np.ascontiguousarray(np.asarray(texels, np.float16).view(np.uint16))
            assert L._ptex.ref_ptex_write(path, rows.ctypes.data, rows.shape[0], tex.ctypes.data) == 0
            paths[gid] = path
        desc, data, off = [], [], 0
        for gid, img in sorted((getattr(rs, "textures", None) or {}).items()):
            a = np.asarray(img, np.float32)
            a = a.reshape(a.shape[0], a.shape[1], -1)
            rgba = np.ones(a.shape[:2] + (4,), np.float32)
            rgba[..., :3] = a[..., :1] if a.shape[2] == 1 else a[..., :3]
            if a.shape[2] == 4:
                rgba[..., 3] = a[..., 3]
            desc += [gid, a.shape[1], a.shape[0], off]
            data.append(rgba.reshape(-1))
            off += rgba.size
        desc = np.array(desc, np.uint32)
        texdata = np.concatenate(data) if data else np.zeros(4, np.float32)
        ibl = getattr(rs, "ibl", None)
        light = miss = None
        rot, expo = 0.0, 1.0
        if ibl:
            light = np.ascontiguousarray(ibl["light"], np.float32)
            miss = ibl.get("miss")
            miss = None if miss is None else np.ascontiguousarray(miss, np.float32)
            rot, expo = float(ibl.get("rotation", 0.0)), float(ibl.get("exposure", 1.0))
        self._keep += [verts, prim, geom, mats, lights, sets, bg, nrm, tan, flags, uvs, paths, desc, texdata, light, miss]
        self.handle = L.ref_scene_new(
            _p(verts), _p(prim), _p(geom), verts.shape[0], _p(mats), n_mat, _p(lights), lights.shape[0], _p(sets),
            sets.shape[0], _p(bg), _p(nrm) if has else None, _p(tan) if has else None, _p(uvs) if has else None,
            _p(flags) if has else None, ctypes.cast(paths, _vp), _p(desc), desc.size // 4, _p(texdata), _p(light),
            0 if light is None else light.shape[1], 0 if light is None else light.shape[0], _p(miss),
            0 if miss is None else miss.shape[1], 0 if miss is None else miss.shape[0], rot, expo)
        self.camera = rs.camera

    def release(self):
        if self.handle:
            lib().ref_scene_release(self.handle)
            self.handle = None
            self._dir.cleanup()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.release()

    def render(self, width, height, pass_begin, pass_end, max_bounces=8, seed=0x5E1A5000, rng="pcg", threads=None):
        """FP64 per-pixel sums of the reference's EvaluatePath over passes [pass_begin, pass_end), shape
        (2, height, width, 3); rng "pcg": the GPU's streams, "mt": the reference's MT19937 per pixel."""
        out = np.zeros((2, height, width, 3), np.float64)
        cam = camera_words(self.camera)
        lib().ref_pt_render(self.handle, _p(cam), width, height, pass_begin, pass_end, max_bounces, seed,
                            0 if rng == "pcg" else 1, threads or os.cpu_count() or 4, _p(out))
        return out

    def deferred_render(self, width, height, samples_per_axis, sample_begin, sample_end, max_bounces=16,
                        seed=0x5E1A5000, threads=None):
        """FP64 per-pixel sums of the reference's deferred path tracer over correlated multi-jittered samples
        [sample_begin, sample_end) of m x m per pixel, shape (height, width, 3), on the GPU's PCG32 streams."""
        out = np.zeros((height, width, 3), np.float64)
        cam = camera_words(self.camera)
        lib().ref_deferred_render(self.handle, _p(cam), width, height, samples_per_axis, sample_begin, sample_end,
                                  max_bounces, seed, threads or os.cpu_count() or 4, _p(out))
        return out

    def surface_params(self, hits, ids):
        hits = np.ascontiguousarray(hits, np.float32)
        ids = np.ascontiguousarray(ids, np.uint32)
        out = np.zeros((hits.shape[0], 40), np.float32)
        lib().ref_surface_params(self.handle, _p(hits), _p(ids), hits.shape[0], _p(out))
        return out

    def nee(self, q, light_sets, u, wi):
        q, u, wi = (np.ascontiguousarray(a, np.float32) for a in (q, u, wi))
        light_sets = np.ascontiguousarray(light_sets, np.uint32)
        out = np.zeros((q.shape[0], 10), np.float32)
        lib().ref_nee(self.handle, _p(q), _p(light_sets), _p(u), _p(wi), q.shape[0], _p(out))
        return out

    def ibl(self, r, dirs, width, height):
        r = np.ascontiguousarray(r, np.float32)
        dirs = np.ascontiguousarray(dirs, np.float32)
        out = np.zeros((r.shape[0], 10), np.float32)
        rgb = np.zeros((r.shape[0], 3), np.float32)
        ev = np.zeros((dirs.shape[0], 7), np.float32)
        mdf = np.zeros(height, np.float32)
        cdf = np.zeros(width * height, np.float32)
        lib().ref_ibl(self.handle, _p(r), r.shape[0], _p(out), _p(rgb), _p(dirs), dirs.shape[0], _p(ev), _p(mdf),
                      _p(cdf))
        return out, rgb, ev, mdf, cdf


def camera_rays(camera, width, height, q):
    q = np.ascontiguousarray(q, np.float32)
    out = np.zeros((q.shape[0], 6), np.float32)
    info = np.zeros(13, np.float32)
    cam = camera_words(camera)
    lib().ref_camera_rays(_p(cam), width, height, _p(q), q.shape[0], _p(out), _p(info))
    return out, info


def vcm_constants(vm_count, vc_count, base_radius, alpha, iteration):
    out = np.zeros(5, np.float32)
    lib().ref_vcm_constants(vm_count, vc_count, base_radius, alpha, iteration, _p(out))
    return out

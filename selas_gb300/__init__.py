"""selas_gb300: GB300-native (sm_103a) render hot path of Selas behind a C ABI.

This module is a thin ctypes view of libselas_gb300.so (declared in include/selas.h).  All work happens
in the CUDA library; there is no Python or CPU fallback: importing the bindings without the built
library raises immediately.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libselas_gb300.so"

SEL_OK = 0
SEL_ERR_INVALID_ARGUMENT = 1
SEL_ERR_OUT_OF_MEMORY = 2
SEL_ERR_CUDA = 3
SEL_ERR_INVALID_OPERATION = 4
SEL_ERR_DEVICE_LIMIT = 5
SEL_ERR_IO = 6

SEL_OPTION_GRAPH_REPLAY = 1
SEL_OPTION_MATERIAL_SORT = 2
SEL_OPTION_RAY_SORT = 3
SEL_OPTION_ZERO_COPY = 4
SEL_BUILD_HOST, SEL_BUILD_DEVICE = 0, 1
SEL_BVH_WIDE8_Q8 = 0
SEL_BVH_BINARY_FP32 = 1

INVALID_ID = 0xFFFFFFFF

# Embree 3.2 RTCRay / RTCRayHit layouts (rtcore_ray.h:26-63)
RAY_DTYPE = np.dtype({
    "names": ["org_x", "org_y", "org_z", "tnear", "dir_x", "dir_y", "dir_z", "time", "tfar", "mask", "id", "flags"],
    "formats": ["<f4"] * 9 + ["<u4"] * 3,
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 44],
    "itemsize": 48,
})
RAYHIT_DTYPE = np.dtype({
    "names": ["org_x", "org_y", "org_z", "tnear", "dir_x", "dir_y", "dir_z", "time", "tfar", "mask", "id", "flags",
              "Ng_x", "Ng_y", "Ng_z", "u", "v", "primID", "geomID", "instID0", "instID1"],
    "formats": ["<f4"] * 9 + ["<u4"] * 3 + ["<f4"] * 5 + ["<u4"] * 4,
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 36, 40, 44, 48, 52, 56, 60, 64, 68, 72, 76, 80],
    "itemsize": 96,
})


class SelError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"selas error {code}: {msg}")
        self.code = code


class SceneInfo(ctypes.Structure):
    _fields_ = [("triangle_count", ctypes.c_uint64), ("node_count", ctypes.c_uint64),
                ("device_bytes", ctypes.c_uint64), ("bvh_kind", ctypes.c_uint32), ("max_depth", ctypes.c_uint32),
                ("build_ms", ctypes.c_double), ("upload_ms", ctypes.c_double),
                ("bounds_lo", ctypes.c_float * 3), ("bounds_hi", ctypes.c_float * 3)]


_lib = None
_vp = ctypes.c_void_p
_i = ctypes.c_int
_u = ctypes.c_uint
_sz = ctypes.c_size_t

# name -> argtypes; every function returns int except sel_get_last_error
_SIGNATURES = {
    "sel_device_new": [_i, ctypes.POINTER(_vp)],
    "sel_device_release": [_vp],
    "sel_device_sync": [_vp, _vp],
    "sel_scene_new": [_vp, ctypes.POINTER(_vp)],
    "sel_scene_set_bvh_kind": [_vp, _i],
    "sel_scene_attach_triangle_mesh": [_vp, _u, _vp, _sz, _sz, _vp, _sz],
    "sel_scene_attach_quad_mesh": [_vp, _u, _vp, _sz, _sz, _vp, _sz],
    "sel_scene_attach_curve_mesh": [_vp, _u, _vp, _sz, _vp, _sz],
    "sel_scene_commit": [_vp],
    "sel_scene_attach_instance": [_vp, _u, _vp, _vp],
    "sel_scene_set_vertex_attribute": [_vp, _u, _u, _vp, _sz, _u],
    "sel_interpolate0": [_vp, _u, _u, ctypes.c_float, ctypes.c_float, _u, _vp, _u],
    "sel_scene_get_info": [_vp, ctypes.POINTER(SceneInfo)],
    "sel_scene_release": [_vp],
    "sel_intersect1": [_vp, _vp],
    "sel_occluded1": [_vp, _vp],
    "sel_intersect1M": [_vp, _vp, _u, _sz],
    "sel_occluded1M": [_vp, _vp, _u, _sz],
    "sel_intersect_device": [_vp, _vp, _u, _vp],
    "sel_occluded_device": [_vp, _vp, _u, _vp],
    "sel_surface_probe_device": [_vp, _vp, _vp, _u, _vp, _vp],
    "sel_light_probe_device": [_vp, _vp, _vp, _vp, _u, _vp, _vp],
    "sel_ibl_probe_device": [_vp, _vp, _u, _vp, _vp, _u, _vp, _vp],
    "sel_vcm_pass_constants": [ctypes.c_float, ctypes.c_float, _u, _u, _vp],
    "sel_scene_last_render_rays": [_vp, _vp],
}


def lib() -> ctypes.CDLL:
    """Loads libselas_gb300.so; raises when it has not been built (run __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        handle = ctypes.CDLL(str(LIB_PATH))
        handle.sel_get_last_error.restype = ctypes.c_char_p
        handle.sel_get_last_error.argtypes = []
        for name, args in _SIGNATURES.items():
            fn = getattr(handle, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = handle
    return _lib


def register_signatures(table: dict) -> None:
    """Lets sibling modules add entry points of the same library."""
    _SIGNATURES.update(table)
    if _lib is not None:
        for name, args in table.items():
            fn = getattr(_lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int


def check(rc: int) -> None:
    if rc != SEL_OK:
        raise SelError(rc, lib().sel_get_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Device:
    """Owns one CUDA device context view (sel_device_new / sel_device_release)."""

    def __init__(self, cuda_device: int = 0):
        h = _vp()
        check(lib().sel_device_new(cuda_device, ctypes.byref(h)))
        self.handle = h

    def sync(self, stream: int | None = None) -> None:
        check(lib().sel_device_sync(self.handle, stream))

    def set_option(self, option: int, value: int) -> None:
        check(lib().sel_device_set_option(self.handle, option, value))

    def release(self) -> None:
        if self.handle:
            check(lib().sel_device_release(self.handle))
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.release()


class Scene:
    """Triangle scene behind the rtcIntersect1 / rtcOccluded1 contract."""

    def __init__(self, device: Device, bvh_kind: int = SEL_BVH_WIDE8_Q8, build_mode: int | None = None):
        h = _vp()
        check(lib().sel_scene_new(device.handle, ctypes.byref(h)))
        if build_mode is not None:
            check(lib().sel_scene_set_build_mode(h, build_mode))
        self.handle = h
        self.device = device
        check(lib().sel_scene_set_bvh_kind(h, bvh_kind))

    def attach_triangle_mesh(self, geom_id: int, vertices: np.ndarray, indices: np.ndarray) -> None:
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
        check(lib().sel_scene_attach_triangle_mesh(self.handle, geom_id, _ptr(v), v.shape[0], 12, _ptr(idx),
                                                   idx.shape[0]))

    def attach_quad_mesh(self, geom_id: int, vertices: np.ndarray, quads: np.ndarray) -> None:
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        q = np.ascontiguousarray(quads, dtype=np.uint32).reshape(-1, 4)
        check(lib().sel_scene_attach_quad_mesh(self.handle, geom_id, _ptr(v), v.shape[0], 12, _ptr(q), q.shape[0]))

    def attach_curve_mesh(self, geom_id: int, points: np.ndarray, indices: np.ndarray) -> None:
        """Round B-spline curves: points (n, 4) = (x, y, z, radius), indices (k,) = first control point of each
        segment."""
        p = np.ascontiguousarray(points, np.float32).reshape(-1, 4)
        i = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        check(lib().sel_scene_attach_curve_mesh(self.handle, geom_id, _ptr(p), p.shape[0], _ptr(i), i.size))

    def attach_instance(self, inst_id: int, instanced: "Scene", local_to_world) -> None:
        """Instance of a committed scene; local_to_world: 4 x 4 (or 3 x 4) affine matrix, row-major maths
        convention (points are columns), passed to the C ABI column-major."""
        m = np.eye(4, dtype=np.float64)
        a = np.asarray(local_to_world, dtype=np.float64)
        m[:a.shape[0], :] = a
        cm = np.ascontiguousarray(m.T.astype(np.float32)).reshape(16)
        check(lib().sel_scene_attach_instance(self.handle, inst_id, instanced.handle, _ptr(cm)))

    def set_vertex_attribute(self, geom_id: int, slot: int, data) -> None:
        """Per-vertex attribute of a mesh (slot 0: normals (n, 3); slot 1: tangents (n, 4); 2..3: anything)."""
        a = np.ascontiguousarray(data, np.float32)
        a = a.reshape(a.shape[0], -1)
        check(lib().sel_scene_set_vertex_attribute(self.handle, geom_id, slot, _ptr(a), a.shape[0], a.shape[1]))

    def set_texture(self, geom_id: int, image) -> None:
        """2D base-colour image of a mesh, (h, w), (h, w, 1), (h, w, 3) or (h, w, 4) floats (None: remove)."""
        if image is None:
            check(lib().sel_scene_set_texture(self.handle, geom_id, None, 0, 0, 3))
            return
        a = np.asarray(image, np.float32)
        a = np.ascontiguousarray(a.reshape(a.shape[0], a.shape[1], -1))
        check(lib().sel_scene_set_texture(self.handle, geom_id, _ptr(a), a.shape[1], a.shape[0], a.shape[2]))

    def interpolate0(self, geom_id: int, prim_id: int, u: float, v: float, slot: int, count: int) -> np.ndarray:
        out = np.zeros(count, np.float32)
        check(lib().sel_interpolate0(self.handle, geom_id, prim_id, u, v, slot, _ptr(out), count))
        return out

    def commit(self) -> None:
        check(lib().sel_scene_commit(self.handle))

    def info(self) -> SceneInfo:
        out = SceneInfo()
        check(lib().sel_scene_get_info(self.handle, ctypes.byref(out)))
        return out

    def intersect1M(self, rayhits: np.ndarray) -> None:
        assert rayhits.dtype == RAYHIT_DTYPE and rayhits.flags.c_contiguous
        check(lib().sel_intersect1M(self.handle, _ptr(rayhits), rayhits.shape[0], 96))

    def occluded1M(self, rays: np.ndarray) -> None:
        assert rays.dtype == RAY_DTYPE and rays.flags.c_contiguous
        check(lib().sel_occluded1M(self.handle, _ptr(rays), rays.shape[0], 48))

    def intersect_device(self, d_ptr: int, n: int, stream: int | None = None) -> None:
        check(lib().sel_intersect_device(self.handle, d_ptr, n, stream))

    def occluded_device(self, d_ptr: int, n: int, stream: int | None = None) -> None:
        check(lib().sel_occluded_device(self.handle, d_ptr, n, stream))

    def release(self) -> None:
        if self.handle:
            check(lib().sel_scene_release(self.handle))
            self.handle = None


def make_rayhits(org: np.ndarray, dirs: np.ndarray, tnear=0.0, tfar=np.inf) -> np.ndarray:
    """Fills RTCRayHit records the way RayPick does (PathTracer.cpp:100-116): ids invalid, mask/flags 0."""
    n = org.shape[0]
    r = np.zeros(n, dtype=RAYHIT_DTYPE)
    r["org_x"], r["org_y"], r["org_z"] = org[:, 0], org[:, 1], org[:, 2]
    r["dir_x"], r["dir_y"], r["dir_z"] = dirs[:, 0], dirs[:, 1], dirs[:, 2]
    r["tnear"] = tnear
    r["tfar"] = tfar
    r["mask"] = 0xFFFFFFFF
    for f in ("primID", "geomID", "instID0", "instID1"):
        r[f] = INVALID_ID
    return r


def make_rays(org: np.ndarray, dirs: np.ndarray, tnear=0.0, tfar=np.inf) -> np.ndarray:
    n = org.shape[0]
    r = np.zeros(n, dtype=RAY_DTYPE)
    r["org_x"], r["org_y"], r["org_z"] = org[:, 0], org[:, 1], org[:, 2]
    r["dir_x"], r["dir_y"], r["dir_z"] = dirs[:, 0], dirs[:, 1], dirs[:, 2]
    r["tnear"] = tnear
    r["tfar"] = tfar
    r["mask"] = 0xFFFFFFFF
    return r


# ---------------------------------------------------------------------------------------------------
# Shading data and the path tracer (include/selas.h: SelMaterial, SelQuadLight, SelCamera, SelPtSettings)
# ---------------------------------------------------------------------------------------------------
_f3 = ctypes.c_float * 3


class SelMaterial(ctypes.Structure):
    _fields_ = [("shader", ctypes.c_int32), ("lightSetIndex", ctypes.c_uint32), ("baseColor", _f3),
                ("transmittanceColor", _f3)] + [(n, ctypes.c_float) for n in (
                    "metallic", "specularTint", "roughness", "anisotropic", "sheen", "sheenTint", "clearcoat",
                    "clearcoatGloss", "specTrans", "diffuseTrans", "flatness", "ior", "scatterDistance")] + [
                ("usesPtex", ctypes.c_uint32)]


class SelNamedMaterial(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 64), ("material", SelMaterial), ("colorMap", ctypes.c_char * 256)]


class SelSceneInstance(ctypes.Structure):
    _fields_ = [("asset", ctypes.c_char * 256), ("localToWorld", ctypes.c_float * 16)]


class SelSceneDescription(ctypes.Structure):
    _fields_ = [("backgroundIntensity", _f3), ("ibl", ctypes.c_char * 256), ("modelCount", ctypes.c_uint),
                ("sceneCount", ctypes.c_uint)]


class SelQuadLight(ctypes.Structure):
    _fields_ = [("position", _f3), ("direction", _f3), ("x", _f3), ("z", _f3), ("radiance", _f3)]


class SelCamera(ctypes.Structure):
    _fields_ = [("position", _f3), ("lookAt", _f3), ("up", _f3), ("fovDegrees", ctypes.c_float),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


class SelPtSettings(ctypes.Structure):
    _fields_ = [("samplesPerPixel", ctypes.c_uint32), ("maxBounces", ctypes.c_uint32), ("seed", ctypes.c_uint64),
                ("pathsInFlight", ctypes.c_uint32), ("traceBlockSize", ctypes.c_uint32)]


class SelVcmSettings(ctypes.Structure):
    _fields_ = [("passes", ctypes.c_uint32), ("firstPass", ctypes.c_uint32), ("maxPathLength", ctypes.c_uint32),
                ("disableMerging", ctypes.c_uint32), ("seed", ctypes.c_uint64), ("radius", ctypes.c_float),
                ("radiusAlpha", ctypes.c_float)]


SEL_SHADER_DISNEY_THIN, SEL_SHADER_DISNEY_SOLID, SEL_SHADER_DIRAC_TRANSPARENT = 0, 1, 2

register_signatures({
    "sel_bsdf_evaluate_device": [_vp, _vp, _vp, _u, _vp, _vp],
    "sel_bsdf_sample_device": [_vp, _vp, _vp, _u, _vp, _vp],
    "sel_material_defaults": [ctypes.POINTER(SelMaterial)],
    "sel_material_from_json": [ctypes.c_char_p, ctypes.POINTER(SelMaterial), ctypes.c_char_p, _u],
    "sel_scene_set_texture": [_vp, _u, _vp, _u, _u, _u],
    "sel_disney_materials_from_json": [ctypes.c_char_p, ctypes.POINTER(SelNamedMaterial), _u,
                                       ctypes.POINTER(ctypes.c_uint)],
    "sel_scene_description_from_json": [ctypes.c_char_p, ctypes.POINTER(SelSceneDescription),
                                        ctypes.POINTER(SelSceneInstance), _u, ctypes.POINTER(SelSceneInstance), _u],
    "sel_scene_set_material": [_vp, _u, ctypes.POINTER(SelMaterial)],
    "sel_scene_add_quad_light": [_vp, _u, ctypes.POINTER(SelQuadLight)],
    "sel_scene_set_background": [_vp, ctypes.c_float, ctypes.c_float, ctypes.c_float],
    "sel_pt_generate_image": [_vp, ctypes.POINTER(SelCamera), ctypes.POINTER(SelPtSettings), _vp],
    "sel_ptex_filter_device": [_vp, _vp, _u, _vp, _vp, _u, _vp, _vp],
    "sel_scene_set_ptex": [_vp, _u, _vp, _sz, _vp, _sz],
    "sel_scene_set_ptex_quads": [_vp, _u, _vp, _sz, _vp, _sz],
    "sel_ptex_quad_filter_device": [_vp, _vp, _u, _vp, _vp, _u, _vp, _vp],
    "sel_pt_render_device": [_vp, ctypes.POINTER(SelCamera), ctypes.POINTER(SelPtSettings), _vp, _vp],
    "sel_vcm_settings_defaults": [ctypes.POINTER(SelVcmSettings)],
    "sel_device_set_option": [_vp, ctypes.c_int, ctypes.c_int],
    "sel_scene_set_build_mode": [_vp, ctypes.c_int],
    "sel_vcm_generate_image": [_vp, ctypes.POINTER(SelCamera), ctypes.POINTER(SelVcmSettings), _vp],
    "sel_vcm_render_device": [_vp, ctypes.POINTER(SelCamera), ctypes.POINTER(SelVcmSettings), _vp, _vp],
    "sel_deferred_settings_defaults": [ctypes.POINTER(SelPtSettings)],
    "sel_scene_set_ibl": [_vp, _vp, _u, _u, _vp, _u, _u, ctypes.c_float, ctypes.c_float],
    "sel_render_views": [_vp, _vp, _u, _u, ctypes.POINTER(SelPtSettings), _vp],
    "sel_render_views_device": [_vp, _vp, _u, _u, ctypes.POINTER(SelPtSettings), _vp, _vp],
    "sel_deferred_generate_image": [_vp, ctypes.POINTER(SelCamera), ctypes.POINTER(SelPtSettings), _vp],
    "sel_deferred_render_device": [_vp, ctypes.POINTER(SelCamera), ctypes.POINTER(SelPtSettings), _vp, _vp],
})


def material(**kw) -> SelMaterial:
    """SelMaterial starting from the reference default material, fields overridden by keyword."""
    m = SelMaterial()
    check(lib().sel_material_defaults(ctypes.byref(m)))
    for k, v in kw.items():
        if isinstance(getattr(m, k), ctypes.Array):
            getattr(m, k)[:] = list(v)
        else:
            setattr(m, k, v)
    return m


def material_from_json(text: str):
    """sel_material_from_json: (SelMaterial, base-colour texture name or "") from a material JSON document."""
    m = SelMaterial()
    tex = ctypes.create_string_buffer(512)
    check(lib().sel_material_from_json(text.encode("utf-8"), ctypes.byref(m), tex, len(tex)))
    return m, tex.value.decode("utf-8")


def disney_materials_from_json(text: str):
    """sel_disney_materials_from_json: [(name, SelMaterial, colorMap)] of a Disney-island materials file, each
    material followed by its assignment names."""
    data = text.encode("utf-8")
    n = ctypes.c_uint(0)
    check(lib().sel_disney_materials_from_json(data, None, 0, ctypes.byref(n)))
    out = (SelNamedMaterial * max(1, n.value))()
    check(lib().sel_disney_materials_from_json(data, out, n.value, ctypes.byref(n)))
    return [(e.name.decode("utf-8"), e.material, e.colorMap.decode("utf-8")) for e in out[:n.value]]


def scene_description_from_json(text: str) -> dict:
    """sel_scene_description_from_json: {"models": [(name, 4x4 localToWorld)], "scenes": [...],
    "background": (r, g, b), "ibl": name}; each matrix is the column-major localToWorld of
    Scene.attach_instance, returned as a (4, 4) array M with M[:, 3] the translation."""
    data = text.encode("utf-8")
    d = SelSceneDescription()
    check(lib().sel_scene_description_from_json(data, ctypes.byref(d), None, 0, None, 0))
    models = (SelSceneInstance * max(1, d.modelCount))()
    scenes = (SelSceneInstance * max(1, d.sceneCount))()
    check(lib().sel_scene_description_from_json(data, ctypes.byref(d), models, d.modelCount, scenes, d.sceneCount))

    def entries(arr, n):
        return [(e.asset.decode("utf-8"), np.array(list(e.localToWorld), np.float32).reshape(4, 4).T) for e in arr[:n]]

    return {"models": entries(models, d.modelCount), "scenes": entries(scenes, d.sceneCount),
            "background": tuple(d.backgroundIntensity), "ibl": d.ibl.decode("utf-8")}


def camera(position, look_at, up, fov_degrees, width, height) -> SelCamera:
    c = SelCamera()
    c.position[:] = list(position)
    c.lookAt[:] = list(look_at)
    c.up[:] = list(up)
    c.fovDegrees = fov_degrees
    c.width, c.height = width, height
    return c


def pt_settings(spp, max_bounces=8, seed=0x5E1A5000, paths_in_flight=0) -> SelPtSettings:
    s = SelPtSettings()
    s.samplesPerPixel, s.maxBounces, s.seed, s.pathsInFlight = spp, max_bounces, seed, paths_in_flight
    return s


def deferred_settings(samples_per_axis=4, max_bounces=64, seed=0x5E1A5000, paths_in_flight=0) -> SelPtSettings:
    """SelPtSettings of the deferred path tracer: samples_per_axis^2 correlated multi-jittered samples per
    pixel (4 x 4 in the reference), at most max_bounces segments per path."""
    s = SelPtSettings()
    check(lib().sel_deferred_settings_defaults(ctypes.byref(s)))
    s.samplesPerPixel, s.maxBounces = samples_per_axis * samples_per_axis, max_bounces
    s.seed, s.pathsInFlight = seed, paths_in_flight
    return s


def vcm_settings(passes, max_path_length=10, seed=0x5E1A5000, first_pass=0, merging=True, radius=0.0,
                 radius_alpha=0.75) -> SelVcmSettings:
    """SelVcmSettings; radius 0 selects the reference's default (0.0025 x the bounding-sphere radius)."""
    s = SelVcmSettings()
    check(lib().sel_vcm_settings_defaults(ctypes.byref(s)))
    s.passes, s.maxPathLength, s.seed, s.firstPass = passes, max_path_length, seed, first_pass
    s.disableMerging = 0 if merging else 1
    s.radius, s.radiusAlpha = radius, radius_alpha
    return s


def _scene_set_material(self, geom_id: int, m: SelMaterial) -> None:
    check(lib().sel_scene_set_material(self.handle, geom_id, ctypes.byref(m)))


def _scene_add_quad_light(self, light_set: int, position, direction, x, z, radiance) -> None:
    q = SelQuadLight()
    q.position[:], q.direction[:], q.x[:], q.z[:], q.radiance[:] = (list(position), list(direction), list(x),
                                                                     list(z), list(radiance))
    check(lib().sel_scene_add_quad_light(self.handle, light_set, ctypes.byref(q)))


def _scene_set_background(self, rgb) -> None:
    check(lib().sel_scene_set_background(self.handle, *map(float, rgb)))


def _scene_set_ibl(self, light, miss=None, rotation=0.0, exposure=1.0) -> None:
    """Image-based light: light (height, width, 3) float32 latitude-longitude RGB; miss likewise (None: light x
    exposure); rotation in radians; exposure scale.  light=None removes it."""
    if light is None:
        check(lib().sel_scene_set_ibl(self.handle, None, 0, 0, None, 0, 0, 0.0, 1.0))
        return
    a = np.ascontiguousarray(light, np.float32)
    m = None if miss is None else np.ascontiguousarray(miss, np.float32)
    check(lib().sel_scene_set_ibl(self.handle, a.ctypes.data, a.shape[1], a.shape[0],
                                  None if m is None else m.ctypes.data, 0 if m is None else m.shape[1],
                                  0 if m is None else m.shape[0], float(rotation), float(exposure)))


def _scene_pt_generate_image(self, cam: SelCamera, settings: SelPtSettings) -> np.ndarray:
    """PathTracer::GenerateImage: (2, height, width, 3) float32 layers, scaled by 1/spp."""
    out = np.zeros((2, cam.height, cam.width, 3), np.float32)
    check(lib().sel_pt_generate_image(self.handle, ctypes.byref(cam), ctypes.byref(settings), out.ctypes.data))
    return out


def _scene_deferred_generate_image(self, cam: SelCamera, settings: SelPtSettings) -> np.ndarray:
    """DeferredPathTracer::GenerateImage: (height, width, 3) float32, scaled by 1/spp."""
    out = np.zeros((cam.height, cam.width, 3), np.float32)
    check(lib().sel_deferred_generate_image(self.handle, ctypes.byref(cam), ctypes.byref(settings), out.ctypes.data))
    return out


def _scene_render_views(self, cams, settings: SelPtSettings, deferred: bool = False) -> list:
    """Several views in one shared wavefront (sel_render_views): one image per camera, as pt_generate_image
    (deferred=False) or deferred_generate_image (deferred=True) gives it with seed settings.seed + k."""
    arr = (SelCamera * len(cams))(*cams)
    layers = 1 if deferred else 2
    sizes = [layers * c.height * c.width * 3 for c in cams]
    out = np.zeros(sum(sizes), np.float32)
    integ = 2 if deferred else 0
    check(lib().sel_render_views(self.handle, ctypes.cast(arr, _vp), len(cams), integ, ctypes.byref(settings),
                                 out.ctypes.data))
    imgs, at = [], 0
    for c, n in zip(cams, sizes):
        shape = (c.height, c.width, 3) if deferred else (2, c.height, c.width, 3)
        imgs.append(out[at:at + n].reshape(shape))
        at += n
    return imgs


def _scene_vcm_generate_image(self, cam: SelCamera, settings: SelVcmSettings) -> np.ndarray:
    """VCM::GenerateImage: (height, width, 3) float32, the mean over the passes."""
    out = np.zeros((cam.height, cam.width, 3), np.float32)
    check(lib().sel_vcm_generate_image(self.handle, ctypes.byref(cam), ctypes.byref(settings), out.ctypes.data))
    return out


def _scene_set_ptex(self, geom_id: int, rows: np.ndarray, texels: np.ndarray) -> None:
    """Binds per-face Ptex texels (rows: (n, 8) int32 SelPtexFace records of a triangle mesh, or (n, 10) int32
    SelPtexQuadFace records of a quad mesh; texels: float16 RGB)."""
    r = np.ascontiguousarray(rows, np.int32)
    t = np.ascontiguousarray(np.asarray(texels, np.float16).view(np.uint16))
    fn = lib().sel_scene_set_ptex_quads if r.shape[1] == 10 else lib().sel_scene_set_ptex
    check(fn(self.handle, geom_id, r.ctypes.data, r.shape[0], t.ctypes.data, t.size))


Scene.set_ptex = _scene_set_ptex
Scene.set_material = _scene_set_material
Scene.add_quad_light = _scene_add_quad_light
Scene.set_background = _scene_set_background
Scene.set_ibl = _scene_set_ibl
Scene.pt_generate_image = _scene_pt_generate_image
Scene.vcm_generate_image = _scene_vcm_generate_image
Scene.deferred_generate_image = _scene_deferred_generate_image
Scene.render_views = _scene_render_views


# ---------------------------------------------------------------------------------------------------
# Render server (include/selas.h: sel_server_*)
# ---------------------------------------------------------------------------------------------------
SEL_INTEGRATOR_PT, SEL_INTEGRATOR_VCM, SEL_INTEGRATOR_DEFERRED = 0, 1, 2


class SelServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("hbm_reserve_bytes", ctypes.c_uint64),
                ("max_jobs", ctypes.c_uint32), ("paths_in_flight", ctypes.c_uint32), ("max_bounces", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class SelJob(ctypes.Structure):
    _fields_ = [("scene", _vp), ("camera", SelCamera), ("integrator", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("pt", SelPtSettings), ("vcm", SelVcmSettings)]


class SelJobStats(ctypes.Structure):
    _fields_ = [("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("device_bytes", ctypes.c_uint64), ("status", ctypes.c_int32), ("reserved", ctypes.c_uint32)]


class SelServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "rays", "peak_jobs", "peak_bytes",
                                                "graph_captures")]


register_signatures({
    "sel_server_config_defaults": [ctypes.POINTER(SelServerConfig)],
    "sel_server_new": [_vp, ctypes.POINTER(SelServerConfig), ctypes.POINTER(_vp)],
    "sel_server_submit": [_vp, ctypes.POINTER(SelJob), ctypes.POINTER(ctypes.c_uint64)],
    "sel_server_result_floats": [ctypes.POINTER(SelJob), ctypes.POINTER(_sz)],
    "sel_server_poll": [_vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int)],
    "sel_server_wait": [_vp, ctypes.c_uint64, _vp, _sz, ctypes.POINTER(SelJobStats)],
    "sel_server_stats": [_vp, ctypes.POINTER(SelServerStats)],
    "sel_server_release": [_vp],
})


def server_config(**kw) -> SelServerConfig:
    c = SelServerConfig()
    check(lib().sel_server_config_defaults(ctypes.byref(c)))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def pt_job(scene, cam: SelCamera, settings: SelPtSettings) -> SelJob:
    j = SelJob()
    j.scene, j.camera, j.integrator, j.pt = scene.handle, cam, SEL_INTEGRATOR_PT, settings
    return j


def deferred_job(scene, cam: SelCamera, settings: SelPtSettings) -> SelJob:
    j = SelJob()
    j.scene, j.camera, j.integrator, j.pt = scene.handle, cam, SEL_INTEGRATOR_DEFERRED, settings
    return j


def vcm_job(scene, cam: SelCamera, settings: SelVcmSettings) -> SelJob:
    j = SelJob()
    j.scene, j.camera, j.integrator, j.vcm = scene.handle, cam, SEL_INTEGRATOR_VCM, settings
    return j


class Server:
    """Continuous-batching render server (sel_server_*): submit() returns a job id at once, wait() returns
    the image (path tracer: (2, H, W, 3) layers; VCM: (H, W, 3)) and the job's SelJobStats."""

    def __init__(self, device: Device, config: SelServerConfig | None = None):
        h = _vp()
        check(lib().sel_server_new(device.handle, ctypes.byref(config) if config is not None else None,
                                   ctypes.byref(h)))
        self.handle = h
        self._shapes = {}

    def submit(self, job: SelJob) -> int:
        jid = ctypes.c_uint64()
        check(lib().sel_server_submit(self.handle, ctypes.byref(job), ctypes.byref(jid)))
        w, h = job.camera.width, job.camera.height
        self._shapes[jid.value] = (2, h, w, 3) if job.integrator == SEL_INTEGRATOR_PT else (h, w, 3)
        return jid.value

    def done(self, job_id: int) -> bool:
        d = ctypes.c_int()
        check(lib().sel_server_poll(self.handle, job_id, ctypes.byref(d)))
        return bool(d.value)

    def wait(self, job_id: int):
        out = np.zeros(self._shapes.pop(job_id), np.float32)
        st = SelJobStats()
        check(lib().sel_server_wait(self.handle, job_id, out.ctypes.data, out.size, ctypes.byref(st)))
        return out, st

    def stats(self) -> SelServerStats:
        s = SelServerStats()
        check(lib().sel_server_stats(self.handle, ctypes.byref(s)))
        return s

    def release(self) -> None:
        if self.handle:
            check(lib().sel_server_release(self.handle))
            self.handle = None


# ---------------------------------------------------------------------------------------------------
# Autotuner (include/selas.h: sel_scene_autotune)
# ---------------------------------------------------------------------------------------------------
class SelTuneTrial(ctypes.Structure):
    _fields_ = [("bvh_kind", ctypes.c_uint32), ("leaf_size", ctypes.c_uint32), ("paths_in_flight", ctypes.c_uint32),
                ("trace_block", ctypes.c_uint32), ("ms", ctypes.c_double)]


class SelTuneResult(ctypes.Structure):
    _fields_ = [("best", SelTuneTrial), ("trials", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("trial", SelTuneTrial * 32)]


register_signatures({
    "sel_scene_set_leaf_size": [_vp, _u],
    "sel_scene_autotune": [_vp, ctypes.POINTER(SelCamera), ctypes.POINTER(SelPtSettings), ctypes.POINTER(SelTuneResult)],
})


def _scene_autotune(self, cam: SelCamera, settings: SelPtSettings) -> SelTuneResult:
    """sel_scene_autotune: times the workload over BVH layout / leaf size / capacity / block size, keeps the
    fastest on the scene and returns every trial."""
    r = SelTuneResult()
    check(lib().sel_scene_autotune(self.handle, ctypes.byref(cam), ctypes.byref(settings), ctypes.byref(r)))
    return r


def _scene_set_leaf_size(self, n: int) -> None:
    check(lib().sel_scene_set_leaf_size(self.handle, n))


Scene.autotune = _scene_autotune
Scene.set_leaf_size = _scene_set_leaf_size


# ---------------------------------------------------------------------------------------------------
# Cooked assets (include/selas.h: SelCookedSceneInfo, SelCookedMesh, sel_scene_load_cooked)
# ---------------------------------------------------------------------------------------------------
SEL_COOKED_PTEX_AS_BASE_COLOR = 1


class SelCookedSceneInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("subscenes", "subsceneInstances", "models", "modelInstances", "meshes",
                                               "quadMeshes")] + [("faces", ctypes.c_uint64)] + [
               (n, ctypes.c_uint32) for n in ("lights", "lightSets", "cameras", "textures", "ptexMeshes", "curves")] + [
               ("backgroundIntensity", ctypes.c_float * 4), ("ibl", ctypes.c_char * 512), ("camera", SelCamera)]


class SelCookedMesh(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("subscene", "model", "mesh", "indicesPerFace", "faces",
                                               "materialFlags")] + [
               ("material", SelMaterial), ("texture", ctypes.c_char * 512), ("name", ctypes.c_char * 64)]


register_signatures({
    "sel_cooked_scene_describe": [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(SelCookedSceneInfo),
                                  ctypes.POINTER(SelCookedMesh), _u],
    "sel_scene_load_cooked": [_vp, ctypes.c_char_p, ctypes.c_char_p, _u, ctypes.POINTER(_vp),
                              ctypes.POINTER(SelCookedSceneInfo)],
})


def cooked_describe(asset_root, scene_name: str):
    """sel_cooked_scene_describe: (SelCookedSceneInfo, list of SelCookedMesh in load order); needs no device."""
    info = SelCookedSceneInfo()
    root, name = str(asset_root).encode(), scene_name.encode()
    check(lib().sel_cooked_scene_describe(root, name, ctypes.byref(info), None, 0))
    meshes = (SelCookedMesh * max(info.meshes, 1))()
    check(lib().sel_cooked_scene_describe(root, name, ctypes.byref(info), meshes, info.meshes))
    return info, list(meshes[:info.meshes])


def load_cooked(device: Device, asset_root, scene_name: str, flags: int = 0):
    """sel_scene_load_cooked: (committed Scene, SelCookedSceneInfo); releasing the scene releases the subscene and
    model scenes it instances."""
    info = SelCookedSceneInfo()
    h = _vp()
    check(lib().sel_scene_load_cooked(device.handle, str(asset_root).encode(), scene_name.encode(), flags,
                                      ctypes.byref(h), ctypes.byref(info)))
    sc = Scene.__new__(Scene)
    sc.handle = h
    sc.device = device
    return sc, info

"""Seeded synthetic scenes and ray sets.

The reference renders assets cooked offline (Source/Core/BuildCommon); its default scene (Disney's Moana
island) is not available, so every workload here is generated procedurally with fixed seeds:

* ``displaced_icospheres``: 64 icospheres at subdivision level 6 (81,920 triangles each, 5,242,880 in
  total), radii U[2, 6], radial value noise of amplitude 0.1, centres uniform in a 100^3 box over a
  200 x 200 ground plane (2 triangles).  Level 5 gives the 1.3 M-triangle variant.
* ``primary_rays``: pinhole camera rays through pixel centres, using the reference camera model
  (Source/Core/GeometryLib/Camera.cpp:56-60,89-115).
* ``surface_rays``: origins at uniformly chosen points on uniformly chosen triangles, offset along the
  face normal, cosine-distributed directions about it.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class TriangleScene:
    meshes: list = field(default_factory=list)  # (geom_id, vertices (n,3) f32, indices (m,3) u32)

    def add(self, geom_id: int, vertices: np.ndarray, indices: np.ndarray) -> None:
        self.meshes.append((int(geom_id), np.ascontiguousarray(vertices, np.float32),
                            np.ascontiguousarray(indices, np.uint32)))

    @property
    def triangle_count(self) -> int:
        return sum(m[2].shape[0] for m in self.meshes)

    def soup(self):
        """(verts (n,9) f32, primID (n,) u32, geomID (n,) u32) in attachment order."""
        vs, ps, gs = [], [], []
        for gid, v, idx in self.meshes:
            vs.append(v[idx].reshape(-1, 9))
            ps.append(np.arange(idx.shape[0], dtype=np.uint32))
            gs.append(np.full(idx.shape[0], gid, dtype=np.uint32))
        return (np.ascontiguousarray(np.concatenate(vs)), np.concatenate(ps), np.concatenate(gs))

    def attach_to(self, scene) -> None:
        for gid, v, idx in self.meshes:
            scene.attach_triangle_mesh(gid, v, idx)

    def bounds(self):
        lo = np.min([m[1].min(axis=0) for m in self.meshes], axis=0)
        hi = np.max([m[1].max(axis=0) for m in self.meshes], axis=0)
        return lo, hi


def icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    return v / np.linalg.norm(v, axis=1, keepdims=True), f


def icosphere(level: int):
    """Unit icosphere: 20 * 4^level triangles, outward winding."""
    v, f = icosahedron()
    for _ in range(level):
        nv = v.shape[0]
        nf = f.shape[0]
        edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        es = np.sort(edges, axis=1)
        keys = es[:, 0] * nv + es[:, 1]
        uniq, inv = np.unique(keys, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid])
        m01, m12, m20 = nv + inv[:nf], nv + inv[nf:2 * nf], nv + inv[2 * nf:]
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f


def value_noise_dirs(p: np.ndarray, rng: np.random.Generator, octaves: int = 4) -> np.ndarray:
    """Smooth noise in [-1, 1] on unit directions: a seeded sum of sinusoids."""
    out = np.zeros(p.shape[0])
    norm = 0.0
    for o in range(octaves):
        w = rng.normal(size=(3,)) * (2.0 ** o) * 2.0
        phase = rng.uniform(0, 2 * np.pi)
        amp = 0.5 ** o
        out += amp * np.sin(p @ w + phase)
        norm += amp
    return out / norm


def displaced_icospheres(count: int = 64, level: int = 6, seed: int = 0x5E1A5001, noise_amp: float = 0.1,
                         ground: bool = True) -> TriangleScene:
    rng = np.random.default_rng(seed)
    unit_v, f = icosphere(level)
    scene = TriangleScene()
    for i in range(count):
        centre = np.array([rng.uniform(-50, 50), rng.uniform(0, 100), rng.uniform(-50, 50)])
        radius = rng.uniform(2.0, 6.0)
        disp = 1.0 + noise_amp * value_noise_dirs(unit_v, rng)
        verts = centre + unit_v * (radius * disp)[:, None]
        scene.add(i, verts.astype(np.float32), f.astype(np.uint32))
    if ground:
        gv = np.array([[-100, 0, -100], [100, 0, -100], [100, 0, 100], [-100, 0, 100]], np.float32)
        gi = np.array([[0, 2, 1], [0, 3, 2]], np.uint32)  # normal +y
        scene.add(count, gv, gi)
    return scene


def camera_basis(position, look_at, up, hfov_deg: float, width: int, height: int):
    """RayCastCameraSettings of InitializeRayCastCamera (Camera.cpp:89-115)."""
    position = np.asarray(position, np.float64)
    look_at = np.asarray(look_at, np.float64)
    up = np.asarray(up, np.float64)
    aspect = width / height
    hfov = np.deg2rad(hfov_deg)
    h_len = np.tan(hfov * 0.5)
    vfov = 2 * np.arctan(h_len / aspect)
    v_len = np.tan(vfov * 0.5)
    fwd = look_at - position
    fwd /= np.linalg.norm(fwd)
    right = np.cross(up, fwd)
    right /= np.linalg.norm(right)
    return {"X": h_len * right, "Y": v_len * np.cross(fwd, right), "Z": fwd, "position": position,
            "width": width, "height": height}


def primary_rays(cam: dict, jitter: np.ndarray | None = None):
    """Directions through pixel centres (or centre + jitter), ImageToWorldDirection (Camera.cpp:56-60)."""
    w, h = cam["width"], cam["height"]
    ys, xs = np.mgrid[0:h, 0:w]
    x = xs.reshape(-1).astype(np.float64) + 0.5
    y = ys.reshape(-1).astype(np.float64) + 0.5
    if jitter is not None:
        x += jitter[:, 0] - 0.5
        y += jitter[:, 1] - 0.5
    cx = (x / w) * 2.0 - 1.0
    cy = 1.0 - 2.0 * y / h
    d = cam["Z"][None, :] - cx[:, None] * cam["X"][None, :] + cy[:, None] * cam["Y"][None, :]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    org = np.broadcast_to(cam["position"], d.shape)
    return np.ascontiguousarray(org, np.float32), np.ascontiguousarray(d, np.float32)


def surface_rays(scene: TriangleScene, n: int, seed: int = 0x5E1A5002, offset: float = 1e-3):
    rng = np.random.default_rng(seed)
    verts, _, _ = scene.soup()
    tri = rng.integers(0, verts.shape[0], size=n)
    v = verts[tri].reshape(n, 3, 3).astype(np.float64)
    r1 = np.sqrt(rng.random(n))
    r2 = rng.random(n)
    p = (1 - r1)[:, None] * v[:, 0] + (r1 * (1 - r2))[:, None] * v[:, 1] + (r1 * r2)[:, None] * v[:, 2]
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    # orthonormal frame (MakeOrthogonalCoordinateSystem, GeometryLib/CoordinateSystem.h:14-21)
    t = np.where((np.abs(nrm[:, 0]) > np.abs(nrm[:, 1]))[:, None],
                 np.stack([-nrm[:, 2], np.zeros(n), nrm[:, 0]], 1), np.stack([np.zeros(n), nrm[:, 2], -nrm[:, 1]], 1))
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    b = np.cross(nrm, t)
    u0, u1 = rng.random(n), rng.random(n)
    rr = np.sqrt(u0)
    phi = 2 * np.pi * u1
    local = np.stack([rr * np.cos(phi), np.sqrt(np.maximum(0.0, 1 - u0)), rr * np.sin(phi)], 1)
    d = local[:, 0:1] * t + local[:, 1:2] * nrm + local[:, 2:3] * b
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    org = p + offset * nrm
    return np.ascontiguousarray(org, np.float32), np.ascontiguousarray(d, np.float32)


def ray_query_workload(level: int = 6, width: int = 2048, height: int = 2048, incoherent: int | None = None,
                       seed: int = 0x5E1A5001):
    """The ray-query benchmark: scene + coherent primary rays + incoherent surface rays."""
    scene = displaced_icospheres(level=level, seed=seed)
    cam = camera_basis([0.0, 70.0, -170.0], [0.0, 40.0, 0.0], [0.0, 1.0, 0.0], 60.0, width, height)
    co, cd = primary_rays(cam)
    n_inc = incoherent if incoherent is not None else width * height
    io, idir = surface_rays(scene, n_inc, seed=seed + 1)
    return scene, (co, cd), (io, idir)


# ---------------------------------------------------------------------------------------------------
# Render scenes: geometry + per-geometry materials + quad lights + camera
# ---------------------------------------------------------------------------------------------------
@dataclass
class RenderScene:
    geometry: TriangleScene
    materials: dict = field(default_factory=dict)   # geomID -> dict of SelMaterial fields
    lights: list = field(default_factory=list)      # (light set, dict(position, direction, x, z, radiance))
    background: tuple = (0.0, 0.0, 0.0)
    camera: dict = field(default_factory=dict)      # position, look_at, up, fov_degrees

    def build(self, sel_module, device, bvh_kind=0):
        """Creates and commits a selas_gb300 Scene with this content."""
        sc = sel_module.Scene(device, bvh_kind)
        self.geometry.attach_to(sc)
        for gid, m in self.materials.items():
            sc.set_material(gid, sel_module.material(**m))
        for ls, l in self.lights:
            sc.add_quad_light(ls, l["position"], l["direction"], l["x"], l["z"], l["radiance"])
        sc.set_background(self.background)
        sc.commit()
        return sc

    def sel_camera(self, sel_module, width, height):
        c = self.camera
        return sel_module.camera(c["position"], c["look_at"], c["up"], c["fov_degrees"], width, height)


def _quad(p0, p1, p2, p3):
    v = np.array([p0, p1, p2, p3], np.float32)
    return v, np.array([[0, 1, 2], [0, 2, 3]], np.uint32)


def _box(centre, size, angle_deg):
    sx, sy, sz = size
    c = np.array(centre, np.float64)
    corners = np.array([[x, y, z] for y in (0.0, sy) for z in (-sz / 2, sz / 2) for x in (-sx / 2, sx / 2)])
    a = np.deg2rad(angle_deg)
    rot = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
    v = (corners @ rot.T) + np.array([c[0], 0.0, c[2]])
    # corner index = 4*y + 2*z + x
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    idx = []
    for a_, b_, c_, d_ in faces:
        idx += [[a_, b_, c_], [a_, c_, d_]]
    return v.astype(np.float32), np.array(idx, np.uint32)


def cornell_box(background=(0.0, 0.0, 0.0)) -> RenderScene:
    """Cornell-style box: 5 axis-aligned quads of side 556, boxes 165 and 330 tall rotated -18 / +18
    degrees about y, a 130 x 105 quad light of radiance (17, 12, 4) just under the ceiling (lights are not
    geometry in the reference: NEE only).  Disney solid, roughness 0.5, metallic 0, ior 1.5, 34 triangles."""
    s = 556.0
    g = TriangleScene()
    g.add(0, *_quad([0, 0, 0], [0, 0, s], [s, 0, s], [s, 0, 0]))          # floor (normal +y)
    g.add(1, *_quad([0, s, 0], [s, s, 0], [s, s, s], [0, s, s]))          # ceiling (normal -y)
    g.add(2, *_quad([0, 0, s], [0, s, s], [s, s, s], [s, 0, s]))          # back wall (normal -z)
    g.add(3, *_quad([s, 0, 0], [s, 0, s], [s, s, s], [s, s, 0]))          # left wall, red (normal -x)
    g.add(4, *_quad([0, 0, 0], [0, s, 0], [0, s, s], [0, 0, s]))          # right wall, green (normal +x)
    g.add(5, *_box([185.0, 0.0, 169.0], (165.0, 165.0, 165.0), -18.0))   # short box
    g.add(6, *_box([368.0, 0.0, 351.0], (165.0, 330.0, 165.0), 18.0))    # tall box
    base = dict(shader=1, lightSetIndex=0, roughness=0.5, metallic=0.0, ior=1.5)
    grey, red, green = (0.73, 0.73, 0.73), (0.65, 0.05, 0.05), (0.12, 0.45, 0.15)
    mats = {gid: dict(base, baseColor=grey) for gid in (0, 1, 2, 5, 6)}
    mats[3] = dict(base, baseColor=red)
    mats[4] = dict(base, baseColor=green)
    light = dict(position=(278.0, 554.0, 279.5), direction=(0.0, -1.0, 0.0), x=(130.0, 0.0, 0.0),
                 z=(0.0, 0.0, 105.0), radiance=(17.0, 12.0, 4.0))
    cam = dict(position=(278.0, 273.0, -800.0), look_at=(278.0, 273.0, 0.0), up=(0.0, 1.0, 0.0), fov_degrees=39.3)
    return RenderScene(g, mats, [(0, light)], tuple(background), cam)


def material_records(materials: dict, count: int) -> np.ndarray:
    """Per-geomID 32-word material records (the renderer's HBM layout) for the CPU oracle; geometries
    without a material get the reference default (CreateDefaultMaterial, ModelResource.cpp:203-211)."""
    recs = np.zeros((count, 32), np.float32)
    words = recs.view(np.uint32)
    defaults = dict(shader=1, lightSetIndex=0, baseColor=(0.6, 0.6, 0.6), transmittanceColor=(0, 0, 0), metallic=0.0,
                    specularTint=0.0, roughness=0.0, anisotropic=0.0, sheen=0.0, sheenTint=0.0, clearcoat=0.0,
                    clearcoatGloss=0.0, specTrans=0.0, diffuseTrans=0.0, flatness=0.0, ior=1.5, scatterDistance=0.0,
                    usesPtex=0)
    for gid in range(count):
        m = dict(defaults, **materials.get(gid, {}))
        transparent = m["shader"] == 1 and (m["diffuseTrans"] > 0 or m["specTrans"] > 0)
        words[gid, 0] = np.uint32(np.int32(m["shader"]).view(np.uint32))
        words[gid, 1] = (1 if transparent else 0) | (2 if m["usesPtex"] else 0)
        words[gid, 2] = m["lightSetIndex"]
        recs[gid, 4:7] = m["baseColor"]
        recs[gid, 7:10] = m["transmittanceColor"]
        for i, k in enumerate(("sheen", "sheenTint", "clearcoat", "clearcoatGloss", "metallic", "specTrans",
                               "diffuseTrans", "flatness", "anisotropic", "specularTint", "roughness",
                               "scatterDistance", "ior")):
            recs[gid, 10 + i] = m[k]
    return recs


def light_records(lights: list):
    """(lights n x 15 floats, sets n_sets x 2 (first, count)) grouped by light set."""
    n_sets = 1 + max((ls for ls, _ in lights), default=-1)
    grouped = [[l for ls, l in lights if ls == k] for k in range(n_sets)]
    flat, sets = [], []
    for group in grouped:
        sets.append((len(flat), len(group)))
        for l in group:
            flat.append(list(l["position"]) + list(l["direction"]) + list(l["x"]) + list(l["z"]) + list(l["radiance"]))
    return (np.array(flat, np.float32).reshape(-1, 15), np.array(sets, np.uint32).reshape(-1, 2))

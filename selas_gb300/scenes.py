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
    quad_geoms: set = field(default_factory=set)  # geomIDs of quad meshes (their indices hold triangle pairs)

    def add(self, geom_id: int, vertices: np.ndarray, indices: np.ndarray) -> None:
        self.meshes.append((int(geom_id), np.ascontiguousarray(vertices, np.float32),
                            np.ascontiguousarray(indices, np.uint32)))

    def add_quads(self, geom_id: int, vertices: np.ndarray, quads: np.ndarray) -> None:
        """A quad mesh, held as Embree holds it: quad q is the triangles 2q = (v0, v1, v3) and 2q + 1 = (v2, v3, v1)
        (RTC_GEOMETRY_TYPE_QUAD.3embree3); soup() numbers those triangles 2q and 2q + 1."""
        q = np.ascontiguousarray(quads, np.uint32).reshape(-1, 4)
        pairs = np.stack([q[:, 0], q[:, 1], q[:, 3], q[:, 2], q[:, 3], q[:, 1]], 1).reshape(-1, 3)
        self.add(geom_id, vertices, pairs)
        self.quad_geoms.add(int(geom_id))

    @staticmethod
    def quads_of(pairs: np.ndarray) -> np.ndarray:
        p = np.asarray(pairs).reshape(-1, 6)
        return np.stack([p[:, 0], p[:, 1], p[:, 3], p[:, 2]], 1)

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
            if gid in self.quad_geoms:
                scene.attach_quad_mesh(gid, v, self.quads_of(idx))
            else:
                scene.attach_triangle_mesh(gid, v, idx)

    def embree_hits(self, rayhits: np.ndarray) -> None:
        """Turns hits on the soup's triangles (primID = soup numbering) into what Embree reports: on a quad mesh
        primID = quad and the second triangle's (u', v') -> (1 - u', 1 - v') in FP32."""
        if not self.quad_geoms:
            return
        hit = rayhits["geomID"] != 0xFFFFFFFF
        q = hit & np.isin(rayhits["geomID"], np.array(sorted(self.quad_geoms), np.uint32))
        second = q & (rayhits["primID"] & 1 == 1)
        one = np.float32(1.0)
        rayhits["u"][second] = one - rayhits["u"][second]
        rayhits["v"][second] = one - rayhits["v"][second]
        rayhits["primID"][q] >>= 1

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
    ptex: dict = field(default_factory=dict)        # geomID -> (face rows (n, 8) int32, texels float16)
    ibl: dict = None                                # light (H, W, 3), miss (h, w, 3) or None, rotation, exposure
    attrs: dict = None                              # geomID -> {"normals": (n, 3), "tangents": (n, 4), "uvs": (n, 2)}
    textures: dict = None                           # geomID -> 2D base-colour image (h, w, 1 | 3 | 4) floats
    curves: dict = None                             # geomID -> (control points (n, 4), segment first points (k,))

    def attach_attributes(self, sc) -> None:
        for gid, a in (self.attrs or {}).items():
            if a.get("normals") is not None:
                sc.set_vertex_attribute(gid, 0, a["normals"])
            if a.get("tangents") is not None:
                sc.set_vertex_attribute(gid, 1, a["tangents"])
            if a.get("uvs") is not None:
                sc.set_vertex_attribute(gid, 2, a["uvs"])
        for gid, img in (self.textures or {}).items():
            sc.set_texture(gid, img)

    def attribute_soup(self):
        """Per-triangle corner normals (n, 9), tangents (n, 12), flags (1 normals, 2 tangents, 4 uvs, 8 the
        triangle is half of a quad) and uvs (n, 6), in soup() order, for the oracle."""
        ns, ts, fs, us = [], [], [], []
        for gid, v, idx in self.geometry.meshes:
            a = (self.attrs or {}).get(gid, {})
            n, t, uv = a.get("normals"), a.get("tangents"), a.get("uvs")
            m = idx.shape[0]
            ns.append(np.asarray(n, np.float32)[idx].reshape(m, 9) if n is not None else np.zeros((m, 9), np.float32))
            ts.append(np.asarray(t, np.float32)[idx].reshape(m, 12) if t is not None else np.zeros((m, 12), np.float32))
            us.append(np.asarray(uv, np.float32)[idx].reshape(m, 6) if uv is not None else np.zeros((m, 6), np.float32))
            fs.append(np.full(m, (1 if n is not None else 0) | (2 if t is not None else 0) | (4 if uv is not None else 0)
                              | (8 if gid in self.geometry.quad_geoms else 0), np.uint8))
        if not ns:
            return (np.zeros((0, 9), np.float32), np.zeros((0, 12), np.float32), np.zeros(0, np.uint8),
                    np.zeros((0, 6), np.float32))
        return np.concatenate(ns), np.concatenate(ts), np.concatenate(fs), np.concatenate(us)

    def ptex_tables(self, material_recs=None):
        """Combined face table (rows rebased) and texels of all textured geometries, in geomID order; writes
        each geometry's first face into word 3 of its material record when given."""
        rows, texels, base_face, base_texel = [], [], 0, 0
        for gid in sorted(self.ptex):
            r, t = self.ptex[gid]
            if np.asarray(r).shape[1] == 10:  # quad-mesh textures: quad_ptex_tables
                continue
            r = np.array(r, np.int32, copy=True)
            r[:, 1] += base_texel
            adj = r[:, 2:5]
            adj[adj >= 0] += base_face
            rows.append(r)
            texels.append(np.asarray(t, np.float16).view(np.uint16))
            if material_recs is not None and gid < material_recs.shape[0]:
                material_recs.view(np.uint32)[gid, 3] = base_face
            base_face += r.shape[0]
            base_texel += t.size // 3
        if not rows:
            return np.zeros((0, 8), np.int32), np.zeros(3, np.uint16)
        return np.ascontiguousarray(np.concatenate(rows)), np.ascontiguousarray(np.concatenate(texels))

    def quad_ptex_tables(self):
        """The quad-mesh Ptex textures: [(geomID, rows (n, 10) int32, texels uint16)]."""
        return [(gid, np.ascontiguousarray(r, np.int32), np.ascontiguousarray(np.asarray(t, np.float16).view(np.uint16)))
                for gid, (r, t) in sorted(self.ptex.items()) if np.asarray(r).shape[1] == 10]

    def build(self, sel_module, device, bvh_kind=0, build_mode=None):
        """Creates and commits a selas_gb300 Scene with this content."""
        sc = sel_module.Scene(device, bvh_kind, build_mode)
        self.geometry.attach_to(sc)
        for gid, (pts, idx) in sorted((self.curves or {}).items()):
            sc.attach_curve_mesh(gid, pts, idx)
        self.attach_attributes(sc)
        for gid, m in self.materials.items():
            sc.set_material(gid, sel_module.material(**m))
        for ls, l in self.lights:
            sc.add_quad_light(ls, l["position"], l["direction"], l["x"], l["z"], l["radiance"])
        sc.set_background(self.background)
        if self.ibl:
            sc.set_ibl(self.ibl["light"], self.ibl.get("miss"), self.ibl.get("rotation", 0.0),
                       self.ibl.get("exposure", 1.0))
        for gid in sorted(self.ptex):
            rows, tex = self.ptex[gid]
            sc.set_ptex(gid, rows, tex)
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


# ---------------------------------------------------------------------------------------------------
# Per-face textures (Ptex model: one square texel block per triangle plus edge adjacency)
# ---------------------------------------------------------------------------------------------------
def triangle_adjacency(faces: np.ndarray):
    """Ptex FaceInfo adjacency of a triangle mesh: edge i of a face runs from vertex i to vertex i+1;
    adj[f, i] = neighbouring face across that edge (-1 on a boundary), adjedge[f, i] = the neighbour's edge
    index for the same edge.  Faces of k vertices give k edges each (a quad mesh: edges 0..3)."""
    f = np.asarray(faces, np.int64)
    n, k = f.shape
    a = np.concatenate([f[:, i] for i in range(k)])
    b = np.concatenate([f[:, (i + 1) % k] for i in range(k)])
    face_of = np.tile(np.arange(n), k)
    edge_of = np.repeat(np.arange(k), n)
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    key = lo * (int(f.max()) + 1) + hi
    order = np.argsort(key, kind="stable")
    ks = key[order]
    adj = np.full((n, k), -1, np.int32)
    adjedge = np.zeros((n, k), np.int32)
    same = np.nonzero(ks[1:] == ks[:-1])[0]
    for i in same:  # manifold edges appear exactly twice
        p, q = order[i], order[i + 1]
        if i + 2 < ks.size and ks[i + 2] == ks[i]:
            continue
        if i > 0 and ks[i - 1] == ks[i]:
            continue
        adj[face_of[p], edge_of[p]] = face_of[q]
        adjedge[face_of[p], edge_of[p]] = edge_of[q]
        adj[face_of[q], edge_of[q]] = face_of[p]
        adjedge[face_of[q], edge_of[q]] = edge_of[p]
    return adj, adjedge


def value_noise_texels(n_faces: int, log2: int, seed: int, lattice: int = 4, lo: float = 0.1, hi: float = 0.9):
    """Per-face value noise: a lattice x lattice grid of seeded RGB values, bilinearly interpolated to
    2^log2 x 2^log2 texels, stored as float16 (face-major, row-major, RGB interleaved)."""
    rng = np.random.default_rng(seed)
    res = 1 << log2
    grid = rng.uniform(lo, hi, size=(n_faces, lattice, lattice, 3))
    t = (np.arange(res) + 0.5) / res * (lattice - 1)
    i0 = np.minimum(np.floor(t).astype(int), lattice - 2)
    fr = t - i0
    rows = grid[:, i0, :, :] * (1 - fr)[None, :, None, None] + grid[:, i0 + 1, :, :] * fr[None, :, None, None]
    tex = rows[:, :, i0, :] * (1 - fr)[None, None, :, None] + rows[:, :, i0 + 1, :] * fr[None, None, :, None]
    return tex.astype(np.float16).reshape(-1)


def ptex_faces(faces: np.ndarray, log2: int):
    """Face table rows (log2, texel offset, adj0..2, adjedge0..2) as int32, one per triangle."""
    n = faces.shape[0]
    adj, adjedge = triangle_adjacency(faces)
    table = np.zeros((n, 8), np.int32)
    table[:, 0] = log2
    table[:, 1] = np.arange(n, dtype=np.int64) * (1 << (2 * log2))
    table[:, 2:5] = adj
    table[:, 5:8] = adjedge
    return table


def ptex_quad_faces(quads: np.ndarray, log2: int):
    """Face table rows (log2, texel offset, adj0..3, adjedge0..3) as int32, one per quad (Ptex quad faces: edge i
    from vertex i to vertex i+1, u along edge 0, v along edge 3 reversed)."""
    n = quads.shape[0]
    adj, adjedge = triangle_adjacency(quads)
    table = np.zeros((n, 10), np.int32)
    table[:, 0] = log2
    table[:, 1] = np.arange(n, dtype=np.int64) * (1 << (2 * log2))
    table[:, 2:6] = adj
    table[:, 6:10] = adjedge
    return table


def quad_cube(m: int = 3):
    """A cube of side 2 whose faces are m x m quads, outward-facing: (vertices (n, 3), quads (6 m^2, 4)); its
    eight corners have valence 3, every other vertex 4."""
    index = {}
    verts, quads = [], []

    def vid(p):
        key = tuple(np.round(p, 6))
        if key not in index:
            index[key] = len(verts)
            verts.append(p)
        return index[key]

    for axis in range(3):
        for sign in (1.0, -1.0):
            n = np.zeros(3)
            n[axis] = sign
            a = np.zeros(3)
            a[(axis + 1) % 3] = 1.0
            b = np.cross(n, a)
            for i in range(m):
                for j in range(m):
                    s0, s1 = -1 + 2 * i / m, -1 + 2 * (i + 1) / m
                    t0, t1 = -1 + 2 * j / m, -1 + 2 * (j + 1) / m
                    quads.append([vid(n + s0 * a + t0 * b), vid(n + s1 * a + t0 * b), vid(n + s1 * a + t1 * b),
                                  vid(n + s0 * a + t1 * b)])
    return np.array(verts, np.float32), np.array(quads, np.uint32)


def quad_fan(k: int = 5):
    """k quads around one interior vertex of valence k (centre, spoke midpoints, rim points), a disc with a
    boundary: (vertices, quads)."""
    verts = [[0.0, 0.0, 0.0]]
    for i in range(k):
        a = 2 * np.pi * i / k
        verts.append([np.cos(a), 0.0, np.sin(a)])
        b = 2 * np.pi * (i + 0.5) / k
        verts.append([1.5 * np.cos(b), 0.0, 1.5 * np.sin(b)])
    quads = [[0, 1 + 2 * i, 2 + 2 * i, 1 + 2 * ((i + 1) % k)] for i in range(k)]
    return np.array(verts, np.float32), np.array(quads, np.uint32)


def quad_textured_cubes(count: int = 4, m: int = 3, log2: int = 3, seed: int = 0x5E1A5F10) -> RenderScene:
    """Quad-mesh cubes of m x m quads a side (corner valence 3) with per-face Ptex value noise (2^log2 texels a
    side, the separable bicubic filter), rotated and scaled on a quad floor, a five-quad fan (interior valence 5)
    with its own Ptex, one 2 x 2 quad light and a dim background."""
    rng = np.random.default_rng(seed)
    v0, q0 = quad_cube(m)
    g = TriangleScene()
    mats, ptex = {}, {}
    for i in range(count):
        a = rng.uniform(0, 2 * np.pi)
        rot = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
        size = rng.uniform(0.5, 1.0)
        centre = np.array([rng.uniform(-3.5, 3.5), size, rng.uniform(-2.0, 2.0)])
        g.add_quads(i, (v0 @ rot.T * size + centre).astype(np.float32), q0)
        mats[i] = dict(shader=1, lightSetIndex=0, roughness=float(rng.uniform(0.2, 0.9)),
                       metallic=float(rng.random() < 0.3), ior=1.5, usesPtex=1)
        ptex[i] = (ptex_quad_faces(q0, log2), value_noise_texels(q0.shape[0], log2, seed + 31 * i))
    fv, fq = quad_fan(5)
    gid = count
    g.add_quads(gid, (fv * 1.2 + np.array([0.0, 0.01, 3.0])).astype(np.float32), fq)
    mats[gid] = dict(shader=1, lightSetIndex=0, roughness=0.6, ior=1.5, usesPtex=1)
    ptex[gid] = (ptex_quad_faces(fq, 4), value_noise_texels(fq.shape[0], 4, seed + 7))
    floor = np.array([[-20, 0, -20], [-20, 0, 20], [20, 0, 20], [20, 0, -20]], np.float32)
    g.add_quads(count + 1, floor, np.array([[0, 1, 2, 3]], np.uint32))
    mats[count + 1] = dict(shader=1, lightSetIndex=0, baseColor=(0.6, 0.6, 0.6), roughness=0.7, ior=1.5)
    light = dict(position=(0.0, 6.0, 0.0), direction=(0.0, -1.0, 0.0), x=(2.0, 0.0, 0.0), z=(0.0, 0.0, 2.0),
                 radiance=(20.0, 18.0, 15.0))
    cam = dict(position=(0.0, 4.0, -9.0), look_at=(0.0, 0.8, 0.0), up=(0.0, 1.0, 0.0), fov_degrees=55.0)
    return RenderScene(g, mats, [(0, light)], (0.1, 0.1, 0.12), cam, ptex=ptex)


def curve_strands(strands: int = 24, points: int = 6, length: float = 2.0, root: float = 0.06, tip: float = 0.015,
                  seed: int = 0x5E1A5C01):
    """Hair-like strands for round B-spline curves, laid out as the reference's curve model builder lays out a
    strand of m control points (CDisneySceneBuildProcessor.cpp:177-220): the first and last points repeated, radii
    from `root` to `tip` along the strand, m - 1 segments starting at consecutive points.  Returns (points (n, 4)
    x, y, z, radius; indices (segments,))."""
    rng = np.random.default_rng(seed)
    pts, idx = [], []
    for _ in range(strands):
        base = np.array([rng.uniform(-1.5, 1.5), 0.0, rng.uniform(-1.0, 1.0)])
        bend = rng.normal(scale=0.4, size=3)
        cps = [base + np.array([0.0, length * k / (points - 1), 0.0]) + bend * (k / (points - 1)) ** 2
               for k in range(points)]
        widths = [root + (tip - root) * k / (points - 1) for k in range(points)]
        first = len(pts)
        pts.append(list(cps[0]) + [root])
        pts += [list(c) + [w] for c, w in zip(cps, widths)]
        pts.append(list(cps[-1]) + [tip])
        idx += [first + k for k in range(points - 1)]
    return np.array(pts, np.float32), np.array(idx, np.uint32)


def textured_spheres(count: int = 6, level: int = 3, log2: int = 4, seed: int = 0x5E1A5F00) -> RenderScene:
    """A few displaced icospheres with per-face Ptex value-noise base colour (16 x 16 FP16 RGB by default)
    on a grey floor, under one 2 x 2 quad light and a dim background."""
    rng = np.random.default_rng(seed)
    unit_v, f = icosphere(level)
    g = TriangleScene()
    mats, ptex = {}, {}
    for i in range(count):
        centre = np.array([rng.uniform(-4, 4), rng.uniform(1.0, 2.5), rng.uniform(-2, 2)])
        radius = rng.uniform(0.6, 1.2)
        disp = 1.0 + 0.1 * value_noise_dirs(unit_v, rng)
        g.add(i, (centre + unit_v * (radius * disp)[:, None]).astype(np.float32), f.astype(np.uint32))
        mats[i] = dict(shader=1, lightSetIndex=0, roughness=float(rng.uniform(0.05, 1.0)),
                       metallic=float(rng.random() < 0.3), ior=1.5, usesPtex=1)
        ptex[i] = (ptex_faces(f, log2), value_noise_texels(f.shape[0], log2, seed + 17 * i))
    floor = np.array([[-20, 0, -20], [-20, 0, 20], [20, 0, 20], [20, 0, -20]], np.float32)
    g.add(count, floor, np.array([[0, 1, 2], [0, 2, 3]], np.uint32))
    mats[count] = dict(shader=1, lightSetIndex=0, baseColor=(0.6, 0.6, 0.6), roughness=0.7, ior=1.5)
    light = dict(position=(0.0, 6.0, 0.0), direction=(0.0, -1.0, 0.0), x=(2.0, 0.0, 0.0), z=(0.0, 0.0, 2.0),
                 radiance=(30.0, 28.0, 25.0))
    cam = dict(position=(0.0, 3.0, -11.0), look_at=(0.0, 1.5, 0.0), up=(0.0, 1.0, 0.0), fov_degrees=55.0)
    return RenderScene(g, mats, [(0, light)], (0.05, 0.05, 0.08), cam, ptex)


def _noise_texels_f32(n_faces: int, log2: int, rng: np.random.Generator, lattice: int = 4, lo: float = 0.1,
                      hi: float = 0.9, chunk: int = 1 << 15) -> np.ndarray:
    """value_noise_texels computed in float32 chunks (the same construction; large meshes)."""
    res = 1 << log2
    out = np.empty((n_faces, res, res, 3), np.float16)
    t = (np.arange(res, dtype=np.float32) + 0.5) / res * (lattice - 1)
    i0 = np.minimum(np.floor(t).astype(int), lattice - 2)
    fr = (t - i0).astype(np.float32)
    for s in range(0, n_faces, chunk):
        e = min(n_faces, s + chunk)
        grid = rng.uniform(lo, hi, size=(e - s, lattice, lattice, 3)).astype(np.float32)
        rows = grid[:, i0, :, :] * (1 - fr)[None, :, None, None] + grid[:, i0 + 1, :, :] * fr[None, :, None, None]
        out[s:e] = rows[:, :, i0, :] * (1 - fr)[None, None, :, None] + rows[:, :, i0 + 1, :] * fr[None, None, :, None]
    return out.reshape(-1)


def vcm_room(icospheres: int = 24, level: int = 6, glass: int = 40, glass_level: int = 3, log2: int = 4,
             seed: int = 0x5E1A5003) -> RenderScene:
    """The VCM scene: displaced icospheres (per-face Ptex value-noise base colour, 16 x 16 FP16 texels) and
    glass spheres (specTrans 1, ior 1.5) inside a 20 x 20 x 10 room shell lit by one 2 x 2 quad light
    below the ceiling.  Per mesh: roughness U[0.05, 1], metallic Bernoulli(0.3), baseColor U[0.1, 0.9]^3.
    Defaults: 24 x 81,920 + 40 x 1,280 + 12 = 2,017,292 triangles."""
    rng = np.random.default_rng(seed)
    unit_v, f = icosphere(level)
    face_table = ptex_faces(f, log2)  # same topology for every icosphere
    g = TriangleScene()
    mats, ptex = {}, {}

    def disney(**kw):
        m = dict(shader=1, lightSetIndex=0, roughness=float(rng.uniform(0.05, 1.0)),
                 metallic=float(rng.random() < 0.3), ior=1.5,
                 baseColor=tuple(float(x) for x in rng.uniform(0.1, 0.9, 3)))
        m.update(kw)
        return m

    gid = 0
    for _ in range(icospheres):
        radius = rng.uniform(0.6, 1.5)
        centre = np.array([rng.uniform(-8.0, 8.0), rng.uniform(radius, 6.0), rng.uniform(-8.0, 8.0)])
        disp = 1.0 + 0.1 * value_noise_dirs(unit_v, rng)
        g.add(gid, (centre + unit_v * (radius * disp)[:, None]).astype(np.float32), f.astype(np.uint32))
        mats[gid] = disney(usesPtex=1)
        ptex[gid] = (face_table, _noise_texels_f32(f.shape[0], log2, rng))
        gid += 1
    gv, gf = icosphere(glass_level)
    for _ in range(glass):
        radius = rng.uniform(0.3, 0.8)
        centre = np.array([rng.uniform(-8.0, 8.0), rng.uniform(radius, 6.0), rng.uniform(-8.0, 8.0)])
        g.add(gid, (centre + gv * radius).astype(np.float32), gf.astype(np.uint32))
        mats[gid] = disney(specTrans=1.0, metallic=0.0, baseColor=(1.0, 1.0, 1.0))
        gid += 1
    # room shell, faces pointing inwards: floor y=0, ceiling y=10, walls at x, z = +-10
    lo, hi = -10.0, 10.0
    c = np.array([[lo, 0, lo], [hi, 0, lo], [hi, 0, hi], [lo, 0, hi], [lo, 10, lo], [hi, 10, lo], [hi, 10, hi],
                  [lo, 10, hi]], np.float32)
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (3, 0, 4, 7)]
    tris = np.array([[q[0], q[1], q[2]] for q in quads] + [[q[0], q[2], q[3]] for q in quads], np.uint32)
    g.add(gid, c, tris)
    mats[gid] = disney(usesPtex=1, metallic=0.0)
    ptex[gid] = (ptex_faces(tris, log2), _noise_texels_f32(tris.shape[0], log2, rng))
    light = dict(position=(0.0, 9.9, 0.0), direction=(0.0, -1.0, 0.0), x=(2.0, 0.0, 0.0), z=(0.0, 0.0, 2.0),
                 radiance=(40.0, 38.0, 34.0))
    cam = dict(position=(0.0, 5.0, -9.5), look_at=(0.0, 3.0, 0.0), up=(0.0, 1.0, 0.0), fov_degrees=75.0)
    return RenderScene(g, mats, [(0, light)], (0.0, 0.0, 0.0), cam, ptex)


def icosphere_field(level: int = 6, seed: int = 0x5E1A5001) -> RenderScene:
    """The ray-query geometry (64 displaced icospheres over a 200 x 200 ground plane) as a render scene:
    grey Disney surfaces (roughness 0.5) under one 80 x 80 quad light, the ray-query camera."""
    g = displaced_icospheres(level=level, seed=seed)
    mats = {gid: dict(shader=1, lightSetIndex=0, roughness=0.5, ior=1.5, baseColor=(0.6, 0.6, 0.6))
            for gid, _, _ in g.meshes}
    light = dict(position=(0.0, 150.0, 0.0), direction=(0.0, -1.0, 0.0), x=(80.0, 0.0, 0.0), z=(0.0, 0.0, 80.0),
                 radiance=(6.0, 6.0, 6.0))
    cam = dict(position=(0.0, 70.0, -170.0), look_at=(0.0, 40.0, 0.0), up=(0.0, 1.0, 0.0), fov_degrees=60.0)
    return RenderScene(g, mats, [(0, light)], (0.05, 0.05, 0.05), cam, {})


def orbit_camera(camera: dict, yaw: float) -> dict:
    """The camera turned by `yaw` radians about the vertical axis through its look-at point."""
    p, c = np.asarray(camera["position"], np.float64), np.asarray(camera["look_at"], np.float64)
    d = p - c
    cs, sn = np.cos(yaw), np.sin(yaw)
    q = c + np.array([cs * d[0] + sn * d[2], d[1], -sn * d[0] + cs * d[2]])
    return {**camera, "position": tuple(float(x) for x in q)}


# ---------------------------------------------------------------------------------------------------
# Instanced scenes (two levels: scene -> instances of scenes -> their instances)
# ---------------------------------------------------------------------------------------------------
@dataclass
class InstancedRenderScene:
    """Render scenes linked by instances.  parts[0] is the world: its lights, background and camera are the
    render's; instances[i] lists (instID, index of the instanced part, local-to-world 3 x 4 or 4 x 4) attached
    to part i.  A part's materials and Ptex belong to its own meshes (ModelDataFromRayIds picks them by the
    hit's instance ids and geomID)."""
    parts: list
    instances: list

    @property
    def camera(self):
        return self.parts[0].camera

    def graph(self):
        """Meshes and instances of every part, as the instanced oracles take them."""
        return [{"meshes": p.geometry.meshes, "instances": list(self.instances[i])} for i, p in enumerate(self.parts)]

    def release(self, built) -> None:
        """Releases the scenes `build` returned, every scene before the scenes it instances."""
        left = set(range(len(built)))
        while left:
            for i in sorted(left):
                if not any(i in {pi for _, pi, _ in self.instances[j]} for j in left):
                    built[i].release()
                    left.discard(i)
                    break

    def build(self, sel_module, device, build_mode=None):
        """Creates and commits one selas_gb300 Scene per part, instanced parts first; returns them in part order
        (free them with `release`)."""
        built = [None] * len(self.parts)

        def make(i):
            if built[i] is not None:
                return
            for _, pi, _ in self.instances[i]:
                make(pi)
            p = self.parts[i]
            sc = sel_module.Scene(device, 0, build_mode)
            if p.geometry.meshes:
                p.geometry.attach_to(sc)
                p.attach_attributes(sc)
            for gid, (pts, idx) in sorted((getattr(p, "curves", None) or {}).items()):
                sc.attach_curve_mesh(gid, pts, idx)
            for gid, m in p.materials.items():
                sc.set_material(gid, sel_module.material(**m))
            for ls, l in p.lights:
                sc.add_quad_light(ls, l["position"], l["direction"], l["x"], l["z"], l["radiance"])
            sc.set_background(p.background)
            if p.ibl:
                sc.set_ibl(p.ibl["light"], p.ibl.get("miss"), p.ibl.get("rotation", 0.0), p.ibl.get("exposure", 1.0))
            for gid in sorted(p.ptex):
                rows, tex = p.ptex[gid]
                sc.set_ptex(gid, rows, tex)
            for iid, pi, m in self.instances[i]:
                sc.attach_instance(iid, built[pi], m)
            sc.commit()
            built[i] = sc

        for i in range(len(self.parts)):
            make(i)
        return built

    def sel_camera(self, sel_module, width, height):
        return self.parts[0].sel_camera(sel_module, width, height)


def _rotation_matrix(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def fbm_heightfield(n: int, octaves: int, seed: int, chunk_rows: int = 256) -> np.ndarray:
    """(n, n) float32 fractal value noise: `octaves` octaves of bilinear value noise on lattices doubling from
    4 x 4, amplitudes halving, normalised to [-1, 1]."""
    rng = np.random.default_rng(seed)
    lattices = [rng.uniform(-1, 1, size=((4 << o) + 1, (4 << o) + 1)).astype(np.float32) for o in range(octaves)]
    out = np.empty((n, n), np.float32)
    t = np.linspace(0.0, 1.0, n, dtype=np.float32)
    for r0 in range(0, n, chunk_rows):
        r1 = min(n, r0 + chunk_rows)
        acc = np.zeros((r1 - r0, n), np.float32)
        amp = 1.0
        for lat in lattices:
            m = lat.shape[0] - 1
            y = t[r0:r1] * m
            x = t * m
            iy = np.minimum(y.astype(np.int64), m - 1)
            ix = np.minimum(x.astype(np.int64), m - 1)
            fy = (y - iy)[:, None]
            fx = (x - ix)[None, :]
            a = lat[iy][:, ix]
            b = lat[iy][:, ix + 1]
            c = lat[iy + 1][:, ix]
            d = lat[iy + 1][:, ix + 1]
            acc += amp * ((a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy)
            amp *= 0.5
        out[r0:r1] = acc
    out /= np.float32(2.0 - 2.0 ** (1 - octaves))
    return out


def heightfield_mesh(h: np.ndarray, extent: float, height: float):
    """Grid mesh of a heightfield over [-extent, extent]^2 in x, z: 2 (n-1)^2 triangles, uint32 indices."""
    n = h.shape[0]
    xs = np.linspace(-extent, extent, n, dtype=np.float32)
    v = np.empty((n * n, 3), np.float32)
    v[:, 0] = np.tile(xs, n)
    v[:, 2] = np.repeat(xs, n)
    v[:, 1] = h.reshape(-1) * np.float32(height)
    i = np.arange(n - 1, dtype=np.uint32)
    a = (i[:, None] * n + i[None, :]).reshape(-1)  # row z, column x
    idx = np.empty((a.size * 2, 3), np.uint32)
    idx[0::2, 0], idx[0::2, 1], idx[0::2, 2] = a, a + n, a + n + 1
    idx[1::2, 0], idx[1::2, 1], idx[1::2, 2] = a, a + n + 1, a + 1
    return v, idx


def instanced_terrain(grid: int = 4096, instances: int = 5000, mesh_level: int = 5, log2: int = 2, groups: int = 0,
                      seed: int = 0x5E1A5004) -> InstancedRenderScene:
    """The instanced-terrain configuration: a grid x grid fBm heightfield (8 octaves; 2 (grid-1)^2 triangles)
    over [-1000, 1000]^2 and `instances` instances of one displaced icosphere of 20 * 4^mesh_level triangles
    (level 5: 20,480) with per-face Ptex FP16 value noise (2^log2 texels a side), each with a random rotation
    and a uniform scale in [0.5, 2] x 8, resting on the terrain.  groups > 0 adds a second instancing level:
    that many instances of a cluster scene holding three instances of the mesh.  One quad light (sun) and a
    sky background; the camera looks over the terrain."""
    rng = np.random.default_rng(seed)
    extent, height = 1000.0, 120.0
    h = fbm_heightfield(grid, 8, seed + 1)
    tv, tf = heightfield_mesh(h, extent, height)
    world = TriangleScene()
    world.add(0, tv, tf)
    unit_v, f = icosphere(mesh_level)
    disp = 1.0 + 0.25 * value_noise_dirs(unit_v, rng)
    mesh = TriangleScene()
    mesh.add(0, (unit_v * disp[:, None]).astype(np.float32), f.astype(np.uint32))
    mesh_mats = {0: dict(shader=1, lightSetIndex=0, roughness=0.45, metallic=0.0, ior=1.5, usesPtex=1)}
    mesh_ptex = {0: (ptex_faces(f, log2), _noise_texels_f32(f.shape[0], log2, rng))}
    parts = [RenderScene(world, {0: dict(shader=1, lightSetIndex=0, baseColor=(0.35, 0.32, 0.25), roughness=0.8,
                                         ior=1.5)},
                         [(0, dict(position=(0.0, 900.0, 0.0), direction=(0.0, -1.0, 0.0), x=(300.0, 0.0, 0.0),
                                   z=(0.0, 0.0, 300.0), radiance=(40.0, 38.0, 34.0)))],
                         (0.35, 0.45, 0.6),
                         dict(position=(-700.0, 260.0, -700.0), look_at=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                              fov_degrees=60.0)),
             RenderScene(mesh, mesh_mats, [], (0.0, 0.0, 0.0), {}, mesh_ptex)]
    inst_lists = [[], []]

    def ground(x, z):
        gx = np.clip(((x + extent) / (2 * extent) * (grid - 1)).astype(np.int64), 0, grid - 1)
        gz = np.clip(((z + extent) / (2 * extent) * (grid - 1)).astype(np.int64), 0, grid - 1)
        return h[gz, gx] * height

    xz = rng.uniform(-0.9 * extent, 0.9 * extent, size=(instances, 2))
    scales = rng.uniform(0.5, 2.0, instances) * 8.0
    ys = ground(xz[:, 0], xz[:, 1]) + scales * 0.6
    for k in range(instances):
        m = np.zeros((3, 4), np.float32)
        m[:, :3] = _rotation_matrix(rng) * scales[k]
        m[:, 3] = (xz[k, 0], ys[k], xz[k, 1])
        inst_lists[0].append((k + 1, 1, m))  # instIDs share the world's ID space with its terrain (0)
    if groups:
        cluster = TriangleScene()
        parts.append(RenderScene(cluster, {}, [], (0.0, 0.0, 0.0), {}, {}))
        inst_lists.append([])
        for j in range(3):
            m = np.zeros((3, 4), np.float32)
            m[:, :3] = _rotation_matrix(rng) * 0.6
            m[:, 3] = rng.uniform(-1.5, 1.5, 3)
            inst_lists[2].append((100 + j, 1, m))
        gxz = rng.uniform(-0.9 * extent, 0.9 * extent, size=(groups, 2))
        gs = rng.uniform(4.0, 12.0, groups)
        gy = ground(gxz[:, 0], gxz[:, 1]) + gs * 2.0
        for k in range(groups):
            m = np.zeros((3, 4), np.float32)
            m[:, :3] = _rotation_matrix(rng) * gs[k]
            m[:, 3] = (gxz[k, 0], gy[k], gxz[k, 1])
            inst_lists[0].append((instances + 1 + k, 2, m))
    return InstancedRenderScene(parts, inst_lists)


def terrain_views(scene: InstancedRenderScene, count: int = 16):
    """`count` cameras circling the terrain at two heights, looking at its centre."""
    cams = []
    for k in range(count):
        a = 2 * np.pi * k / count
        r = 700.0 if k % 2 == 0 else 450.0
        y = 260.0 if k % 2 == 0 else 160.0
        cams.append(dict(position=(r * np.cos(a), y, r * np.sin(a)), look_at=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                         fov_degrees=60.0))
    return cams


def sky_ibl(width: int = 256, height: int = 128, sun=(0.4, 0.75, 0.3), sun_radius: float = 0.06,
            sun_radiance=(60.0, 52.0, 40.0), miss_size=(64, 32), rotation: float = 0.3, exposure: float = 1.5,
            seed: int = 0x5E1A5105) -> dict:
    """A synthetic latitude-longitude sky for the image-based light: a zenith-to-horizon gradient with seeded
    value-noise clouds, a dark ground hemisphere and a bright sun disc; the miss image is a coarser copy
    without the sun.  Returns the dict RenderScene.ibl takes."""
    rng = np.random.default_rng(seed)

    def image(w, h, with_sun):
        theta = (np.arange(h, dtype=np.float64) + 0.5) * np.pi / h
        phi = (np.arange(w, dtype=np.float64) + 0.5) * 2 * np.pi / w - np.pi
        th, ph = np.meshgrid(theta, phi, indexing="ij")
        d = np.stack([np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph)], -1)
        up = np.clip(d[..., 1], 0.0, 1.0)[..., None]
        sky = (1.0 - up) * np.array([0.9, 0.95, 1.0]) + up * np.array([0.25, 0.4, 0.85])
        ground = np.array([0.12, 0.1, 0.08])
        img = np.where(d[..., 1:2] > 0, sky, ground)
        lat = rng.uniform(0.7, 1.3, size=(8, 16))
        iy = np.minimum((th / np.pi * 8).astype(int), 7)
        ix = np.minimum(((ph + np.pi) / (2 * np.pi) * 16).astype(int), 15)
        img = img * lat[iy, ix][..., None]
        if with_sun:
            s = np.array(sun, np.float64)
            s /= np.linalg.norm(s)
            img = np.where((np.arccos(np.clip(d @ s, -1, 1)) < sun_radius)[..., None], np.array(sun_radiance), img)
        return img.astype(np.float32)

    return dict(light=image(width, height, True), miss=image(miss_size[0], miss_size[1], False), rotation=rotation,
                exposure=exposure)


def smooth_spheres(count: int = 4, level: int = 3, seed: int = 0x5E1A5106) -> RenderScene:
    """Displaced icospheres shaded with vertex normals (the normalised radial direction) on a grey floor; the
    even ones also carry vertex tangents (around +y, alternating handedness).  One quad light, a dim
    background."""
    rng = np.random.default_rng(seed)
    unit_v, f = icosphere(level)
    g = TriangleScene()
    mats, attrs = {}, {}
    for i in range(count):
        centre = np.array([rng.uniform(-3, 3), rng.uniform(1.0, 2.0), rng.uniform(-2, 2)])
        radius = rng.uniform(0.6, 1.1)
        disp = 1.0 + 0.08 * value_noise_dirs(unit_v, rng)
        g.add(i, (centre + unit_v * (radius * disp)[:, None]).astype(np.float32), f.astype(np.uint32))
        mats[i] = dict(shader=1, lightSetIndex=0, baseColor=tuple(rng.uniform(0.2, 0.9, 3)),
                       roughness=float(rng.uniform(0.1, 0.8)), metallic=float(i % 3 == 0), ior=1.5)
        n = unit_v.astype(np.float32)
        a = {"normals": n}
        if i % 2 == 0:
            t = np.cross(np.array([0.0, 1.0, 0.0]), unit_v)
            t /= np.maximum(np.linalg.norm(t, axis=1, keepdims=True), 1e-6)
            sign = np.where(np.arange(unit_v.shape[0]) % 2 == 0, 1.0, -1.0)[:, None]
            a["tangents"] = np.concatenate([t, sign], 1).astype(np.float32)
        attrs[i] = a
    floor = np.array([[-20, 0, -20], [-20, 0, 20], [20, 0, 20], [20, 0, -20]], np.float32)
    g.add(count, floor, np.array([[0, 1, 2], [0, 2, 3]], np.uint32))
    mats[count] = dict(shader=1, lightSetIndex=0, baseColor=(0.6, 0.6, 0.6), roughness=0.7, ior=1.5)
    light = dict(position=(0.0, 6.0, 0.0), direction=(0.0, -1.0, 0.0), x=(2.0, 0.0, 0.0), z=(0.0, 0.0, 2.0),
                 radiance=(30.0, 28.0, 25.0))
    cam = dict(position=(0.0, 3.0, -10.0), look_at=(0.0, 1.2, 0.0), up=(0.0, 1.0, 0.0), fov_degrees=55.0)
    return RenderScene(g, mats, [(0, light)], (0.05, 0.05, 0.08), cam, {}, attrs=attrs)


# ---------------------------------------------------------------------------------------------------
# Scene files: the reference's scene JSON (model and subscene instances with transforms, background) with models
# as Wavefront OBJ text and materials as the reference's material JSON files.  The reference cooks FBX / OBJ
# models through assimp (BuildCommon/ImportModel.cpp) into binary model resources; the OBJ reader here stands in
# for that import for OBJ content.
# ---------------------------------------------------------------------------------------------------
def load_obj(text: str, with_uvs: bool = False):
    """Wavefront OBJ text -> list of (material name, vertices (n, 3) f32, indices (m, 3) u32, normals (n, 3) or
    None), one entry per `usemtl` group in order of first use ("" before any); with_uvs appends uvs (n, 2) or
    None to each entry.  Faces may be polygons (fanned from their first corner) with v, v/vt, v//vn or v/vt/vn
    corners and negative (relative) indices; a group's vertices are its distinct (position, uv, normal) triples."""
    pos, nrm, tex = [], [], []
    groups = {}
    order = []
    cur = ""

    def index(tok, count):
        k = int(tok)
        return k - 1 if k > 0 else count + k

    for line in text.splitlines():
        parts = line.split("#", 1)[0].split()
        if not parts:
            continue
        tag = parts[0]
        if tag == "v":
            pos.append([float(x) for x in parts[1:4]])
        elif tag == "vn":
            nrm.append([float(x) for x in parts[1:4]])
        elif tag == "vt":
            tex.append([float(x) for x in parts[1:3]] + [0.0] * max(0, 3 - len(parts)))
        elif tag == "usemtl":
            cur = parts[1] if len(parts) > 1 else ""
        elif tag == "f":
            corners = []
            for c in parts[1:]:
                f = c.split("/")
                vi = index(f[0], len(pos))
                ti = index(f[1], len(tex)) if len(f) > 1 and f[1] else -1
                ni = index(f[2], len(nrm)) if len(f) > 2 and f[2] else -1
                if not 0 <= vi < len(pos) or not -1 <= ni < len(nrm) or not -1 <= ti < len(tex):
                    raise ValueError(f"face corner {c!r} indexes past the vertices read so far")
                corners.append((vi, ni, ti))
            if len(corners) < 3:
                raise ValueError("a face needs at least three corners")
            if cur not in groups:
                groups[cur] = ({}, [])
                order.append(cur)
            remap, tris = groups[cur]
            ids = [remap.setdefault(key, len(remap)) for key in corners]
            for k in range(1, len(ids) - 1):
                tris.append((ids[0], ids[k], ids[k + 1]))
    pos_a = np.asarray(pos, np.float32).reshape(-1, 3)
    nrm_a = np.asarray(nrm, np.float32).reshape(-1, 3)
    tex_a = np.asarray(tex, np.float32).reshape(-1, 2)
    out = []
    for name in order:
        remap, tris = groups[name]
        keys = sorted(remap, key=remap.get)
        v = pos_a[[k[0] for k in keys]]
        has_n = all(k[1] >= 0 for k in keys)
        n = nrm_a[[k[1] for k in keys]] if has_n and keys else None
        entry = (name, np.ascontiguousarray(v), np.asarray(tris, np.uint32).reshape(-1, 3), n)
        if with_uvs:
            has_t = all(k[2] >= 0 for k in keys)
            entry += (np.ascontiguousarray(tex_a[[k[2] for k in keys]]) if has_t and keys else None,)
        out.append(entry)
    return out


def _material_fields(m) -> dict:
    out = {}
    for name, _ in type(m)._fields_:
        v = getattr(m, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def load_scene_file(path, camera: dict = None, lights: list = (), materials_dir=None) -> "InstancedRenderScene":
    """A scene JSON file (ParseSceneFile, BuildCommon/CSceneBuildProcessor.cpp:32-63) as an InstancedRenderScene:
    part 0 is the world (the given lights and camera, the file's backgroundIntensity), each distinct model an
    instanced part (its OBJ `usemtl` groups geomIDs 0, 1, ... with the material `<materials_dir>/<name>.json`
    when that file exists, else the default material; `usesPtex` is cleared, since no Ptex texels come with an
    OBJ; a base colour naming a .hdr image makes it the group's 2D base-colour texture at the OBJ's uvs), and each
    subscene file a part instancing its own models (one level of subscenes).  Asset paths are read
    relative to the scene file's folder; the image-based light the file names (a .hdr image or a dual-IBL JSON
    file, `load_ibl`) lights the world when the file exists.  Without a camera, one looks at the instanced
    bounds from outside them."""
    import pathlib

    import selas_gb300 as sel

    path = pathlib.Path(path)
    mat_dir = pathlib.Path(materials_dir) if materials_dir else path.parent
    parts, instances, index_of = [None], [[]], {}

    def model_part(asset):
        key = ("model", asset)
        if key in index_of:
            return index_of[key]
        geometry, mats, attrs, images = TriangleScene(), {}, {}, {}
        for gid, (name, v, idx, n, uv) in enumerate(load_obj((path.parent / asset).read_text(), with_uvs=True)):
            geometry.add(gid, v, idx)
            f = mat_dir / f"{name}.json"
            if name and f.exists():
                m, texture = sel.material_from_json(f.read_text())
                fields = _material_fields(m)
                fields["usesPtex"] = 0
                mats[gid] = fields
                if texture.lower().endswith(".hdr") and (mat_dir / texture).exists():
                    images[gid] = read_hdr((mat_dir / texture).read_bytes())
            a = {}
            if n is not None:
                a["normals"] = n
            if uv is not None:
                a["uvs"] = uv
            if a:
                attrs[gid] = a
        parts.append(RenderScene(geometry, mats, [], (0.0, 0.0, 0.0), {}, {}, None, attrs or None, images or None))
        instances.append([])
        index_of[key] = len(parts) - 1
        return index_of[key]

    def scene_instances(desc, owner, allow_subscenes):
        next_id = 1
        for asset, m in desc["models"]:
            instances[owner].append((next_id, model_part(asset), m))
            next_id += 1
        for asset, m in desc["scenes"]:
            if not allow_subscenes:
                raise ValueError(f"{asset}: subscenes of subscenes exceed the two instance levels")
            key = ("scene", asset)
            if key not in index_of:
                sub = sel.scene_description_from_json((path.parent / asset).read_text())
                parts.append(RenderScene(TriangleScene(), {}, [], (0.0, 0.0, 0.0), {}))
                instances.append([])
                index_of[key] = len(parts) - 1
                scene_instances(sub, index_of[key], False)
            instances[owner].append((next_id, index_of[key], m))
            next_id += 1

    desc = sel.scene_description_from_json(path.read_text())
    scene_instances(desc, 0, True)
    if camera is None:
        corners = []

        def collect(i, xform):
            p = parts[i]
            if p is not None and p.geometry.meshes:  # part 0, the world, holds no meshes
                lo, hi = p.geometry.bounds()
                box = np.array([[x, y, z, 1.0] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])])
                corners.append((xform @ box.T).T[:, :3])
            for _, j, m in instances[i]:
                collect(j, xform @ np.asarray(m, np.float64))

        collect(0, np.eye(4))
        pts = np.concatenate(corners) if corners else np.zeros((1, 3))
        lo, hi = pts.min(axis=0), pts.max(axis=0)
        centre, radius = (lo + hi) / 2, max(float(np.linalg.norm(hi - lo)) / 2, 1e-3)
        camera = dict(position=tuple(centre + np.array([0.0, 0.5, -2.5]) * radius), look_at=tuple(centre),
                      up=(0.0, 1.0, 0.0), fov_degrees=45.0)
    ibl = None
    if desc["ibl"] and (path.parent / desc["ibl"]).exists():
        ibl = load_ibl(path.parent / desc["ibl"])
    parts[0] = RenderScene(TriangleScene(), {}, list(lights), tuple(desc["background"]), camera, {}, ibl)
    return InstancedRenderScene(parts, instances)


def read_hdr(data: bytes) -> np.ndarray:
    """Radiance RGBE (.hdr) image bytes -> float32 (height, width, 3), rows top to bottom (the format of Greg Ward's
    Radiance; the reference reads it through stb_image, BuildImageBasedLight.cpp:124-150).  Flat and new-style
    run-length scanlines; `-Y h +X w` orientation only."""
    pos = 0

    def line():
        nonlocal pos
        end = data.index(b"\n", pos)
        s = data[pos:end].decode("ascii", "replace")
        pos = end + 1
        return s

    if not line().startswith("#?"):
        raise ValueError("not a Radiance HDR file")
    while True:
        s = line()
        if s == "":
            break
        if s.startswith("FORMAT=") and s != "FORMAT=32-bit_rle_rgbe":
            raise ValueError(f"unsupported {s}")
    res = line().split()
    if len(res) != 4 or res[0] != "-Y" or res[2] != "+X":
        raise ValueError("only -Y height +X width images are read")
    h, w = int(res[1]), int(res[3])
    rgbe = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if 8 <= w < 32768 and data[pos] == 2 and data[pos + 1] == 2 and (data[pos + 2] << 8 | data[pos + 3]) == w:
            pos += 4
            for c in range(4):  # one run-length coded channel after the other
                x = 0
                while x < w:
                    n = data[pos]
                    pos += 1
                    if n > 128:
                        n -= 128
                        if x + n > w:
                            raise ValueError("run past the end of a scanline")
                        rgbe[y, x:x + n, c] = data[pos]
                        pos += 1
                    else:
                        if n == 0 or x + n > w:
                            raise ValueError("bad count in a scanline")
                        rgbe[y, x:x + n, c] = np.frombuffer(data, np.uint8, n, pos)
                        pos += n
                    x += n
        else:
            rgbe[y] = np.frombuffer(data, np.uint8, 4 * w, pos).reshape(w, 4)
            pos += 4 * w
    e = rgbe[..., 3].astype(np.int32)
    scale = np.where(e > 0, np.ldexp(np.float32(1.0), e - (128 + 8)), 0.0).astype(np.float32)
    return rgbe[..., :3].astype(np.float32) * scale[..., None]


def load_ibl(path) -> dict:
    """An image-based light asset as RenderScene.ibl takes it: a .hdr image (ImportImageBasedLight,
    BuildImageBasedLight.cpp:155-178: no miss image, no rotation) or a dual-IBL JSON file {"light", "miss",
    "rotationDegrees", "exposure"} (ImageBasedLightBuildProcessor.cpp:52-119: rotation in radians, exposure scale
    2^exposure), its images read relative to the file."""
    import json
    import pathlib

    path = pathlib.Path(path)
    if path.suffix.lower() == ".json":
        d = json.loads(path.read_text())
        if "light" not in d or "miss" not in d:
            raise ValueError(f"{path}: a dual IBL names a light and a miss image")
        return dict(light=read_hdr((path.parent / d["light"]).read_bytes()),
                    miss=read_hdr((path.parent / d["miss"]).read_bytes()),
                    rotation=float(np.float32(d.get("rotationDegrees", 0.0)) * np.float32(np.pi / 180.0)),
                    exposure=float(np.float32(2.0) ** np.float32(d.get("exposure", 0.0))))
    return dict(light=read_hdr(path.read_bytes()), miss=None, rotation=0.0, exposure=1.0)

"""The cooked-asset test scenes: a Cornell box split the way the reference's asset pipeline splits a scene
(SceneResource -> SubsceneResource instances -> ModelResource instances -> meshes), as plain Python data.

tests/golden/make_cooked.py writes these descriptions as cooked blobs with the reference's own serializer
(tests/golden/cooked/_Assets/...); the tests parse and render those blobs with the product's loader and compare
the result with what the descriptions say: the mesh table FindMeshMaterial resolves (ModelResource.cpp:203-229),
and images against the oracle's instanced path tracer over `instanced_scene(description)`.

What the scenes exercise:
  * "cornell": two subscenes ("room", "props"); the room's model instanced at scale 2 by the scene's first
    subscene instance (the walls are authored at half size); the props subscene instanced with a small shift, its
    quad-mesh box model instanced twice (short and tall box: non-uniform scale, rotation, translation);
  * materials from the model's own sorted table (binary search), from the subscene's scene materials (linear
    search), a model material shadowing a scene material of the same name, and an unknown name taking the
    default material; a floor material with a 2D base-colour texture (a Float3 Textures blob with two mips, of
    which shading samples mip 0); walls with normals, tangents and uvs, the box model without attributes;
  * "cornell_sky": the same subscenes under an image-based light (an IBL blob with the reference's densities);
  * "cornell_ptex": a subscene whose material samples Ptex (eUsesPtex), which the loader refuses unless asked to
    render such materials with their base colour;
  * "cornell_hair": the Cornell subscenes plus a third whose model holds a plate mesh and two round B-spline
    curves (CurveMetaData ranges over one shared curve vertex array, the material named by curveModelName and
    found among the subscene's scene materials), loaded as geomIDs after the model's meshes
    (InitializeCurves, ModelResource.cpp:300-332).
"""
from __future__ import annotations

import copy
import dataclasses
import struct

import numpy as np

from selas_gb300 import scenes

# Material property order of MaterialResourceData::scalarAttributeValues (ModelResource.h:45-66).
SCALARS = ("metallic", "specularTint", "roughness", "anisotropic", "sheen", "sheenTint", "clearcoat", "clearcoatGloss",
           "specTrans", "diffuseTrans", "flatness", "ior", "scatterDistance", "displacement")
E_TRANSPARENT, E_USES_PTEX = 1, 16
SHADERS = {"DisneyThin": 0, "DisneySolid": 1, "DiracTransparent": 2}


def murmur3_32(data: bytes, seed: int = 0) -> int:
    """MurmurHash3_x86_32 (Austin Appleby's published algorithm), the hash the reference names assets and
    materials with (UtilityLib/MurmurHash.h)."""
    c1, c2, m = 0xCC9E2D51, 0x1B873593, 0xFFFFFFFF
    h = seed & m
    n = len(data) // 4
    for (k,) in struct.iter_unpack("<I", data[:4 * n]):
        k = (k * c1) & m
        k = ((k << 15) | (k >> 17)) & m
        h ^= (k * c2) & m
        h = ((h << 13) | (h >> 19)) & m
        h = (h * 5 + 0xE6546B64) & m
    tail = data[4 * n:]
    k = 0
    for i in reversed(range(len(tail))):
        k = (k << 8) | tail[i]
    if tail:
        k = (k * c1) & m
        k = ((k << 15) | (k >> 17)) & m
        h ^= (k * c2) & m
    h ^= len(data)
    h ^= h >> 16
    h = (h * 0x85EBCA6B) & m
    h ^= h >> 13
    h = (h * 0xC2B2AE35) & m
    return h ^ (h >> 16)


def name_hash(name: str) -> int:
    return murmur3_32(name.encode())


def material(shader="DisneySolid", base=(0.6, 0.6, 0.6), transmittance=(0.0, 0.0, 0.0), texture="", ptex=False,
             **scalars):
    """A MaterialResourceData as the reference's build step writes it: the importer's defaults for absent scalars
    (ImportMaterial.cpp:36-52) and eTransparent derived as BuildModel.cpp:60-65 derives it."""
    values = dict(metallic=0.3, roughness=0.5, ior=1.5)
    values.update(scalars)
    sc = [float(values.get(k, 0.0)) for k in SCALARS]
    flags = E_USES_PTEX if ptex else 0
    if shader == "DisneySolid" and (values.get("diffuseTrans", 0.0) > 0 or values.get("specTrans", 0.0) > 0):
        flags |= E_TRANSPARENT
    return dict(shader=SHADERS[shader], flags=flags, baseColor=tuple(map(float, base)),
                transmittanceColor=tuple(map(float, transmittance)), scalars=sc, texture=texture)


def default_material():
    """CreateDefaultMaterial (ModelResource.cpp:203-211): grey 0.6, DisneySolid, ior 1.5, every other scalar 0."""
    sc = [0.0] * len(SCALARS)
    sc[SCALARS.index("ior")] = 1.5
    return dict(shader=1, flags=0, baseColor=(0.6, 0.6, 0.6), transmittanceColor=(0.0, 0.0, 0.0), scalars=sc,
                texture="")


def l2w_words(m) -> list:
    """The 16 floats of a float4x4 localToWorld in memory (rows of the reference's row-vector matrix, translation
    in the last row) for a column-vector maths matrix m (4 x 4)."""
    return [float(x) for x in np.asarray(m, np.float32).T.reshape(16)]


def _affine(scale=(1, 1, 1), angle_deg=0.0, translate=(0, 0, 0)):
    a = np.deg2rad(angle_deg)
    rot = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
    m = np.eye(4)
    m[:3, :3] = rot @ np.diag(scale)
    m[:3, 3] = translate
    return m.astype(np.float32)


def _wall_model():
    """Five walls of a half-size Cornell room (side 278), one mesh each, sharing one vertex array; normals from
    the winding, tangents along the first edge (bitangent sign 1), uvs 0..2.5 across each wall."""
    s = 278.0
    quads = [("floor", [0, 0, 0], [0, 0, s], [s, 0, s], [s, 0, 0]),
             ("ceiling", [0, s, 0], [s, s, 0], [s, s, s], [0, s, s]),
             ("back", [0, 0, s], [0, s, s], [s, s, s], [s, 0, s]),
             ("left", [s, 0, 0], [s, 0, s], [s, s, s], [s, s, 0]),
             ("right", [0, 0, 0], [0, s, 0], [0, s, s], [0, 0, s])]
    mats = {"floor": "floor", "ceiling": "white", "back": "unnamed_paint", "left": "red", "right": "green"}
    pos, nrm, tan, uvs, idx, meshes = [], [], [], [], [], []
    for name, *corners in quads:
        v = np.array(corners, np.float32)
        n = np.cross(v[1] - v[0], v[2] - v[0])
        n /= np.linalg.norm(n)
        t = (v[1] - v[0]) / np.linalg.norm(v[1] - v[0])
        base = len(pos) * 4
        meshes.append(dict(name=name, material=mats[name], indicesPerFace=3, indexOffset=len(idx) * 6,
                           indexCount=6, vertexOffset=base, vertexCount=4))
        pos.append(v)
        nrm.append(np.tile(n, (4, 1)))
        tan.append(np.tile(np.append(t, 1.0), (4, 1)))
        uvs.append(np.array([[0, 0], [0, 2.5], [2.5, 2.5], [2.5, 0]], np.float32))
        idx.append(np.array([0, 1, 2, 0, 2, 3], np.uint32) + base)
    materials = {"floor": material(base=(0.73, 0.73, 0.73), texture="checker", roughness=0.5, metallic=0.0),
                 "white": material(base=(0.73, 0.73, 0.73), roughness=0.5, metallic=0.0),
                 "red": material(base=(0.65, 0.05, 0.05), roughness=0.5, metallic=0.0)}
    return dict(positions=np.concatenate(pos), normals=np.concatenate(nrm).astype(np.float32),
                tangents=np.concatenate(tan).astype(np.float32), uvs=np.concatenate(uvs), indices=np.concatenate(idx),
                meshes=meshes, materials=materials)


def _box_model():
    """A unit box ([-0.5, 0.5] x [0, 1] x [-0.5, 0.5]) as one quad mesh of six outward-facing quads, no
    attributes; its material comes from the subscene that instances it."""
    faces = []
    for axis in range(3):
        for sign in (1.0, -1.0):
            n = np.zeros(3)
            n[axis] = sign
            a = np.zeros(3)
            a[(axis + 1) % 3] = 0.5
            b = np.cross(n, a)
            c = np.array([0.0, 0.5, 0.0]) + 0.5 * n
            faces.append([c - a - b, c + a - b, c + a + b, c - a + b])
    pos = np.array(faces, np.float32).reshape(-1, 3)
    quads = np.arange(24, dtype=np.uint32)
    return dict(positions=pos, normals=None, tangents=None, uvs=None, indices=quads,
                meshes=[dict(name="box", material="box_paint", indicesPerFace=4, indexOffset=0, indexCount=24,
                             vertexOffset=0, vertexCount=24)],
                materials={})


def _strands_model():
    """A plate (one triangle mesh of two triangles) and hair strands as two curves over one curve vertex array:
    the first three strands' segments, then the rest (indices into the shared array, as the build writes them)."""
    pts, idx = scenes.curve_strands(strands=8, seed=0x5E1A5C07)
    per = idx.size // 8
    plate = np.float32([[-2, 0, -1.5], [2, 0, -1.5], [2, 0, 1.5], [-2, 0, 1.5]])
    return dict(positions=plate, normals=None, tangents=None, uvs=None, indices=np.uint32([0, 2, 1, 0, 3, 2]),
                meshes=[dict(name="plate", material="plate", indicesPerFace=3, indexOffset=0, indexCount=6,
                             vertexOffset=0, vertexCount=4)],
                materials={"plate": material(base=(0.2, 0.2, 0.25), roughness=0.8, metallic=0.0)},
                curves=[(0, 3 * per), (3 * per, idx.size - 3 * per)], curve_indices=idx, curve_vertices=pts,
                curve_material="hair")


def curve_geometry(model):
    """The model's curves as the loader attaches them: [(geomID, control points, segment first points)], each
    curve's points cut to the range its segments use."""
    out = []
    for c, (off, count) in enumerate(model.get("curves", [])):
        idx = model["curve_indices"][off:off + count]
        lo, hi = int(idx.min()), int(idx.max()) + 4
        out.append((len(model["meshes"]) + c, model["curve_vertices"][lo:hi], (idx - lo).astype(np.uint32)))
    return out


def _checker_texture():
    n = 8
    y, x = np.mgrid[0:n, 0:n]
    a, b = np.array([0.9, 0.8, 0.1]), np.array([0.1, 0.2, 0.9])
    mip0 = np.where(((x + y) % 2 == 0)[..., None], a, b).astype(np.float32)
    mip0[0, 0] = [1.0, 0.0, 0.0]
    mip1 = mip0.reshape(4, 2, 4, 2, 3).mean(axis=(1, 3)).astype(np.float32)
    return dict(format=2, mips=[mip0, mip1])


def cooked_cornell():
    """The asset set of the three scenes (dict of scenes, subscenes, models, textures, ibls by asset name)."""
    green = material(base=(0.12, 0.45, 0.15), roughness=0.5, metallic=0.0)
    red_shadowed = material(base=(0.1, 0.1, 0.8), roughness=0.5, metallic=0.0)
    box_paint = material(base=(0.8, 0.78, 0.7), roughness=0.3, metallic=0.5, clearcoat=0.5, clearcoatGloss=0.8)
    subscenes = {
        "room": dict(light_set=0, models=["walls"], instances=[(0, np.eye(4, dtype=np.float32))],
                     materials=[("green", green), ("red", red_shadowed)]),
        "props": dict(light_set=0, models=["box"],
                      instances=[(0, _affine((165, 165, 165), -18.0, (185.0, 0.0, 169.0))),
                                 (0, _affine((165, 330, 165), 18.0, (368.0, 0.0, 351.0)))],
                      materials=[("box_paint", box_paint)]),
        "room_ptex": dict(light_set=0, models=["walls"], instances=[(0, np.eye(4, dtype=np.float32))],
                          materials=[("green", material(base=(0.12, 0.45, 0.15), texture="ptex/walls", ptex=True))]),
        "hairy": dict(light_set=0, models=["strands"],
                      instances=[(0, _affine((70, 70, 70), 25.0, (170.0, 0.5, 110.0)))],
                      materials=[("hair", material(base=(0.45, 0.3, 0.15), roughness=0.35, metallic=0.1))]),
    }
    light = dict(type=0, position=(278.0, 554.0, 279.5), direction=(0.0, -1.0, 0.0), x=(130.0, 0.0, 0.0),
                 z=(0.0, 0.0, 105.0), radiance=(17.0, 12.0, 4.0))
    camera = dict(position=(278.0, 273.0, -800.0), look_at=(278.0, 273.0, 0.0), up=(0.0, 1.0, 0.0), fov_degrees=39.3,
                  znear=0.1, zfar=10000.0)
    base_scene = dict(ibl="", background=(0.05, 0.05, 0.05, 1.0), subscenes=["room", "props"],
                      instances=[(0, _affine((2, 2, 2))), (1, _affine(translate=(6.0, 0.0, -4.0)))],
                      lights=[light], ranges=[(0, 1)], cameras=[camera])
    scenes_ = {"cornell": base_scene,
               "cornell_sky": dict(copy.deepcopy(base_scene), ibl="sky", background=(0.0, 0.0, 0.0, 1.0)),
               "cornell_ptex": dict(copy.deepcopy(base_scene), subscenes=["room_ptex", "props"]),
               "cornell_hair": dict(copy.deepcopy(base_scene), subscenes=["room", "props", "hairy"],
                                    instances=base_scene["instances"] + [(2, _affine())])}
    sky = scenes.sky_ibl(width=32, height=16, miss_size=(16, 8))
    return dict(scenes=scenes_, subscenes=subscenes,
                models={"walls": _wall_model(), "box": _box_model(), "strands": _strands_model()},
                textures={"checker": _checker_texture()},
                ibls={"sky": dict(light=sky["light"], miss=sky["miss"], rotation=float(sky.get("rotation", 0.0)),
                                  exposure=float(sky.get("exposure", 1.0)))})


def find_mesh_material(model, subscene, material_name):
    """FindMeshMaterial (ModelResource.cpp:213-229): the model's materials by binary search of their sorted
    hashes, then the subscene's scene materials in order, else the default material."""
    h = name_hash(material_name)
    own = {name_hash(k): v for k, v in model["materials"].items()}
    if h in own:
        return own[h]
    for name, m in subscene["materials"]:
        if name_hash(name) == h:
            return m
    return default_material()


def mesh_table(assets, scene_name):
    """(subscene slot, model slot, mesh index, resolved material, indicesPerFace, faces) for every mesh the scene's
    subscenes load, in load order (subscene names, then their model names, then meshes)."""
    rows = []
    for si, sname in enumerate(assets["scenes"][scene_name]["subscenes"]):
        sub = assets["subscenes"][sname]
        for mi, mname in enumerate(sub["models"]):
            model = assets["models"][mname]
            for k, mesh in enumerate(model["meshes"]):
                rows.append((si, mi, k, find_mesh_material(model, sub, mesh["material"]), mesh["indicesPerFace"],
                             mesh["indexCount"] // mesh["indicesPerFace"]))
    return rows


def _sel_material(m, light_set):
    sc = dict(zip(SCALARS, m["scalars"]))
    sc.pop("displacement")
    return dict(shader=m["shader"], lightSetIndex=light_set, baseColor=m["baseColor"],
                transmittanceColor=m["transmittanceColor"], usesPtex=0, **sc)


def instanced_scene(assets, scene_name):
    """The scene as an InstancedRenderScene (parts: the world, then per subscene its part and one part per model
    it loads, as the reference loads a model once per subscene), for the oracle and the directly built GPU scene."""
    sd = assets["scenes"][scene_name]
    cam = sd["cameras"][0]
    camera = dict(position=cam["position"], look_at=cam["look_at"], up=cam["up"], fov_degrees=cam["fov_degrees"])
    lights = []
    for set_index, (start, count) in enumerate(sd["ranges"]):
        for l in sd["lights"][start:start + count]:
            lights.append((set_index, {k: l[k] for k in ("position", "direction", "x", "z", "radiance")}))
    ibl = None
    if sd["ibl"]:
        b = assets["ibls"][sd["ibl"]]
        ibl = dict(light=b["light"], miss=b["miss"], rotation=b["rotation"], exposure=b["exposure"])
    world = scenes.RenderScene(scenes.TriangleScene(), {}, lights, tuple(sd["background"][:3]), camera, ibl=ibl)
    parts, instances = [world], [[]]
    sub_part = {}
    for si, sname in enumerate(sd["subscenes"]):
        sub = assets["subscenes"][sname]
        sub_part[si] = len(parts)
        parts.append(scenes.RenderScene(scenes.TriangleScene(), {}, [], (0.0, 0.0, 0.0), {}))
        instances.append([])
        model_part = []
        for mname in sub["models"]:
            model = assets["models"][mname]
            g = scenes.TriangleScene()
            mats, attrs, textures = {}, {}, {}
            for k, mesh in enumerate(model["meshes"]):
                ipf = mesh["indicesPerFace"]
                idx = model["indices"][mesh["indexOffset"]:mesh["indexOffset"] + mesh["indexCount"]]
                lo, hi = int(idx.min()), int(idx.max()) + 1
                v = model["positions"][lo:hi]
                local = (idx - lo).astype(np.uint32)
                if ipf == 4:
                    g.add_quads(k, v, local.reshape(-1, 4))
                else:
                    g.add(k, v, local.reshape(-1, 3))
                m = find_mesh_material(model, sub, mesh["material"])
                mats[k] = _sel_material(m, sub["light_set"])
                a = {}
                for key in ("normals", "tangents", "uvs"):
                    if model[key] is not None:
                        a[key] = model[key][lo:hi]
                if a:
                    attrs[k] = a
                if m["texture"] and not m["flags"] & E_USES_PTEX:
                    textures[k] = assets["textures"][m["texture"]]["mips"][0]
            curves = {}
            for gid, pts, idx in curve_geometry(model):
                curves[gid] = (pts, idx)
                mats[gid] = _sel_material(find_mesh_material(model, sub, model["curve_material"]), sub["light_set"])
            model_part.append(len(parts))
            parts.append(scenes.RenderScene(g, mats, [], (0.0, 0.0, 0.0), {}, attrs=attrs or None,
                                            textures=textures or None, curves=curves or None))
            instances.append([])
        for j, (index, m) in enumerate(sub["instances"]):
            instances[sub_part[si]].append((j, model_part[index], np.asarray(m, np.float32)))
    for i, (index, m) in enumerate(sd["instances"]):
        instances[0].append((i, sub_part[index], np.asarray(m, np.float32)))
    return scenes.InstancedRenderScene(parts, instances)

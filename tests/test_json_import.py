"""Import of the reference's JSON asset descriptions, host code only (no device): ImportMaterial
(BuildCommon/ImportMaterial.cpp:56-88) and ImportDisneyMaterials (ImportMaterial.cpp:91-146), each followed by
BuildMaterial (BuildCommon/BuildModel.cpp:22-64), and ParseSceneFile (BuildCommon/CSceneBuildProcessor.cpp:32-63).
The documents below are written for these tests in the files' format: one material per file with "shaderName",
"baseColor" and the scalar attributes; the Disney-island materials file of named materials with "type",
"colorMap" and "assignment"; a scene file with model and subscene instances, background and image-based light."""
import json

import numpy as np
import pytest

import selas_gb300 as sel


def test_single_material_fields():
    doc = {"shaderName": "DisneySolid", "baseColor": [0.25, 0.5, 0.75], "transmittanceColor": [0.1, 0.2, 0.3],
           "ior": 1.33, "metallic": 0.8, "specularTint": 0.2, "roughness": 0.05, "anisotropic": 0.1, "sheen": 0.3,
           "sheenTint": 0.4, "clearcoat": 0.5, "clearcoatGloss": 0.6, "specTrans": 0.0, "diffTrans": 0.0,
           "flatness": 0.7, "scatterDistance": 2.5, "usesPtex": True}
    m, tex = sel.material_from_json(json.dumps(doc))
    assert m.shader == sel.SEL_SHADER_DISNEY_SOLID and tex == ""
    np.testing.assert_array_equal(list(m.baseColor), np.float32([0.25, 0.5, 0.75]))
    np.testing.assert_array_equal(list(m.transmittanceColor), np.float32([0.1, 0.2, 0.3]))
    for field, key in (("ior", "ior"), ("metallic", "metallic"), ("specularTint", "specularTint"),
                       ("roughness", "roughness"), ("anisotropic", "anisotropic"), ("sheen", "sheen"),
                       ("sheenTint", "sheenTint"), ("clearcoat", "clearcoat"), ("clearcoatGloss", "clearcoatGloss"),
                       ("flatness", "flatness"), ("scatterDistance", "scatterDistance")):
        assert getattr(m, field) == np.float32(doc[key]), field
    assert m.usesPtex == 1


def test_importer_defaults_and_shader_names():
    m, tex = sel.material_from_json("{}")
    assert m.shader == sel.SEL_SHADER_DISNEY_SOLID and tex == ""
    np.testing.assert_array_equal(list(m.baseColor), np.float32([0.6, 0.6, 0.6]))
    np.testing.assert_array_equal(list(m.transmittanceColor), [0.0, 0.0, 0.0])
    assert (m.metallic, m.roughness, m.ior) == (np.float32(0.3), np.float32(0.5), np.float32(1.5))
    assert (m.specTrans, m.diffuseTrans, m.sheen, m.clearcoat, m.usesPtex) == (0.0, 0.0, 0.0, 0.0, 0)
    for name, shader in (("disneythin", sel.SEL_SHADER_DISNEY_THIN), ("DISNEYSOLID", sel.SEL_SHADER_DISNEY_SOLID),
                         ("DeltaTransparent", sel.SEL_SHADER_DIRAC_TRANSPARENT), ("Unknown", sel.SEL_SHADER_DISNEY_SOLID)):
        assert sel.material_from_json(json.dumps({"shaderName": name}))[0].shader == shader, name
    # integers are read as floats, wrong types and short arrays fall back to the defaults
    m, _ = sel.material_from_json('{"metallic": 1, "roughness": "rough.png", "baseColor": [0.2, 0.3], "ior": true}')
    assert m.metallic == 1.0 and m.roughness == np.float32(0.5) and m.ior == np.float32(1.5)
    np.testing.assert_array_equal(list(m.baseColor), np.float32([0.6, 0.6, 0.6]))
    # a fourth component is ignored, as the reference reads the first three
    m, _ = sel.material_from_json('{"baseColor": [0.1, 0.2, 0.3, 0.4]}')
    np.testing.assert_array_equal(list(m.baseColor), np.float32([0.1, 0.2, 0.3]))


def test_texture_named_base_colour():
    m, tex = sel.material_from_json('{"baseColor": "Textures/paper_col.png", "usesPtex": false}')
    assert tex == "Textures/paper_col.png"
    np.testing.assert_array_equal(list(m.baseColor), np.float32([0.6, 0.6, 0.6]))
    # escapes and non-ASCII names survive
    m, tex = sel.material_from_json(r'{"baseColor": "dir\\subé\/a.ptx"}')
    assert tex == "dir\\subé/a.ptx"


def test_transmission_fields_for_the_build_rule():
    """BuildMaterial marks DisneySolid materials with diffTrans or specTrans above 0 transparent; the scene upload
    applies that rule to the SelMaterial, so the importer hands over the shader and both transmission weights."""
    glass, _ = sel.material_from_json('{"shaderName": "DisneySolid", "specTrans": 1.0, "ior": 1.5}')
    assert glass.specTrans == 1.0 and glass.shader == sel.SEL_SHADER_DISNEY_SOLID
    thin, _ = sel.material_from_json('{"shaderName": "DisneyThin", "diffTrans": 0.5}')
    assert thin.diffuseTrans == 0.5 and thin.shader == sel.SEL_SHADER_DISNEY_THIN


@pytest.mark.parametrize("bad", ['', '{', '{"a": }', '{"a": 1,}', '[1, 2]', '{"a": tru}', '{"a": "x\\q"}',
                                 '{"a": 1} x', '{"a": 01.}', '"text"'])
def test_malformed_documents_are_errors(bad):
    with pytest.raises(sel.SelError):
        sel.material_from_json(bad)


def test_disney_materials_file():
    doc = {
        "bark": {"baseColor": [0.3, 0.2, 0.1], "roughness": 0.9, "type": "solid",
                 "colorMap": "textures\\bark\\Color", "assignment": ["trunk", "branches"]},
        "leaf": {"type": "thin", "diffTrans": 0.6, "assignment": []},
        "water": {"specTrans": 1.0, "ior": 1.33, "type": "solid"},
    }
    entries = sel.disney_materials_from_json(json.dumps(doc))
    assert [e[0] for e in entries] == ["bark", "trunk", "branches", "leaf", "water"]
    bark = entries[0][1]
    assert bark.shader == sel.SEL_SHADER_DISNEY_SOLID and bark.usesPtex == 1
    assert entries[0][2] == "textures/bark/Color" and entries[1][2] == entries[0][2]
    np.testing.assert_array_equal(list(bark.baseColor), np.float32([0.3, 0.2, 0.1]))
    np.testing.assert_array_equal(list(bark.transmittanceColor), [1.0, 1.0, 1.0])
    assert bark.roughness == np.float32(0.9) and bark.metallic == np.float32(0.3)
    for alias in entries[1:3]:
        assert bytes(alias[1]) == bytes(bark)
    leaf = entries[3][1]
    assert leaf.shader == sel.SEL_SHADER_DISNEY_THIN and leaf.usesPtex == 0 and entries[3][2] == ""
    np.testing.assert_array_equal(list(leaf.baseColor), [1.0, 1.0, 1.0])
    water = entries[4][1]
    assert water.ior == np.float32(1.33) and water.specTrans == 1.0


def test_disney_materials_count_and_errors():
    text = json.dumps({f"m{k}": {"assignment": [f"a{k}"]} for k in range(40)})
    n = ctypes_count(text)
    assert n == 80
    assert len(sel.disney_materials_from_json(text)) == 80
    for bad in ('{"m": 3}', '{"m": {"assignment": "x"}}', '{"m": {"assignment": [1]}}', '{"m": {"colorMap": 2}}'):
        with pytest.raises(sel.SelError):
            sel.disney_materials_from_json(bad)


def ctypes_count(text):
    import ctypes
    n = ctypes.c_uint(0)
    sel.check(sel.lib().sel_disney_materials_from_json(text.encode(), None, 0, ctypes.byref(n)))
    return n.value


def test_scene_description():
    # the reference's row-vector matrices: a rotation of 90 degrees about y, then a translation in the last row
    rot_t = [0, 0, -1, 0,  0, 1, 0, 0,  1, 0, 0, 0,  5, 6, 7, 1]
    doc = {"instances": [{"model": "Meshes/rock.fbx", "transform": rot_t},
                         {"model": "Meshes/tree.fbx"},
                         {"model": "Meshes/rock.fbx", "transform": [1, 2, 3]}],
           "scenes": [{"scene": "Scenes/island.json", "transform": [2, 0, 0, 0, 0, 2, 0, 0, 0, 0, 2, 0, 0, 0, 0, 1]}],
           "backgroundIntensity": [0.5, 0.25, 0.125], "ibl": "HDR/sky.hdr"}
    d = sel.scene_description_from_json(json.dumps(doc))
    assert [m[0] for m in d["models"]] == ["Meshes/rock.fbx", "Meshes/tree.fbx", "Meshes/rock.fbx"]
    a = d["models"][0][1]
    # as a column-vector matrix: the translation in the last column, and p' = A p maps x to -z as p M does
    np.testing.assert_array_equal(a[:3, 3], [5, 6, 7])
    np.testing.assert_array_equal(a @ np.float32([1, 0, 0, 1]), np.float32([1, 0, 0, 1]) @ np.float32(rot_t).reshape(4, 4))
    np.testing.assert_array_equal(d["models"][1][1], np.eye(4))  # no transform: identity
    np.testing.assert_array_equal(d["models"][2][1], np.eye(4))  # not 16 numbers: identity
    assert d["scenes"][0][0] == "Scenes/island.json" and d["scenes"][0][1][0, 0] == 2.0
    assert d["background"] == (0.5, 0.25, 0.125) and d["ibl"] == "HDR/sky.hdr"
    empty = sel.scene_description_from_json("{}")
    assert empty["models"] == [] and empty["scenes"] == [] and empty["background"] == (1.0, 1.0, 1.0)
    assert empty["ibl"] == ""
    for bad in ('{"instances": {}}', '{"scenes": [1]}', '{"instances": [', '[]'):
        with pytest.raises(sel.SelError):
            sel.scene_description_from_json(bad)


CUBE_OBJ = """# a cube, quads with normals, two material groups, relative indices on the last faces
v -1 -1 -1
v 1 -1 -1
v 1 1 -1
v -1 1 -1
v -1 -1 1
v 1 -1 1
v 1 1 1
v -1 1 1
vn 0 0 -1
vn 0 0 1
vn -1 0 0
vn 1 0 0
vn 0 -1 0
vn 0 1 0
usemtl Red
f 1//1 4//1 3//1 2//1
f 5//2 6//2 7//2 8//2
f 1//3 5//3 8//3 4//3
f 2//4 3//4 7//4 6//4
usemtl Gold
f 1//5 2//5 6//5 5//5
f -5//6 -1//6 -2//6 -6//6
"""

FLOOR_OBJ = """v -20 0 -20
v 20 0 -20
v 20 0 20
v -20 0 20
vt 0 0
usemtl Floor
f 1/1 4/1 3/1
f 1/1 3/1 2/1
"""


def test_load_obj_groups_fans_and_indices():
    from selas_gb300 import scenes
    groups = scenes.load_obj(CUBE_OBJ)
    assert [g[0] for g in groups] == ["Red", "Gold"]
    red, gold = groups[0], groups[1]
    assert red[2].shape == (8, 3) and gold[2].shape == (4, 3)  # quads fanned into two triangles each
    assert red[1].shape == (16, 3) and red[3].shape == (16, 3)  # distinct (position, normal) corners
    # the relative indices of the last face name the top (y = 1) corners with the +y normal
    top = gold[1][gold[2][2:].reshape(-1)]
    assert np.all(top[:, 1] == 1.0) and np.all(gold[3][gold[2][2:].reshape(-1)] == [0, 1, 0])
    floor = scenes.load_obj(FLOOR_OBJ)
    assert floor[0][0] == "Floor" and floor[0][3] is None and floor[0][2].shape == (2, 3)
    floor_uv = scenes.load_obj(FLOOR_OBJ.replace("vt 0 0", "vt 0 0\nvt 1 0.5"), with_uvs=True)
    assert floor_uv[0][4].shape == (4, 2) and np.all(floor_uv[0][4] == 0.0)
    assert scenes.load_obj(CUBE_OBJ, with_uvs=True)[0][4] is None  # v//vn corners carry no uvs
    with pytest.raises(ValueError):
        scenes.load_obj("v 0 0 0\nf 1 2 3\n")


def _write_scene(tmp_path):
    (tmp_path / "cube.obj").write_text(CUBE_OBJ)
    (tmp_path / "floor.obj").write_text(FLOOR_OBJ)
    (tmp_path / "Red.json").write_text(json.dumps({"shaderName": "DisneySolid", "baseColor": [0.8, 0.1, 0.1],
                                                   "roughness": 0.6, "metallic": 0.0}))
    (tmp_path / "Gold.json").write_text(json.dumps({"shaderName": "DisneySolid", "baseColor": [0.9, 0.7, 0.3],
                                                    "roughness": 0.3, "metallic": 1.0, "usesPtex": True}))
    c, s = np.cos(0.6), np.sin(0.6)
    rot = [c, 0, -s, 0, 0, 1, 0, 0, s, 0, c, 0, 0, 0, 0, 1]  # row-vector matrices, translation in the last row
    doc = {"instances": [{"model": "floor.obj"},
                         {"model": "cube.obj", "transform": rot[:12] + [-3, 1, 0, 1]},
                         {"model": "cube.obj", "transform": [0.5, 0, 0, 0, 0, 0.5, 0, 0, 0, 0, 0.5, 0, 2, 0.5, 1, 1]}],
           "backgroundIntensity": [0.2, 0.3, 0.4]}
    (tmp_path / "scene.json").write_text(json.dumps(doc))
    light = dict(position=(0.0, 8.0, 0.0), direction=(0.0, -1.0, 0.0), x=(4.0, 0.0, 0.0), z=(0.0, 0.0, 4.0),
                 radiance=(20.0, 20.0, 18.0))
    return tmp_path / "scene.json", [(0, light)]


def test_load_scene_file(tmp_path):
    from selas_gb300 import scenes
    path, lights = _write_scene(tmp_path)
    s = scenes.load_scene_file(path, lights=lights)
    assert len(s.parts) == 3  # world, floor, cube (shared by both of its instances)
    world = s.instances[0]
    assert [(i, p) for i, p, _ in world] == [(1, 1), (2, 2), (3, 2)]
    np.testing.assert_allclose(world[1][2][:3, 3], [-3, 1, 0])
    np.testing.assert_allclose(world[2][2][:3, :3], 0.5 * np.eye(3))
    cube = s.parts[2]
    assert [m[0] for m in cube.geometry.meshes] == [0, 1] and set(cube.attrs) == {0, 1}
    assert cube.materials[0]["metallic"] == 0.0 and cube.materials[1]["metallic"] == 1.0
    assert cube.materials[1]["usesPtex"] == 0  # no texels come with an OBJ
    assert s.parts[1].materials == {}  # Floor.json does not exist: the default material
    assert s.parts[0].background == pytest.approx((0.2, 0.3, 0.4)) and s.parts[0].lights == lights
    assert s.parts[1].attrs[0]["uvs"].shape == (4, 2) and s.parts[1].textures is None
    assert set(s.camera) == {"position", "look_at", "up", "fov_degrees"}


@pytest.mark.gpu
def test_gpu_scene_file_renders_the_oracles_image(device, tmp_path):
    """A scene file with OBJ models and JSON materials, built through the instancing API: the GPU traces the
    oracle's paths on the same streams."""
    import selas_gb300 as sel
    import oracle
    from selas_gb300 import scenes
    path, lights = _write_scene(tmp_path)
    s = scenes.load_scene_file(path, lights=lights)
    built = s.build(sel, device)
    gpu = built[0].pt_generate_image(s.sel_camera(sel, 48, 36), sel.pt_settings(8, 6, 0x5E1A5000)).astype(np.float64)
    s.release(built)
    cpu = oracle.graph_render(s, 48, 36, 0, 8, seed=0x5E1A5000, max_bounces=6) / 8.0
    for layer in (0, 1):
        g, c = gpu[layer], cpu[layer]
        rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-3 * c.mean())
        assert np.median(rel) < 1e-4, np.median(rel)
        assert (rel < 1e-2).mean() > 0.97
    assert gpu[1].mean() > 0


def _rgbe(img):
    """float (h, w, 3) -> RGBE bytes (h, w, 4), the format's shared-exponent encoding."""
    m = img.max(axis=-1)
    e = np.where(m > 1e-32, np.floor(np.log2(np.maximum(m, 1e-32))) + 1, 0).astype(np.int32)
    scale = np.where(m > 1e-32, np.ldexp(1.0, 8 - e), 0.0)
    out = np.zeros(img.shape[:2] + (4,), np.uint8)
    out[..., :3] = np.clip(np.floor(img * scale[..., None]), 0, 255).astype(np.uint8)
    out[..., 3] = np.where(m > 1e-32, e + 128, 0).astype(np.uint8)
    return out


def _hdr_bytes(img, rle):
    h, w = img.shape[:2]
    rgbe = _rgbe(img)
    out = bytearray(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {h} +X {w}\n".encode())
    for y in range(h):
        if not rle:
            out += rgbe[y].tobytes()
            continue
        out += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            row, x = rgbe[y, :, c], 0
            while x < w:
                run = 1
                while x + run < w and run < 127 and row[x + run] == row[x]:
                    run += 1
                if run >= 3:
                    out += bytes([128 + run, row[x]])
                    x += run
                else:
                    n = min(w - x, 128)
                    out += bytes([n]) + row[x:x + n].tobytes()
                    x += n
    return bytes(out)


@pytest.mark.parametrize("rle", [False, True])
def test_read_hdr(rle):
    from selas_gb300 import scenes
    rng = np.random.default_rng(3)
    img = rng.uniform(0.0, 4.0, (5, 24, 3)).astype(np.float32)
    img[1, 3:12] = [0.5, 0.25, 2.0]  # runs
    img[2, 0] = 0.0
    got = scenes.read_hdr(_hdr_bytes(img, rle))
    want = _rgbe(img)
    e = want[..., 3].astype(np.int32)
    ref = want[..., :3] * np.where(e > 0, np.ldexp(1.0, e - 136), 0.0)[..., None]
    np.testing.assert_array_equal(got, ref.astype(np.float32))
    # the shared exponent keeps each component to 8 bits of the pixel's largest one
    assert np.all(np.abs(got - img) <= img.max(axis=-1, keepdims=True) * 2 ** -7 + 1e-6)
    with pytest.raises(ValueError):
        scenes.read_hdr(b"P6\n")


def test_scene_file_with_dual_ibl(tmp_path):
    from selas_gb300 import scenes
    path, lights = _write_scene(tmp_path)
    sky = np.full((8, 16, 3), 0.5, np.float32)
    sky[:4] = [1.0, 1.5, 2.0]
    (tmp_path / "sky.hdr").write_bytes(_hdr_bytes(sky, True))
    (tmp_path / "miss.hdr").write_bytes(_hdr_bytes(sky[::2, ::2].copy(), False))
    (tmp_path / "sky.json").write_text(json.dumps({"light": "sky.hdr", "miss": "miss.hdr", "rotationDegrees": 90,
                                                   "exposure": 1.5}))
    doc = json.loads(path.read_text())
    doc["ibl"] = "sky.json"
    path.write_text(json.dumps(doc))
    ibl = scenes.load_scene_file(path, lights=lights).parts[0].ibl
    assert np.all(np.abs(ibl["light"] - sky) <= sky.max(axis=-1, keepdims=True) * 2 ** -7)
    assert ibl["miss"].shape == (4, 8, 3)
    assert ibl["rotation"] == pytest.approx(np.pi / 2) and ibl["exposure"] == pytest.approx(2 ** 1.5)
    single = scenes.load_ibl(tmp_path / "sky.hdr")
    assert single["miss"] is None and single["rotation"] == 0.0 and single["exposure"] == 1.0


def test_scene_file_with_textured_material(tmp_path):
    from selas_gb300 import scenes
    path, lights = _write_scene(tmp_path)
    img = np.linspace(0.0, 1.0, 8 * 16 * 3, dtype=np.float32).reshape(8, 16, 3)
    (tmp_path / "floor.hdr").write_bytes(_hdr_bytes(img, True))
    (tmp_path / "Floor.json").write_text(json.dumps({"baseColor": "floor.hdr", "roughness": 0.8}))
    s = scenes.load_scene_file(path, lights=lights)
    floor = s.parts[1]
    assert floor.materials[0]["roughness"] == np.float32(0.8) and floor.textures[0].shape == (8, 16, 3)
    assert floor.attrs[0]["uvs"].shape == (4, 2)


@pytest.mark.gpu
def test_gpu_textured_scene_file_renders_the_oracles_image(device, tmp_path):
    """The floor's material file names a .hdr base-colour image sampled at the OBJ's texture coordinates."""
    import selas_gb300 as sel
    import oracle
    from selas_gb300 import scenes
    path, lights = _write_scene(tmp_path)
    (tmp_path / "floor.obj").write_text(FLOOR_OBJ.replace("vt 0 0", "vt 0 0\nvt 3 0\nvt 3 3\nvt 0 3")
                                        .replace("f 1/1 4/1 3/1\nf 1/1 3/1 2/1", "f 1/1 4/4 3/3\nf 1/1 3/3 2/2"))
    y, x = np.mgrid[0:8, 0:8]
    img = np.where(((x + y) % 2 == 0)[..., None], [0.9, 0.85, 0.3], [0.15, 0.3, 0.8]).astype(np.float32)
    (tmp_path / "floor.hdr").write_bytes(_hdr_bytes(img, True))
    (tmp_path / "Floor.json").write_text(json.dumps({"baseColor": "floor.hdr", "roughness": 0.7}))
    s = scenes.load_scene_file(path, lights=lights)
    assert s.parts[1].textures is not None
    built = s.build(sel, device)
    gpu = built[0].pt_generate_image(s.sel_camera(sel, 48, 36), sel.pt_settings(8, 6, 0x5E1A5000)).astype(np.float64)
    s.release(built)
    cpu = oracle.graph_render(s, 48, 36, 0, 8, seed=0x5E1A5000, max_bounces=6) / 8.0
    for layer in (0, 1):
        g, c = gpu[layer], cpu[layer]
        rel = np.abs(g - c) / np.maximum(np.abs(c), 1e-3 * c.mean())
        assert np.median(rel) < 1e-4, np.median(rel)
        assert (rel < 1e-2).mean() > 0.97

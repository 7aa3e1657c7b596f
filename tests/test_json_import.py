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

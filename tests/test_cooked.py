"""Cooked asset loading (sel_cooked_scene_describe, sel_scene_load_cooked) against the blobs the reference's own
serializer wrote (tests/golden/cooked/, tests/golden/make_cooked.py) from the descriptions in cooked_scene.py.

CPU: the parsed scene graph and FindMeshMaterial's choices equal the descriptions; malformed blobs are refused.
GPU: the loaded scene reports the instance / geometry ids the reference's Embree scenes report, renders the
same image as the same scene built by hand, and traces the oracle's paths."""
import shutil
from pathlib import Path

import numpy as np
import pytest

import cooked_scene as cs
import oracle
import selas_gb300 as sel

ROOT = Path(__file__).resolve().parent / "golden" / "cooked"
SEED = 0x5E1A5000
ASSETS = cs.cooked_cornell()


def _material_fields(m):
    sc = dict(zip(cs.SCALARS, m["scalars"]))
    return m["shader"], tuple(np.float32(m["baseColor"])), tuple(np.float32(m["transmittanceColor"])), tuple(
        np.float32([sc[k] for k in ("metallic", "specularTint", "roughness", "anisotropic", "sheen", "sheenTint",
                                    "clearcoat", "clearcoatGloss", "specTrans", "diffuseTrans", "flatness", "ior",
                                    "scatterDistance")]))


def _sel_fields(m):
    return m.shader, tuple(np.float32(m.baseColor[:])), tuple(np.float32(m.transmittanceColor[:])), tuple(
        np.float32([m.metallic, m.specularTint, m.roughness, m.anisotropic, m.sheen, m.sheenTint, m.clearcoat,
                    m.clearcoatGloss, m.specTrans, m.diffuseTrans, m.flatness, m.ior, m.scatterDistance]))


@pytest.mark.parametrize("name", ["cornell", "cornell_sky", "cornell_ptex", "cornell_hair"])
def test_describe_matches_the_description(name):
    info, meshes = sel.cooked_describe(ROOT, name)
    sd = ASSETS["scenes"][name]
    subs = [ASSETS["subscenes"][s] for s in sd["subscenes"]]
    assert info.subscenes == len(sd["subscenes"]) and info.subsceneInstances == len(sd["instances"])
    assert info.models == sum(len(s["models"]) for s in subs)
    assert info.modelInstances == sum(len(s["instances"]) for s in subs)
    curves = sum(len(ASSETS["models"][m].get("curves", [])) for s in subs for m in s["models"])
    assert (info.lights, info.lightSets, info.cameras, info.curves) == (1, 1, 1, curves)
    assert curves == (2 if name == "cornell_hair" else 0)
    assert list(info.backgroundIntensity) == list(np.float32(sd["background"]))
    assert info.ibl.decode() == sd["ibl"]
    cam = sd["cameras"][0]
    assert list(info.camera.position) == list(np.float32(cam["position"]))
    assert list(info.camera.lookAt) == list(np.float32(cam["look_at"]))
    assert info.camera.fovDegrees == np.float32(cam["fov_degrees"])
    rows = cs.mesh_table(ASSETS, name)
    assert len(meshes) == info.meshes == len(rows)
    assert info.quadMeshes == sum(r[4] == 4 for r in rows) and info.faces == sum(r[5] for r in rows)
    ptex = 0
    for m, (si, mi, k, mat, ipf, faces) in zip(meshes, rows):
        assert (m.subscene, m.model, m.mesh, m.indicesPerFace, m.faces) == (si, mi, k, ipf, faces)
        assert m.materialFlags == mat["flags"]
        assert _sel_fields(m.material) == _material_fields(mat)
        assert m.material.usesPtex == (1 if mat["flags"] & cs.E_USES_PTEX else 0)
        assert m.material.lightSetIndex == subs[si]["light_set"]
        assert m.texture.decode() == mat["texture"]
        ptex += bool(mat["flags"] & cs.E_USES_PTEX)
    assert info.ptexMeshes == ptex == (1 if name == "cornell_ptex" else 0)
    assert info.textures == 1


def test_find_mesh_material_order():
    """The walls take the model's own materials first (left: the model's red, not the subscene's blue 'red'),
    then the subscene's ('green'), then the default (an unknown name)."""
    _, meshes = sel.cooked_describe(ROOT, "cornell")
    by_name = {m.name.decode(): m for m in meshes}
    assert tuple(np.float32(by_name["left"].material.baseColor[:])) == tuple(np.float32((0.65, 0.05, 0.05)))
    assert tuple(np.float32(by_name["right"].material.baseColor[:])) == tuple(np.float32((0.12, 0.45, 0.15)))
    d = by_name["back"].material
    assert tuple(np.float32(d.baseColor[:])) == tuple(np.float32((0.6, 0.6, 0.6))) and d.ior == np.float32(1.5)
    assert d.roughness == 0.0 and d.metallic == 0.0 and d.shader == sel.SEL_SHADER_DISNEY_SOLID


def _copy_tree(tmp_path):
    dst = tmp_path / "cooked"
    shutil.copytree(ROOT, dst)
    return dst


def test_missing_and_truncated_blobs_are_refused(tmp_path):
    root = _copy_tree(tmp_path)
    (root / "_Assets" / "SubsceneResource" / "1539551841" / "props.bin").unlink()
    with pytest.raises(sel.SelError) as e:
        sel.cooked_describe(root, "cornell")
    assert e.value.code == sel.SEL_ERR_IO and "props.bin" in str(e.value)
    root = _copy_tree(tmp_path / "b")
    geo = root / "_Assets" / "ModelGeometryResource" / "1539636447" / "walls.bin"
    geo.write_bytes(geo.read_bytes()[:200])
    with pytest.raises(sel.SelError) as e:
        sel.cooked_describe(root, "cornell")
    assert e.value.code == sel.SEL_ERR_IO and "past the end" in str(e.value)


def test_offsets_and_indices_outside_the_file_are_refused(tmp_path):
    root = _copy_tree(tmp_path)
    model = root / "_Assets" / "ModelResource" / "1539636447" / "walls.bin"
    raw = bytearray(model.read_bytes())
    raw[232 + 24:232 + 32] = (len(raw) + 8).to_bytes(8, "little")  # meshes data offset past the end
    model.write_bytes(bytes(raw))
    with pytest.raises(sel.SelError) as e:
        sel.cooked_describe(root, "cornell")
    assert e.value.code == sel.SEL_ERR_IO
    root = _copy_tree(tmp_path / "b")
    geo = root / "_Assets" / "ModelGeometryResource" / "1539636447" / "box.bin"
    raw = bytearray(geo.read_bytes())
    first = int.from_bytes(raw[64:72], "little")  # offset of the index array
    raw[first:first + 4] = (1000).to_bytes(4, "little")  # a vertex index past the 24 vertices
    geo.write_bytes(bytes(raw))
    with pytest.raises(sel.SelError) as e:
        sel.cooked_describe(root, "cornell")
    assert e.value.code == sel.SEL_ERR_IO and "vertex array" in str(e.value)


# ---------------------------------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------------------------------

def _assert_same_paths(gpu, cpu):
    assert np.isfinite(gpu).all() and np.isfinite(cpu).all()
    rel = np.abs(gpu - cpu) / np.maximum(np.abs(cpu), 1e-3 * cpu.mean())
    assert np.median(rel) < 1e-4, np.median(rel)
    assert (rel < 1e-2).mean() > 0.97, (rel < 1e-2).mean()
    assert abs(gpu.mean() / cpu.mean() - 1.0) < 5e-3


def _camera(info, w, h):
    c = sel.SelCamera()
    c.position[:] = list(info.camera.position)
    c.lookAt[:] = list(info.camera.lookAt)
    c.up[:] = list(info.camera.up)
    c.fovDegrees = info.camera.fovDegrees
    c.width, c.height = w, h
    return c


def _embree_quad_hits(iscene, r):
    """The oracle reports quads as their two triangles; Embree reports the quad (TriangleScene.embree_hits), here
    for hits inside the instance chains of the graph (top part 0, two levels)."""
    hit = r["geomID"] != 0xFFFFFFFF
    for i, sub, _ in iscene.instances[0]:
        for j, model, _ in iscene.instances[sub]:
            sel_ = hit & (r["instID0"] == i) & (r["instID1"] == j)
            part = np.zeros(sel_.sum(), dtype=r.dtype)
            part[:] = r[sel_]
            iscene.parts[model].geometry.embree_hits(part)
            r[sel_] = part


@pytest.mark.gpu
def test_gpu_cooked_queries_report_the_reference_ids(device):
    """Rays from the camera through the room: instID[0] = subscene instance, instID[1] = model instance, geomID =
    mesh, primID and t exactly as the oracle's two-level traversal of the same graph reports them."""
    sc, info = sel.load_cooked(device, ROOT, "cornell")
    try:
        iscene = cs.instanced_scene(ASSETS, "cornell")
        rng = np.random.default_rng(3)
        n = 20000
        org = np.tile(np.float32(info.camera.position), (n, 1))
        target = rng.uniform([0, 0, 0], [556, 556, 556], size=(n, 3)).astype(np.float32)
        d = (target - org).astype(np.float32)
        want = sel.make_rayhits(org, d)
        oracle.instanced_query(iscene.graph(), 0, want)
        _embree_quad_hits(iscene, want)
        got = sel.make_rayhits(org, d)
        sc.intersect1M(got)
        for f in ("geomID", "primID", "instID0", "instID1", "tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z"):
            np.testing.assert_array_equal(got[f], want[f], err_msg=f)
        assert set(np.unique(got["instID0"][got["geomID"] != 0xFFFFFFFF])) == {0, 1}
        assert set(np.unique(got["instID1"][got["instID0"] == 1])) >= {0, 1}
    finally:
        sc.release()


@pytest.mark.gpu
def test_gpu_cooked_scene_equals_the_scene_built_by_hand(device):
    sc, info = sel.load_cooked(device, ROOT, "cornell")
    iscene = cs.instanced_scene(ASSETS, "cornell")
    built = iscene.build(sel, device)
    try:
        cam = _camera(info, 48, 40)
        a = sc.pt_generate_image(cam, sel.pt_settings(4, 6, SEED))
        b = built[0].pt_generate_image(cam, sel.pt_settings(4, 6, SEED))
        np.testing.assert_array_equal(a, b)
    finally:
        iscene.release(built)
        sc.release()


@pytest.mark.gpu
def test_gpu_cooked_curves_report_the_reference_ids(device):
    """The hair subscene's curves load as geomIDs 1 and 2 of the strands model (after its plate mesh), with the
    material curveModelName names; every query field equals that of the same graph built by hand."""
    sc, info = sel.load_cooked(device, ROOT, "cornell_hair")
    iscene = cs.instanced_scene(ASSETS, "cornell_hair")
    built = iscene.build(sel, device)
    try:
        rng = np.random.default_rng(4)
        n = 20000
        org = np.tile(np.float32(info.camera.position), (n, 1))
        # half the rays aimed near the strands' control points (world space), half over the region around them
        model, (_, l2w) = ASSETS["models"]["strands"], ASSETS["subscenes"]["hairy"]["instances"][0]
        cp = model["curve_vertices"][:, :3] @ np.asarray(l2w)[:3, :3].T + np.asarray(l2w)[:3, 3]
        near = cp[rng.integers(0, cp.shape[0], n // 2)] + rng.normal(scale=3.0, size=(n // 2, 3))
        target = np.concatenate([near, rng.uniform([60, 0, 30], [280, 160, 190], size=(n - n // 2, 3))])
        target = target.astype(np.float32)
        d = (target - org).astype(np.float32)
        got, want = sel.make_rayhits(org, d), sel.make_rayhits(org, d)
        sc.intersect1M(got)
        built[0].intersect1M(want)
        for f in ("geomID", "primID", "instID0", "instID1", "tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z"):
            np.testing.assert_array_equal(got[f], want[f], err_msg=f)
        hair = got["instID0"] == 2
        assert set(np.unique(got["geomID"][hair])) == {0, 1, 2}
        assert (got["v"][hair & (got["geomID"] > 0)] == 0).all()
        cam = _camera(info, 48, 40)
        a = sc.pt_generate_image(cam, sel.pt_settings(4, 6, SEED))
        b = built[0].pt_generate_image(cam, sel.pt_settings(4, 6, SEED))
        np.testing.assert_array_equal(a, b)
    finally:
        iscene.release(built)
        sc.release()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cornell", "cornell_sky", "cornell_hair"])
def test_gpu_cooked_scene_traces_the_oracles_paths(device, name):
    sc, info = sel.load_cooked(device, ROOT, name)
    try:
        img = sc.pt_generate_image(_camera(info, 40, 40), sel.pt_settings(8, 6, SEED)).astype(np.float64)
    finally:
        sc.release()
    cpu = oracle.graph_render(cs.instanced_scene(ASSETS, name), 40, 40, 0, 8, max_bounces=6, seed=SEED) / 8.0
    for layer in range(2):
        _assert_same_paths(img[layer], cpu[layer])


@pytest.mark.gpu
def test_gpu_cooked_scene_renders_with_vcm(device):
    sc, info = sel.load_cooked(device, ROOT, "cornell")
    iscene = cs.instanced_scene(ASSETS, "cornell")
    built = iscene.build(sel, device)
    try:
        cam = _camera(info, 32, 32)
        settings = sel.vcm_settings(2, 8, SEED)
        a = sc.vcm_generate_image(cam, settings)
        b = built[0].vcm_generate_image(cam, settings)
        np.testing.assert_array_equal(a, b)
        assert np.isfinite(a).all() and a.mean() > 0
    finally:
        iscene.release(built)
        sc.release()


@pytest.mark.gpu
def test_gpu_ptex_materials_are_refused_unless_asked_for_base_colour(device):
    with pytest.raises(sel.SelError) as e:
        sel.load_cooked(device, ROOT, "cornell_ptex")
    assert e.value.code == sel.SEL_ERR_INVALID_OPERATION and "Ptex" in str(e.value)
    sc, info = sel.load_cooked(device, ROOT, "cornell_ptex", sel.SEL_COOKED_PTEX_AS_BASE_COLOR)
    try:
        assert info.ptexMeshes == 1
        img = sc.pt_generate_image(_camera(info, 24, 24), sel.pt_settings(2, 4, SEED))
        assert np.isfinite(img).all() and img.mean() > 0
    finally:
        sc.release()


@pytest.mark.gpu
def test_gpu_missing_texture_asset_is_refused(device, tmp_path):
    root = tmp_path / "cooked"
    shutil.copytree(ROOT, root)
    (root / "_Assets" / "Textures" / "1534887410" / "checker.bin").unlink()
    with pytest.raises(sel.SelError) as e:
        sel.load_cooked(device, root, "cornell")
    assert e.value.code == sel.SEL_ERR_IO and "checker.bin" in str(e.value)

"""Writes the cooked asset fixtures of tests/golden/cooked/ with the reference's own serializer.

Run on a machine with the reference checkout after `python oracle/ref/build_ref.py`:

    python tests/golden/make_cooked.py

Every blob is produced by SerializeToBinary over the reference's data structures (oracle/ref/cooked_harness.cpp,
compiled into oracle/_ref/libref_pt.so) from the descriptions in tests/cooked_scene.py, then attached again with
the reference's AttachToBinary and checked field by field against the description.  The tests read only the
written files.
"""
from __future__ import annotations

import ctypes
import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import cooked_scene as cs  # noqa: E402

OUT = HERE / "cooked"
_vp, u32, u64, f32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float


def _lib():
    L = ctypes.CDLL(str(ROOT / "oracle" / "_ref" / "libref_pt.so"))
    cp = ctypes.c_char_p
    L.ref_cooked_write_scene.argtypes = [cp, cp, cp, _vp, _vp, u32, _vp, _vp, u32, _vp, u32, _vp, u32, _vp, u32]
    L.ref_cooked_write_subscene.argtypes = [cp, cp, u64, _vp, u32, _vp, _vp, u32, _vp, _vp, _vp, _vp, u32]
    L.ref_cooked_write_model.argtypes = [cp, cp, u32, _vp, _vp, _vp, _vp, u32, _vp, _vp, _vp, u32, _vp, _vp, _vp, _vp,
                                         u32, u32, _vp, u32, _vp, u32, _vp, u32]
    L.ref_cooked_write_texture.argtypes = [cp, cp, u32, u32, _vp, _vp, _vp]
    L.ref_cooked_write_ibl.argtypes = [cp, cp, u32, u32, _vp, u32, u32, _vp, f32, f32]
    L.ref_cooked_read_scene.argtypes = [cp, cp, _vp, _vp, _vp, _vp, _vp, ctypes.c_char_p, u32]
    L.ref_cooked_read_model.argtypes = [cp, cp, _vp, _vp, u32, _vp, u32]
    return L


def _p(a):
    return None if a is None else a.ctypes.data


def _strings(names):
    arr = (ctypes.c_char_p * max(len(names), 1))()
    for i, n in enumerate(names):
        arr[i] = n.encode()
    return arr


def _materials(pairs):
    """(hashes u32, ints (n, 2) u32, floats (n, 20) f32, textures char**) of (name, material) pairs."""
    hashes = np.array([cs.name_hash(n) for n, _ in pairs], np.uint32)
    ints = np.array([[m["shader"], m["flags"]] for _, m in pairs], np.uint32).reshape(-1, 2)
    floats = np.array([list(m["baseColor"]) + list(m["transmittanceColor"]) + list(m["scalars"]) for _, m in pairs],
                      np.float32).reshape(-1, 20)
    return hashes, ints, floats, _strings([m["texture"] for _, m in pairs])


def _instances(insts):
    index = np.array([i for i, _ in insts], np.uint64)
    l2w = np.array([cs.l2w_words(m) for _, m in insts], np.float32).reshape(-1, 16)
    return index, l2w


def write_all(assets, root: Path):
    L = _lib()
    r = str(root).encode()
    for name, t in assets["textures"].items():
        mips = t["mips"]
        w = np.array([m.shape[1] for m in mips], np.uint32)
        h = np.array([m.shape[0] for m in mips], np.uint32)
        data = np.concatenate([m.reshape(-1) for m in mips]).astype(np.float32)
        assert L.ref_cooked_write_texture(r, name.encode(), t["format"], len(mips), _p(w), _p(h), _p(data)) == 0
    for name, b in assets["ibls"].items():
        light = np.ascontiguousarray(b["light"], np.float32)
        miss = np.ascontiguousarray(b["miss"], np.float32)
        assert L.ref_cooked_write_ibl(r, name.encode(), light.shape[1], light.shape[0], _p(light), miss.shape[1],
                                      miss.shape[0], _p(miss), b["rotation"], b["exposure"]) == 0
    for name, m in assets["models"].items():
        pairs = sorted(m["materials"].items(), key=lambda kv: cs.name_hash(kv[0]))  # the build sorts by hash
        hashes, ints, floats, tex = _materials(pairs)
        words = np.array([[x["indexCount"], x["indexOffset"], x["vertexCount"], x["vertexOffset"],
                           cs.name_hash(x["material"]), x["indicesPerFace"], cs.name_hash(x["name"])]
                          for x in m["meshes"]], np.uint32)
        pos = np.ascontiguousarray(m["positions"], np.float32)
        nrm, tan, uvs = (None if m[k] is None else np.ascontiguousarray(m[k], np.float32)
                         for k in ("normals", "tangents", "uvs"))
        idx = np.ascontiguousarray(m["indices"], np.uint32)
        curves = np.ascontiguousarray(np.array(m.get("curves", []), np.uint32).reshape(-1, 2))
        cidx = np.ascontiguousarray(m.get("curve_indices", np.zeros(0)), np.uint32)
        cpts = np.ascontiguousarray(m.get("curve_vertices", np.zeros((0, 4))), np.float32)
        cname = cs.name_hash(m["curve_material"]) if "curve_material" in m else 0
        assert L.ref_cooked_write_model(r, name.encode(), pos.shape[0], _p(pos), _p(nrm), _p(tan), _p(uvs), idx.size,
                                        _p(idx), _p(words), _strings([x["name"] for x in m["meshes"]]),
                                        len(m["meshes"]), _p(hashes), _p(ints), _p(floats), tex, len(pairs), cname,
                                        _p(curves) if curves.size else None, curves.shape[0],
                                        _p(cidx) if cidx.size else None, cidx.size,
                                        _p(cpts) if cpts.size else None, cpts.shape[0]) == 0
        counts = np.zeros(6, np.uint64)
        back_words = np.zeros_like(words)
        back_idx = np.zeros_like(idx)
        assert L.ref_cooked_read_model(r, name.encode(), _p(counts), _p(back_words), words.shape[0], _p(back_idx),
                                       idx.size) == 0
        assert list(counts[:5]) == [len(m["meshes"]), len(pairs), curves.shape[0], pos.shape[0], idx.size], counts
        assert counts[5] == (0 if uvs is None else uvs.size * 4)
        np.testing.assert_array_equal(back_words, words)
        np.testing.assert_array_equal(back_idx, idx)
    for name, s in assets["subscenes"].items():
        hashes, ints, floats, tex = _materials(s["materials"])
        index, l2w = _instances(s["instances"])
        assert L.ref_cooked_write_subscene(r, name.encode(), s["light_set"], _strings(s["models"]), len(s["models"]),
                                           _p(index), _p(l2w), len(index), _p(hashes), _p(ints), _p(floats), tex,
                                           len(hashes)) == 0
    for name, s in assets["scenes"].items():
        index, l2w = _instances(s["instances"])
        lights = np.array([[l["type"], *l["position"], *l["direction"], *l["x"], *l["z"], *l["radiance"]]
                           for l in s["lights"]], np.float32).reshape(-1, 16)
        ranges = np.array(s["ranges"], np.uint32).reshape(-1, 2)
        cams = np.array([[*c["position"], *c["look_at"], *c["up"], c["fov_degrees"], c["znear"], c["zfar"]]
                         for c in s["cameras"]], np.float32).reshape(-1, 12)
        bg = np.array(s["background"], np.float32)
        assert L.ref_cooked_write_scene(r, name.encode(), s["ibl"].encode(), _p(bg), _strings(s["subscenes"]),
                                        len(s["subscenes"]), _p(index), _p(l2w), len(index), _p(lights),
                                        lights.shape[0], _p(ranges), ranges.shape[0], _p(cams), cams.shape[0]) == 0
        counts = np.zeros(5, np.uint64)
        bg_back, inst, light, cam = (np.zeros(n, np.float32) for n in (4, 17, 16, 12))
        ibl = ctypes.create_string_buffer(512)
        assert L.ref_cooked_read_scene(r, name.encode(), _p(counts), _p(bg_back), _p(inst), _p(light), _p(cam), ibl,
                                       512) == 0
        assert list(counts) == [len(s["subscenes"]), len(index), lights.shape[0], ranges.shape[0], cams.shape[0]]
        np.testing.assert_array_equal(bg_back, bg)
        np.testing.assert_array_equal(inst, np.concatenate([[float(index[0])], l2w[0]]).astype(np.float32))
        np.testing.assert_array_equal(light, lights[0])
        np.testing.assert_array_equal(cam, cams[0])
        assert ibl.value.decode() == s["ibl"]


def main():
    if OUT.exists():
        shutil.rmtree(OUT)
    OUT.mkdir(parents=True)
    write_all(cs.cooked_cornell(), OUT)
    total = sum(p.stat().st_size for p in OUT.rglob("*.bin"))
    print(f"wrote {len(list(OUT.rglob('*.bin')))} blobs, {total} bytes, under {OUT}")


if __name__ == "__main__":
    main()

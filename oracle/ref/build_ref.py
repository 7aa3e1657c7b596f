"""ORACLE build recipe for the reference-compiled checker - test infrastructure only.

Compiles the reference's own C++ sources, where they lie in the reference checkout, together with the
harness sources in this folder, into oracle/_ref/.  Nothing is copied into this repository; the outputs
are git-ignored.  Only the machine that has the checkout builds these, to generate the golden fixtures
under tests/golden/ (tests/golden/make_golden.py).

  libref_bsdf.so  - Source/Core/Shading/{Disney,Ggx,Fresnel,SurfaceScattering,Lambert,DiracTransparent}.cpp
                    + Source/Core/MathLib/{FloatFuncs,FloatStructs,Trigonometric,CorrelatedMultiJitter}.cpp
                    + bsdf_harness.cpp
  libref_ptex.so  - Middleware/ptex/Include/Ptex*.cpp (vendored Ptex 2.2, minus the half-table generator)
                    + ptex_harness.cpp, linked with the system zlib
  libref_pt.so    - the reference's path tracer and the code around it: PathTracer.cpp and
                    BuildCommon/BuildImageBasedLight.cpp (compiled inside pt_harness.cpp, whose static functions
                    it calls), Shading/, the scene tables of SceneLib/, GeometryLib/, MathLib/ (all but
                    Sampler.cpp, which the harness supplies), the SystemLib / IoLib / StringLib / UtilityLib /
                    ThreadingLib files those reference, VCMCommon.cpp, and the Ptex objects above; ray queries go
                    to the oracle's BVH (linked from oracle/liboracle.so) through pt_harness.cpp's Embree shim
                    (embree_stubs.c aborts on the scene-building entry points, which nothing reaches);
                    with cooked_harness.cpp and TextureLib/TextureResource.cpp, the reference's serializer writes
                    the cooked asset blobs of tests/golden/cooked/ (tests/golden/make_cooked.py).

The reference checkout is found at $SELAS_REFERENCE, else at ../reference beside this repository.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
REFERENCE = Path(os.environ.get("SELAS_REFERENCE", str(HERE.parents[2] / "reference")))

SELAS_FLAGS = ["-std=c++14", "-O2", "-fPIC", "-include", "cstdlib", "-include", "cstring", "-DIsOsx_=1",
               "-DRelease_=1", "-w"]


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(" ".join(map(str, cmd)) + "\n" + proc.stdout)


def _compile(srcs, flags, objdir):
    objdir.mkdir(parents=True, exist_ok=True)
    cmds, objs = [], []
    for s in srcs:
        o = objdir / (s.stem + ".o")
        objs.append(o)
        if not o.exists() or o.stat().st_mtime < s.stat().st_mtime:
            cmds.append(["g++", *flags, "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, cmds))
    return objs


def build_bsdf(force=False):
    core = REFERENCE / "Source" / "Core"
    srcs = [core / "Shading" / f"{n}.cpp" for n in ("Disney", "Ggx", "Fresnel", "SurfaceScattering", "Lambert",
                                                     "DiracTransparent")]
    srcs += [core / "MathLib" / f"{n}.cpp" for n in ("FloatFuncs", "FloatStructs", "Trigonometric",
                                                     "CorrelatedMultiJitter")]
    srcs += [HERE / "bsdf_harness.cpp"]
    inc = [f"-I{core}", f"-I{REFERENCE / 'Middleware'}", f"-I{REFERENCE / 'Middleware' / 'embree-latest' / 'include'}"]
    objs = _compile(srcs, SELAS_FLAGS + inc, OUT / "obj_bsdf")
    lib = OUT / "libref_bsdf.so"
    if force or not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        _run(["g++", "-shared", "-Wl,--no-undefined", *map(str, objs), "-o", str(lib), "-lm"])
    return lib


def build_ptex(force=False):
    pdir = REFERENCE / "Middleware" / "ptex" / "Include"
    srcs = [p for p in sorted(pdir.glob("Ptex*.cpp")) if p.name != "PtexHalfTableGen.cpp"]
    harness = HERE / "ptex_harness.cpp"
    if harness.exists():
        srcs.append(harness)
    objs = _compile(srcs, ["-std=c++14", "-O2", "-fPIC", "-DPTEX_STATIC", "-w", f"-I{pdir}"], OUT / "obj_ptex")
    lib = OUT / "libref_ptex.so"
    if force or not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        _run(["g++", "-shared", *map(str, objs), "-o", str(lib), "-lz", "-lpthread"])
    return lib


def build_pt(force=False):
    core = REFERENCE / "Source" / "Core"
    app = REFERENCE / "Source" / "Applications" / "Selas" / "Source"
    oracle_dir = HERE.parent
    lib_oracle = oracle_dir / "liboracle.so"
    if not lib_oracle.exists():
        raise RuntimeError("build oracle/liboracle.so first (oracle/build.py)")
    names = {
        "Shading": ["SurfaceParameters", "AreaLighting", "VolumetricScattering", "IsotropicScattering", "Disney",
                    "Ggx", "Fresnel", "SurfaceScattering", "Lambert", "DiracTransparent"],
        "GeometryLib": ["RectangulerLightSampler", "Camera", "Ray", "AxisAlignedBox", "Disc", "SurfaceDifferentials"],
        "SceneLib": ["SceneResource", "SubsceneResource", "ModelResource", "ImageBasedLightResource"],
        "SystemLib": ["MemoryAllocation", "Memory", "JsAssert", "Atomic_Osx", "Error", "SystemTime", "Logging",
                      "BasicTypes"],
        "IoLib": ["BinarySerializers", "Serializer", "SizeSerializer"],
        "StringLib": ["StringUtil"],
        "UtilityLib": ["MurmurHash"],
        "ThreadingLib": ["ThreadLinux"],
        "TextureLib": ["TextureFiltering", "TextureResource"],
    }
    srcs = [core / d / f"{n}.cpp" for d, ns in names.items() for n in ns]
    srcs += [p for p in sorted((core / "MathLib").glob("*.cpp")) if p.name != "Sampler.cpp"]
    srcs += [app / "VCMCommon.cpp", HERE / "pt_harness.cpp", HERE / "cooked_harness.cpp"]
    inc = [f"-I{core}", f"-I{app}", f"-I{REFERENCE / 'Middleware'}", f"-I{REFERENCE / 'Middleware' / 'ptex' / 'Include'}",
           f"-I{REFERENCE / 'Middleware' / 'embree-latest' / 'include'}", f"-I{oracle_dir}"]
    objs = _compile(srcs, SELAS_FLAGS + ["-DPTEX_STATIC"] + inc, OUT / "obj_pt")
    stub = OUT / "obj_pt" / "embree_stubs.o"
    if not stub.exists() or stub.stat().st_mtime < (HERE / "embree_stubs.c").stat().st_mtime:
        _run(["gcc", "-O2", "-fPIC", "-c", str(HERE / "embree_stubs.c"), "-o", str(stub)])
    ptex_objs = [o for o in sorted((OUT / "obj_ptex").glob("*.o")) if o.name != "ptex_harness.o"]
    objs = objs + [stub] + ptex_objs
    lib = OUT / "libref_pt.so"
    deps = objs + [lib_oracle]
    if force or not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in deps):
        _run(["g++", "-shared", "-Wl,--no-undefined", *map(str, objs), "-o", str(lib), f"-L{oracle_dir}", "-loracle",
              f"-Wl,-rpath,{oracle_dir}", "-lz", "-lpthread", "-lm"])
    return lib


def build(force: bool = False):
    if not (REFERENCE / "Source").exists():
        return None
    OUT.mkdir(exist_ok=True)
    build_bsdf(force)
    build_ptex(force)
    build_pt(force)
    return OUT


if __name__ == "__main__":
    print(build(force=True))

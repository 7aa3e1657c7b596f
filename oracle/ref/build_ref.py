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
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
REFERENCE = Path(os.environ.get("SELAS_REFERENCE", "/root/reference"))

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


def build(force: bool = False):
    if not (REFERENCE / "Source").exists():
        return None
    OUT.mkdir(exist_ok=True)
    build_bsdf(force)
    build_ptex(force)
    return OUT


if __name__ == "__main__":
    print(build(force=True))

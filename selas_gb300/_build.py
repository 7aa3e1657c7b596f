"""Builds libselas_gb300.so in-tree from selas_gb300/csrc (CUDA for sm_103a + host C++).

Only nvcc and g++ are used (no cmake, no torch extension machinery).  Objects go to selas_gb300/_build/
and are rebuilt when a source or any header in csrc/ or include/ is newer than the object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libselas_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))


def _stale(src: Path, obj: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or newest_header > t


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def build_library(force: bool = False, jobs: int | None = None) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    OBJ.mkdir(exist_ok=True)
    headers = _headers()
    newest = max((h.stat().st_mtime for h in headers), default=0.0)
    inc = [f"-I{ROOT / 'include'}", f"-I{CSRC}"]
    cmds = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJ / (src.stem + ".cu.o")
        objs.append(obj)
        if force or _stale(src, obj, newest):
            # -fmad=false: no implicit multiply-add contraction, so FP32 shading rounds like the
            # reference's (uncontracted) CPU build; traversal spells out its fmaf / __fmul_rn steps.
            cmds.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-fmad=false",
                         "-Xcompiler", "-fPIC", *inc, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OBJ / (src.stem + ".cpp.o")
        objs.append(obj)
        if force or _stale(src, obj, newest):
            cmds.append(["g++", "-O3", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off",
                         f"-I{cuda / 'include'}", *inc, "-c", str(src), "-o", str(obj)])
    if cmds:
        with ThreadPoolExecutor(max_workers=jobs or min(len(cmds), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, cmds))
    if cmds or force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-Xcompiler", "-pthread",
              *map(str, objs), "-o", str(tmp)])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library())

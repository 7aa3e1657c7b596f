"""ORACLE build recipe - test infrastructure only (the product never loads anything built here).

Builds
  * oracle/liboracle.so  - the CPU restatements in oracle/*.cpp (g++, -ffp-contract=off), always;
  * oracle/_ref/...      - the reference's own C++ sources compiled where they lie under the reference
                           checkout, when that checkout is present (see oracle/ref/build_ref.py).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"


def build_oracle(force: bool = False) -> Path:
    srcs = sorted(HERE.glob("*.cpp"))
    deps = srcs + sorted(HERE.glob("*.h"))
    if not force and LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in deps):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
           *map(str, srcs), "-o", str(tmp)]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    os.replace(tmp, LIB)
    return LIB


def build_reference(force: bool = False) -> Path | None:
    """Compiles the reference's BSDF/Ptex sources into oracle/_ref when the checkout exists."""
    sys.path.insert(0, str(HERE / "ref"))
    try:
        import build_ref  # type: ignore
    finally:
        sys.path.pop(0)
    return build_ref.build(force=force)


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))

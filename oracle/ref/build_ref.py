"""ORACLE build recipe for the reference-compiled checker - test infrastructure only.

Compiles the reference's own C++ sources, where they lie in the reference checkout, together with the
small harness sources in this folder, into oracle/_ref/.  Nothing is copied into this repository; the
outputs are git-ignored.  Used only on the machine that has the checkout, to generate the golden
fixtures under tests/golden/.
"""
from __future__ import annotations

import os
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"
REFERENCE = Path(os.environ.get("SELAS_REFERENCE", "/root/reference"))


def build(force: bool = False):
    if not (REFERENCE / "Source").exists():
        return None
    OUT.mkdir(exist_ok=True)
    return OUT

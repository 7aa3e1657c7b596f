"""The drop-in boundary as a C++ caller sees it (tests/boundary/boundary.cpp): include/selas.h compiled against
Embree 3.2's own headers asserts every RTCRay / RTCHit / RTCRayHit field offset at compile time (CPU, where the
reference's Middleware/embree-latest/include is present), and the INTEGRATION.md calls run against
libselas_gb300.so on a small scene (GPU)."""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "boundary" / "boundary.cpp"
EMBREE = Path(os.environ.get("SELAS_REFERENCE", str(ROOT.parent / "reference"))) / "Middleware" / "embree-latest" / "include"


def _compile(out, embree: bool):
    cmd = ["g++", "-std=c++14", "-O1", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(SRC), "-o", str(out),
           f"-L{ROOT / 'selas_gb300'}", "-lselas_gb300", f"-Wl,-rpath,{ROOT / 'selas_gb300'}"]
    if embree:
        cmd[1:1] = ["-DSEL_CHECK_EMBREE_LAYOUT", f"-I{EMBREE}"]
    return subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)


@pytest.fixture(scope="module")
def library():
    from selas_gb300._build import build_library
    return build_library()


def test_records_match_embree_headers(library, tmp_path):
    if not (EMBREE / "embree3" / "rtcore_ray.h").exists():
        pytest.skip("the reference's Embree headers are not on this machine")
    proc = _compile(tmp_path / "boundary", embree=True)
    assert proc.returncode == 0, proc.stdout


@pytest.mark.gpu
def test_integration_calls_run(library, tmp_path):
    embree = (EMBREE / "embree3" / "rtcore_ray.h").exists()
    exe = tmp_path / "boundary"
    proc = _compile(exe, embree=embree)
    assert proc.returncode == 0, proc.stdout
    run = subprocess.run([str(exe)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    assert run.returncode == 0 and "boundary ok" in run.stdout, run.stdout

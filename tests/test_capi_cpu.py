"""CPU checks of the C ABI: the library loads, exports every function include/selas.h declares, its record
layouts match Embree's, and argument errors come back as status codes (no GPU needed)."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(sel_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from selas_gb300._build import build_library
    build_library()
    import selas_gb300
    return selas_gb300.lib()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 16
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"


def test_record_layouts_match_embree():
    import selas_gb300 as sel
    assert sel.RAY_DTYPE.itemsize == 48 and sel.RAYHIT_DTYPE.itemsize == 96
    assert sel.RAYHIT_DTYPE.fields["Ng_x"][1] == 48
    assert sel.RAYHIT_DTYPE.fields["primID"][1] == 68
    assert sel.RAY_DTYPE.fields["tfar"][1] == 32


def test_null_handles_are_rejected(lib):
    import selas_gb300 as sel
    assert lib.sel_scene_commit(None) == sel.SEL_ERR_INVALID_ARGUMENT
    assert lib.sel_intersect1M(None, None, 0, 96) == sel.SEL_ERR_INVALID_ARGUMENT
    assert lib.sel_occluded_device(None, None, 0, None) == sel.SEL_ERR_INVALID_ARGUMENT
    assert lib.sel_device_new(0, None) == sel.SEL_ERR_INVALID_ARGUMENT
    assert b"null" in lib.sel_get_last_error()


def test_no_gpu_reports_an_error_instead_of_aborting(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.sel_device_new(0, ctypes.byref(h))
    assert rc != 0 and not h.value


def test_vcm_settings_defaults_and_layout(lib):
    import selas_gb300 as sel
    assert ctypes.sizeof(sel.SelVcmSettings) == 32
    s = sel.vcm_settings(7)
    assert (s.passes, s.maxPathLength, s.disableMerging) == (7, 10, 0)
    assert s.radiusAlpha == pytest.approx(0.75) and s.radius == 0.0
    assert lib.sel_vcm_settings_defaults(None) == sel.SEL_ERR_INVALID_ARGUMENT
    assert lib.sel_vcm_generate_image(None, None, None, None) == sel.SEL_ERR_INVALID_ARGUMENT


def test_deferred_settings_defaults(lib):
    import selas_gb300 as sel
    s = sel.SelPtSettings()
    assert lib.sel_deferred_settings_defaults(ctypes.byref(s)) == 0
    assert (s.samplesPerPixel, s.maxBounces, s.pathsInFlight, s.traceBlockSize) == (16, 64, 0, 0)
    assert sel.deferred_settings(5, 12).samplesPerPixel == 25
    assert lib.sel_deferred_settings_defaults(None) == sel.SEL_ERR_INVALID_ARGUMENT
    assert lib.sel_deferred_generate_image(None, None, None, None) == sel.SEL_ERR_INVALID_ARGUMENT
    j = sel.SelJob()
    j.camera.width, j.camera.height, j.integrator = 10, 6, sel.SEL_INTEGRATOR_DEFERRED
    n = ctypes.c_size_t()
    assert lib.sel_server_result_floats(ctypes.byref(j), ctypes.byref(n)) == 0 and n.value == 180


def test_server_records_and_defaults(lib):
    import selas_gb300 as sel
    assert ctypes.sizeof(sel.SelJob) == 120 and ctypes.sizeof(sel.SelServerConfig) == 32
    c = sel.server_config()
    assert (c.max_jobs, c.paths_in_flight, c.max_bounces) == (16, 1 << 22, 8)
    assert c.hbm_reserve_bytes == 2 << 30
    assert lib.sel_server_new(None, None, None) == sel.SEL_ERR_INVALID_ARGUMENT
    j = sel.SelJob()
    j.camera.width, j.camera.height, j.integrator = 10, 6, sel.SEL_INTEGRATOR_PT
    n = ctypes.c_size_t()
    assert lib.sel_server_result_floats(ctypes.byref(j), ctypes.byref(n)) == 0 and n.value == 360

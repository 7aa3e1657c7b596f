import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

HIT_FIELDS = ("tfar", "u", "v", "Ng_x", "Ng_y", "Ng_z", "primID", "geomID", "instID0", "instID1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 host)")


def assert_hits_equal(got, want, fields=HIT_FIELDS):
    """Bit-exact comparison of ray/hit records field by field (padding bytes are ignored)."""
    for f in fields:
        a, b = got[f], want[f]
        same = (a.view(np.uint32) == b.view(np.uint32)) if a.dtype.kind == "f" else (a == b)
        if not same.all():
            bad = np.nonzero(~same)[0]
            i = bad[0]
            raise AssertionError(f"field {f}: {bad.size} of {a.size} records differ; first at {i}: got {a[i]!r} want {b[i]!r}")


@pytest.fixture(scope="session")
def device():
    from selas_gb300._build import build_library
    build_library()
    import selas_gb300 as sel
    dev = sel.Device(0)
    yield dev
    dev.release()

"""ORACLE - test infrastructure only.

ctypes view of oracle/liboracle.so (the CPU restatements in oracle/*.cpp).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this package, as the checker; the product
(selas_gb300) never does.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_lib = None
_vp, _i64, _i = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        from .build import build_oracle
        path = build_oracle()
        _lib = ctypes.CDLL(str(path))
        sig = {
            "oracle_intersect_bruteforce": ([_vp, _vp, _vp, _i64, _vp, _i64, _i], None),
            "oracle_occluded_bruteforce": ([_vp, _vp, _vp, _i64, _vp, _i64, _i], None),
            "oracle_bvh_build": ([_vp, _vp, _vp, _i64], _vp),
            "oracle_bvh_free": ([_vp], None),
            "oracle_intersect_bvh": ([_vp, _vp, _i64, _i], None),
            "oracle_occluded_bvh": ([_vp, _vp, _i64, _i], None),
        }
        for name, (args, res) in sig.items():
            fn = getattr(_lib, name)
            fn.argtypes = args
            fn.restype = res
        extra = getattr(__import__(__name__), "_extra_signatures", {})
        for name, (args, res) in extra.items():
            fn = getattr(_lib, name)
            fn.argtypes = args
            fn.restype = res
    return _lib


def threads() -> int:
    return int(os.environ.get("ORACLE_THREADS", os.cpu_count() or 1))


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def intersect_bruteforce(soup, rayhits: np.ndarray, nthreads: int | None = None) -> None:
    v, p, g = soup
    lib().oracle_intersect_bruteforce(_p(v), _p(p), _p(g), v.shape[0], _p(rayhits), rayhits.shape[0],
                                      nthreads or threads())


def occluded_bruteforce(soup, rays: np.ndarray, nthreads: int | None = None) -> None:
    v, p, g = soup
    lib().oracle_occluded_bruteforce(_p(v), _p(p), _p(g), v.shape[0], _p(rays), rays.shape[0], nthreads or threads())


class OracleBvh:
    """The oracle's own binned-SAH binary BVH over a triangle soup."""

    def __init__(self, soup):
        v, p, g = soup
        self._keep = soup
        self.handle = lib().oracle_bvh_build(_p(v), _p(p), _p(g), v.shape[0])

    def intersect(self, rayhits: np.ndarray, nthreads: int | None = None) -> None:
        lib().oracle_intersect_bvh(self.handle, _p(rayhits), rayhits.shape[0], nthreads or threads())

    def occluded(self, rays: np.ndarray, nthreads: int | None = None) -> None:
        lib().oracle_occluded_bvh(self.handle, _p(rays), rays.shape[0], nthreads or threads())

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.oracle_bvh_free(self.handle)
            self.handle = None

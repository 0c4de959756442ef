"""TEST INFRASTRUCTURE ONLY: Python handle on the FP64 CPU oracle (oracle/glia_oracle.cpp).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline legs to check results; the
product path never imports this module. `load()` builds the oracle with its Makefile when the
shared library is missing or older than its source.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from glia_gb300 import _abi  # noqa: E402
from glia_gb300.context import Context  # noqa: E402

LIB = os.path.join(_HERE, "_build", "liboracle.so")
_SRC = [os.path.join(_HERE, "glia_oracle.cpp"), os.path.join(_ROOT, "include", "glia_rd.h")]
_api = None


def build(force: bool = False) -> str:
    stale = not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in _SRC)
    if force or stale:
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB


def load() -> _abi.Bound:
    global _api
    if _api is None:
        build()
        lib = ctypes.CDLL(LIB)
        _api = _abi.Bound(lib, "oracle_glia_", optional=("set_timing", "get_timing", "mismatch_f32_noalloc",
                                                       "set_launch_geometry",
                                                       "selftest_bounded_wait",
                                                       *_abi.BATCH_NAMES))
        for name, res, args in (
            ("oracle_fft_r2c", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
            ("oracle_fft_c2r", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
            ("oracle_glia_set_num_threads", ctypes.c_int, [ctypes.c_int]),
        ):
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _api.fft_r2c = lib.oracle_fft_r2c
        _api.fft_c2r = lib.oracle_fft_c2r
        _api.set_num_threads = lib.oracle_glia_set_num_threads
    return _api


def context(n: int) -> Context:
    """An oracle context (FP64, host pointers)."""
    return Context(load(), n, _abi.GLIA_FP64, _abi.GLIA_ENGINE_REFERENCE)


def set_num_threads(k: int) -> int:
    return load().set_num_threads(int(k))

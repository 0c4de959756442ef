"""Loader of the in-tree CUDA library. There is no CPU fallback: if the library is missing or
no GPU is visible, the calls that need it raise."""
from __future__ import annotations

import ctypes
import os

from . import _abi
from .build import LIB, build, up_to_date

_api = None


def load(auto_build: bool = True) -> _abi.Bound:
    """Bind libglia_rd.so (building it in-tree first when it is missing or stale)."""
    global _api
    if _api is not None:
        return _api
    if not up_to_date():
        if not auto_build:
            raise RuntimeError(f"{LIB} is missing or stale; run glia_gb300.build.build()")
        build()
    if not os.path.exists(LIB):
        raise RuntimeError(f"CUDA library {LIB} was not built")
    lib = ctypes.CDLL(LIB, mode=ctypes.RTLD_GLOBAL)
    _api = _abi.Bound(lib, "glia_")
    return _api


def library_path() -> str:
    return LIB

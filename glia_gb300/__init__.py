"""glia_gb300 — GB300-native reaction–diffusion forward / adjoint path of GLIA.

The compute path is the CUDA library glia_gb300/_build/libglia_rd.so behind the C-ABI of
include/glia_rd.h. This package binds it (ctypes), mirrors the reference's solver classes on top
(`solver`), and offers a torch.autograd.Function over the adjoint gradient (`autograd`).
"""
from . import _abi  # noqa: F401
from .context import Context, GliaError  # noqa: F401

__all__ = ["Context", "GliaError", "open_context"]


def open_context(n: int, precision: int = _abi.GLIA_MIXED, engine: int = _abi.GLIA_ENGINE_FUSED):
    """A context on the CUDA library (builds the library in-tree on first use)."""
    from .native import load

    return Context(load(), n, precision, engine)

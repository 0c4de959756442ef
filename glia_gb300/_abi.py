"""ctypes description of the C-ABI declared in include/glia_rd.h.

`bind(lib, prefix)` returns an object whose attributes are the C entry points with their
argument and return types set. The same table binds the CUDA library (prefix "glia_") and any
other library that exports the same entry points under another prefix.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_int, c_int64, c_void_p

GLIA_OK = 0
GLIA_ERR_INVALID = -1
GLIA_ERR_CUDA = -2
GLIA_ERR_CUFFT = -3
GLIA_ERR_NOT_CONVERGED = -4
GLIA_ERR_STATE = -5
GLIA_ERR_OOM = -6
GLIA_ERR_NONFINITE = -7
GLIA_ERR_NO_DEVICE = -8

GLIA_FP64 = 0
GLIA_MIXED = 1
GLIA_ENGINE_FUSED = 0
GLIA_ENGINE_REFERENCE = 1
GLIA_PTR_HOST_F64 = 0
GLIA_PTR_DEVICE_F64 = 1
GLIA_PTR_DEVICE_F32 = 2
GLIA_HISTORY_FULL = 0
GLIA_HISTORY_CHECKPOINT = 1
GLIA_HISTORY_OFF = 2
GLIA_PC_DT_REFERENCE = 0
GLIA_PC_DT_FIXED = 1
GLIA_PC_DT_MATCHED = 2

ERROR_NAMES = {
    GLIA_ERR_INVALID: "GLIA_ERR_INVALID",
    GLIA_ERR_CUDA: "GLIA_ERR_CUDA",
    GLIA_ERR_CUFFT: "GLIA_ERR_CUFFT",
    GLIA_ERR_NOT_CONVERGED: "GLIA_ERR_NOT_CONVERGED",
    GLIA_ERR_STATE: "GLIA_ERR_STATE",
    GLIA_ERR_OOM: "GLIA_ERR_OOM",
    GLIA_ERR_NONFINITE: "GLIA_ERR_NONFINITE",
    GLIA_ERR_NO_DEVICE: "GLIA_ERR_NO_DEVICE",
}


class GliaOptSettings(ctypes.Structure):
    _fields_ = [
        ("np", c_int),
        ("nk", c_int),
        ("nr", c_int),
        ("flag_reaction_inv", c_int),
        ("diffusivity_inversion", c_int),
        ("regularization_norm", c_int),
        ("beta", c_double),
        ("k_scale", c_double),
        ("rho_scale", c_double),
        ("phi_store", c_int),
        ("all_gradients", c_int),
    ]


class GliaStats(ctypes.Structure):
    _fields_ = [
        ("nb_state_solves", c_int64),
        ("nb_adjoint_solves", c_int64),
        ("nb_obj_evals", c_int64),
        ("nb_grad_evals", c_int64),
        ("diff_ksp_itr_state", c_int64),
        ("diff_ksp_itr_adj", c_int64),
        ("total_diffusion_solves", c_int64),
        ("total_pcg_iterations", c_int64),
        ("total_fft_execs", c_int64),
        ("last_ksp_itr", c_int),
        ("max_ksp_itr", c_int),
        ("last_rnorm", c_double),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_P = c_void_p
_D = POINTER(c_double)
_CTX = c_void_p

# name -> (restype, argtypes); every entry point of include/glia_rd.h
SIGNATURES = {
    "create": (c_int, [c_int, c_int, c_int, POINTER(c_void_p)]),
    "destroy": (c_int, [_CTX]),
    "last_error": (c_char_p, [_CTX]),
    "version": (c_char_p, []),
    "set_pointer_mode": (c_int, [_CTX, c_int]),
    "set_stream": (c_int, [_CTX, c_void_p]),
    "synchronize": (c_int, [_CTX]),
    "set_launch_geometry": (c_int, [_CTX, c_int, c_int]),
    "device_bytes": (c_int, [_CTX, POINTER(c_int64)]),
    "set_time": (c_int, [_CTX, c_double, c_int, c_int]),
    "set_pcg": (c_int, [_CTX, c_double, c_int, c_int, c_double]),
    "set_history": (c_int, [_CTX, c_int, c_int, c_int]),
    "set_opt": (c_int, [_CTX, POINTER(GliaOptSettings)]),
    "set_tissue": (c_int, [_CTX, _P, _P, _P, _P]),
    "set_tissue_sinusoidal": (c_int, [_CTX]),
    "set_coefficients": (c_int, [_CTX, c_double, c_double, c_double, c_double, c_double, c_double]),
    "set_diffusivity_sinusoidal": (c_int, [_CTX, c_double]),
    "prec_factor": (c_int, [_CTX]),
    "diffusion_solve": (c_int, [_CTX, _P, c_double, POINTER(c_int)]),
    "apply_d": (c_int, [_CTX, _P, _P]),
    "smooth": (c_int, [_CTX, _P, _P, c_double]),
    "phi_mesh": (c_int, [c_int, _D, c_double, c_double, _D]),
    "set_phi": (c_int, [_CTX, _D, c_int, c_double, c_double]),
    "phi_apply": (c_int, [_CTX, _D, _P]),
    "phi_apply_transpose": (c_int, [_CTX, _P, _D]),
    "phi_data_centers": (c_int, [_CTX, _P, c_double, c_double, c_double, c_double, c_int, _D,
                                 POINTER(c_int), _P]),
    "set_obs_threshold": (c_int, [_CTX, _P, c_double]),
    "set_obs_filter": (c_int, [_CTX, _P]),
    "set_obs_threshold0": (c_int, [_CTX, _P, c_double]),
    "set_obs_filter0": (c_int, [_CTX, _P]),
    "set_data0": (c_int, [_CTX, _P]),
    "set_c0": (c_int, [_CTX, _P]),
    "set_secondary_coefficients": (c_int, [_CTX, c_double, c_double, c_double]),
    "solve_state": (c_int, [_CTX, c_int, _P, _P]),
    "solve_adjoint": (c_int, [_CTX, c_int, _P, _P]),
    "get_state": (c_int, [_CTX, c_int, _P]),
    "get_adjoint": (c_int, [_CTX, c_int, _P]),
    "eval_objective": (c_int, [_CTX, _D, c_int, _P, _D]),
    "eval_gradient": (c_int, [_CTX, _D, c_int, _P, _D]),
    "eval_objective_and_gradient": (c_int, [_CTX, _D, c_int, _P, _D, _D]),
    "hessian_matvec": (c_int, [_CTX, _D, c_int, _D]),
    "selftest_bounded_wait": (c_int, [_CTX]),
    "get_stats": (c_int, [_CTX, POINTER(GliaStats)]),
    "reset_stats": (c_int, [_CTX]),
    "set_timing": (c_int, [_CTX, c_int]),
    "mismatch_f32_noalloc": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p,
                                     c_void_p]),
    "get_timing": (c_int, [_CTX, c_int, POINTER(c_char_p), POINTER(c_int64), POINTER(c_double),
                           POINTER(c_double)]),
    "batch_create": (c_int, [POINTER(c_void_p), c_int, POINTER(c_void_p)]),
    "batch_capture": (c_int, [c_void_p, POINTER(_D), POINTER(c_int), POINTER(c_void_p),
                              POINTER(c_int)]),
    "batch_launch": (c_int, [c_void_p, c_void_p]),
    "batch_results": (c_int, [c_void_p, c_void_p, _D, POINTER(_D)]),
    "batch_last_error": (c_char_p, [c_void_p]),
    "batch_destroy": (c_int, [c_void_p]),
}

# entry points of the CUDA library only (the oracle evaluates one problem per call)
BATCH_NAMES = ("batch_create", "batch_capture", "batch_launch", "batch_results",
               "batch_last_error", "batch_destroy")


class Bound:
    """Entry points of one library, looked up as `<prefix><name>`."""

    def __init__(self, lib: ctypes.CDLL, prefix: str, names=None, optional=()):
        self.lib = lib
        self.prefix = prefix
        self.missing = []
        for name in names or SIGNATURES:
            restype, argtypes = SIGNATURES[name]
            sym = prefix + name
            try:
                fn = getattr(lib, sym)
            except AttributeError:
                if name in optional:
                    self.missing.append(name)
                    continue
                raise
            fn.restype = restype
            fn.argtypes = argtypes
            setattr(self, name, fn)


def exported_names(prefix: str = "glia_") -> list[str]:
    return [prefix + n for n in SIGNATURES]

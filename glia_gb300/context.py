"""Python handle over one C-ABI context (include/glia_rd.h).

`Context` owns a `glia_ctx*` and converts arguments: grid fields may be numpy float64 arrays
(host pointer mode) or torch CUDA tensors (device pointer modes); parameter vectors are numpy
float64. Errors raise `GliaError` with the library's message. The class is agnostic of which
library it drives: `bind` decides (the CUDA library for the product path).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi


class GliaError(RuntimeError):
    def __init__(self, code: int, where: str, message: str):
        self.code = code
        super().__init__(f"{where}: {_abi.ERROR_NAMES.get(code, code)}: {message}")


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Context:
    def __init__(self, api: _abi.Bound, n: int, precision: int = _abi.GLIA_FP64,
                 engine: int = _abi.GLIA_ENGINE_FUSED):
        self.api = api
        self.n = int(n)
        self.N = self.n ** 3
        self.precision = precision
        self.engine = engine
        self.ptr_mode = _abi.GLIA_PTR_HOST_F64
        self._h = ctypes.c_void_p()
        rc = api.create(self.n, precision, engine, ctypes.byref(self._h))
        if rc != _abi.GLIA_OK:
            raise GliaError(rc, "create", f"n={n} precision={precision} engine={engine}")
        # advanced by every call that rewrites the state history, the coefficients or the model
        # settings (autograd backward passes compare it with the value seen by their forward)
        self.generation = 0
        self.phi_generation = 0  # advanced when the Gaussian basis may change
        self.stream = 0          # the CUDA stream handle last given to set_stream (0 = own)
        self._opt = _abi.GliaOptSettings(np=1, nk=1, nr=1, flag_reaction_inv=0,
                                         diffusivity_inversion=1, regularization_norm=0,
                                         beta=1e-4, k_scale=1.0, rho_scale=1.0, phi_store=0,
                                         all_gradients=0)

    # -- plumbing -------------------------------------------------------------------------
    def close(self):
        if self._h:
            self.api.destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int, where: str):
        if rc != _abi.GLIA_OK:
            msg = self.api.last_error(self._h)
            raise GliaError(rc, where, msg.decode() if msg else "")

    def _field_in(self, a):
        """Pointer for an input grid field (or None)."""
        if a is None:
            return None
        if isinstance(a, np.ndarray):
            if self.ptr_mode != _abi.GLIA_PTR_HOST_F64:
                raise ValueError("numpy field given while the context is in device pointer mode")
            a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
            if a.size != self.N:
                raise ValueError(f"field has {a.size} values, expected {self.N}")
            self._keep.append(a)
            return ctypes.c_void_p(a.ctypes.data)
        # torch tensor
        if a.numel() != self.N or not a.is_contiguous():
            raise ValueError("device field must be contiguous with n^3 values")
        want = {_abi.GLIA_PTR_DEVICE_F64: "torch.float64",
                _abi.GLIA_PTR_DEVICE_F32: "torch.float32"}.get(self.ptr_mode)
        if want is None or str(a.dtype) != want or not a.is_cuda:
            raise ValueError(f"device field must be a CUDA tensor of {want}")
        return ctypes.c_void_p(a.data_ptr())

    def _field_out(self, out):
        if out is None:
            if self.ptr_mode != _abi.GLIA_PTR_HOST_F64:
                raise ValueError("device pointer mode needs an explicit output tensor")
            out = np.empty(self.N, dtype=np.float64)
        return out, self._field_in(out)

    def _touch(self, phi=False):
        self.generation += 1
        if phi:
            self.phi_generation += 1

    def _call(self, where, fn, *args):
        self._keep = []
        try:
            self._check(fn(self._h, *args), where)
        finally:
            self._keep = []

    # -- configuration --------------------------------------------------------------------
    def set_pointer_mode(self, mode: int):
        self._call("set_pointer_mode", self.api.set_pointer_mode, mode)
        self.ptr_mode = mode

    def set_time(self, dt: float, nt: int, order: int = 2):
        self._touch()
        self._call("set_time", self.api.set_time, dt, nt, order)

    def set_pcg(self, rtol=1e-6, maxit=5000, pc_dt_mode=_abi.GLIA_PC_DT_REFERENCE, pc_dt=0.0):
        self._touch()
        self._call("set_pcg", self.api.set_pcg, rtol, maxit, pc_dt_mode, pc_dt)

    def set_history(self, mode=_abi.GLIA_HISTORY_FULL, every=0, adjoint_store=False):
        self._touch()
        self._call("set_history", self.api.set_history, mode, every, int(adjoint_store))

    def set_opt(self, **kw):
        self._touch(phi=True)
        for k, v in kw.items():
            if not hasattr(self._opt, k):
                raise KeyError(k)
            setattr(self._opt, k, v)
        self._call("set_opt", self.api.set_opt, ctypes.byref(self._opt))

    @property
    def nx(self) -> int:
        return self._opt.np + self._opt.nk + self._opt.nr

    def set_tissue(self, wm=None, gm=None, csf=None, vt=None):
        self._touch(phi=True)
        self._keep = []
        args = [self._field_in(a) for a in (wm, gm, csf, vt)]
        try:
            self._check(self.api.set_tissue(self._h, *args), "set_tissue")
        finally:
            self._keep = []

    def set_tissue_sinusoidal(self):
        self._touch(phi=True)
        self._call("set_tissue_sinusoidal", self.api.set_tissue_sinusoidal)

    def set_coefficients(self, k, rho, k_gm_wm=0.0, k_glm_wm=0.0, r_gm_wm=0.0, r_glm_wm=0.0):
        self._touch()
        self._call("set_coefficients", self.api.set_coefficients, k, k_gm_wm, k_glm_wm, rho,
                   r_gm_wm, r_glm_wm)

    def set_diffusivity_sinusoidal(self, scale):
        self._touch()
        self._call("set_diffusivity_sinusoidal", self.api.set_diffusivity_sinusoidal, scale)

    def prec_factor(self):
        self._touch()
        self._call("prec_factor", self.api.prec_factor)

    def set_phi(self, centers, sigma, smoothing_factor=1.0):
        self._touch(phi=True)
        c = np.ascontiguousarray(centers, dtype=np.float64).reshape(-1)
        self._call("set_phi", self.api.set_phi, _dptr(c), c.size // 3, sigma, smoothing_factor)

    def set_obs_threshold(self, data, thr):
        self._keep = []
        try:
            self._check(self.api.set_obs_threshold(self._h, self._field_in(data), thr),
                        "set_obs_threshold")
        finally:
            self._keep = []

    def set_obs_filter(self, f):
        self._keep = []
        try:
            self._check(self.api.set_obs_filter(self._h, self._field_in(f)), "set_obs_filter")
        finally:
            self._keep = []

    def set_obs_threshold0(self, data, thr):
        """Observation operator at t = 0 of the two-snapshot objective: [data > thr]."""
        self._keep = []
        try:
            self._check(self.api.set_obs_threshold0(self._h, self._field_in(data), thr),
                        "set_obs_threshold0")
        finally:
            self._keep = []

    def set_obs_filter0(self, f):
        self._keep = []
        try:
            self._check(self.api.set_obs_filter0(self._h, self._field_in(f)), "set_obs_filter0")
        finally:
            self._keep = []

    def set_data0(self, d0):
        """Data at t = 0 (two-snapshot objective); None returns to one snapshot."""
        self._keep = []
        try:
            p = None if d0 is None else self._field_in(d0)
            self._check(self.api.set_data0(self._h, p), "set_data0")
        finally:
            self._keep = []

    def set_c0(self, c0):
        self._touch()
        self._keep = []
        try:
            self._check(self.api.set_c0(self._h, self._field_in(c0)), "set_c0")
        finally:
            self._keep = []

    # -- operators ------------------------------------------------------------------------
    def diffusion_solve(self, c, dt):
        """In place on `c`; returns the PCG iteration count."""
        self._touch()
        self._keep = []
        its = ctypes.c_int(0)
        try:
            if isinstance(c, np.ndarray):
                if c.dtype != np.float64 or not c.flags.c_contiguous or c.size != self.N:
                    raise ValueError("host field must be contiguous float64 with n^3 values")
                p = ctypes.c_void_p(c.ctypes.data)
            else:
                p = self._field_in(c)
            self._check(self.api.diffusion_solve(self._h, p, dt, ctypes.byref(its)),
                        "diffusion_solve")
        finally:
            self._keep = []
        return its.value

    def _unary(self, name, fn, x, out, *extra):
        self._keep = []
        try:
            out, po = self._field_out(out)
            self._check(fn(self._h, po, self._field_in(x), *extra) if name == "smooth"
                        else fn(self._h, self._field_in(x), po, *extra), name)
        finally:
            self._keep = []
        return out

    def apply_d(self, c, out=None):
        return self._unary("apply_d", self.api.apply_d, c, out)

    def smooth(self, c, sigma, out=None):
        return self._unary("smooth", self.api.smooth, c, out, sigma)

    def phi_apply(self, p, out=None):
        p = np.ascontiguousarray(p, dtype=np.float64)
        self._keep = []
        try:
            out, po = self._field_out(out)
            self._check(self.api.phi_apply(self._h, _dptr(p), po), "phi_apply")
        finally:
            self._keep = []
        return out

    def phi_apply_transpose(self, v, np_):
        pout = np.zeros(np_, dtype=np.float64)
        self._keep = []
        try:
            self._check(self.api.phi_apply_transpose(self._h, self._field_in(v), _dptr(pout)),
                        "phi_apply_transpose")
        finally:
            self._keep = []
        return pout

    def phi_data_centers(self, data, sigma, data_threshold=0.05, gaussian_vol_frac=0.0,
                         spacing_factor=2.0, with_frac=False):
        """Phi::setGaussians(Vec data): (centres (np, 3), num_tumor_output field or None)."""
        n, h = self.n, 2 * np.pi / self.n
        space = spacing_factor * sigma / h
        hits = [x for x in range(n) if space >= 1 and np.fmod(x, space) == 0.0]
        cap = max(1, (len(range(hits[0], hits[-1] + 1, max(1, int(space)))) + 1) ** 3) \
            if hits else 1
        out = np.zeros(3 * cap, dtype=np.float64)
        cnt = ctypes.c_int(0)
        self._keep = []
        try:
            frac, pf = self._field_out(None) if with_frac else (None, None)
            self._check(self.api.phi_data_centers(self._h, self._field_in(data), sigma,
                                                  data_threshold, gaussian_vol_frac,
                                                  spacing_factor, cap, _dptr(out),
                                                  ctypes.byref(cnt), pf), "phi_data_centers")
        finally:
            self._keep = []
        return out[:3 * cnt.value].reshape(-1, 3).copy(), frac

    def set_secondary_coefficients(self, k1, k2=0.0, k3=0.0):
        """DiffCoef::setSecondaryCoefficients: the diffusivity direction of solve_state(2)."""
        self._touch()
        self._call("set_secondary_coefficients", self.api.set_secondary_coefficients, k1, k2, k3)

    def solve_state(self, c0=None, out=None, linearized=0):
        self._touch()
        self._keep = []
        try:
            out, po = self._field_out(out)
            self._check(self.api.solve_state(self._h, linearized, self._field_in(c0), po),
                        "solve_state")
        finally:
            self._keep = []
        return out

    def solve_adjoint(self, pt=None, out=None, linearized=1):
        self._keep = []
        try:
            out, po = self._field_out(out)
            self._check(self.api.solve_adjoint(self._h, linearized, self._field_in(pt), po),
                        "solve_adjoint")
        finally:
            self._keep = []
        return out

    def get_state(self, i, out=None):
        return self._indexed("get_state", self.api.get_state, i, out)

    def get_adjoint(self, i, out=None):
        return self._indexed("get_adjoint", self.api.get_adjoint, i, out)

    def _indexed(self, name, fn, i, out):
        self._keep = []
        try:
            out, po = self._field_out(out)
            self._check(fn(self._h, i, po), name)
        finally:
            self._keep = []
        return out

    def eval_objective(self, x, d1) -> float:
        self._touch()
        x = np.ascontiguousarray(x, dtype=np.float64)
        J = ctypes.c_double(0)
        self._keep = []
        try:
            self._check(self.api.eval_objective(self._h, _dptr(x), x.size, self._field_in(d1),
                                                ctypes.byref(J)), "eval_objective")
        finally:
            self._keep = []
        return J.value

    def eval_gradient(self, x, d1) -> np.ndarray:
        self._touch()
        x = np.ascontiguousarray(x, dtype=np.float64)
        dJ = np.zeros_like(x)
        self._keep = []
        try:
            self._check(self.api.eval_gradient(self._h, _dptr(x), x.size, self._field_in(d1),
                                               _dptr(dJ)), "eval_gradient")
        finally:
            self._keep = []
        return dJ

    def eval_objective_and_gradient(self, x, d1):
        self._touch()
        x = np.ascontiguousarray(x, dtype=np.float64)
        dJ = np.zeros_like(x)
        J = ctypes.c_double(0)
        self._keep = []
        try:
            self._check(self.api.eval_objective_and_gradient(
                self._h, _dptr(x), x.size, self._field_in(d1), ctypes.byref(J), _dptr(dJ)),
                "eval_objective_and_gradient")
        finally:
            self._keep = []
        return J.value, dJ

    def hessian_matvec(self, x):
        """Gauss-Newton matvec y = H x of the p block (DerivativeOperatorsRD::evaluateHessian),
        linearised at the last gradient evaluation or state solve."""
        self._touch()
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self._check(self.api.hessian_matvec(self._h, _dptr(x), x.size, _dptr(y)), "hessian_matvec")
        return y

    def stats(self) -> dict:
        st = _abi.GliaStats()
        self._check(self.api.get_stats(self._h, ctypes.byref(st)), "get_stats")
        return st.as_dict()

    def reset_stats(self):
        self._call("reset_stats", self.api.reset_stats)

    def set_launch_geometry(self, pointwise_blocks_per_sm: int, reduce_blocks_per_sm: int):
        self._call("set_launch_geometry", self.api.set_launch_geometry,
                   int(pointwise_blocks_per_sm), int(reduce_blocks_per_sm))

    def set_stream(self, stream_handle: int):
        self._call("set_stream", self.api.set_stream, ctypes.c_void_p(int(stream_handle)))
        self.stream = int(stream_handle)

    def set_timing(self, enable: bool):
        self._call("set_timing", self.api.set_timing, int(enable))

    def timing(self) -> dict:
        """Per-kernel {name: (launches, ms, algorithmic_bytes)} since timing was enabled."""
        out = {}
        slot, count = 0, 1
        while slot < count:
            name = ctypes.c_char_p()
            launches, ms, b = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
            rc = self.api.get_timing(self._h, slot, ctypes.byref(name), ctypes.byref(launches),
                                     ctypes.byref(ms), ctypes.byref(b))
            if rc < 0:
                self._check(rc, "get_timing")
            count = rc
            out[name.value.decode()] = (launches.value, ms.value, b.value)
            slot += 1
        return out

    def synchronize(self):
        self._call("synchronize", self.api.synchronize)

    def device_bytes(self) -> int:
        b = ctypes.c_int64(0)
        self._check(self.api.device_bytes(self._h, ctypes.byref(b)), "device_bytes")
        return b.value


def phi_mesh(api: _abi.Bound, np_: int, cm, sigma: float, spacing_factor: float) -> np.ndarray:
    """Phi::phiMesh lattice (src/mat/Phi.cpp:148-234) through the library's host helper."""
    cm = np.ascontiguousarray(cm, dtype=np.float64)
    out = np.zeros(3 * np_, dtype=np.float64)
    rc = api.phi_mesh(np_, _dptr(cm), sigma, spacing_factor, _dptr(out))
    if rc != _abi.GLIA_OK:
        raise GliaError(rc, "phi_mesh", "")
    return out.reshape(np_, 3)

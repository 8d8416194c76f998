"""ctypes binding of libhyperelastic_cuda.so (the C ABI declared in include/hyperelastic.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present, every call raises.
"""
import ctypes
import os

import numpy as np

from . import build as _build

HYP_OK = 0
HYP_ERR_INVALID = 1
HYP_ERR_CUDA = 2
HYP_ERR_NEG_DET = 3
HYP_ERR_NONFINITE = 4
HYP_ERR_TIMEOUT = 5
HYP_ERR_UNSUPPORTED = 6
HYP_ERR_NO_DEVICE = 7

HYP_MODEL_SINGLE, HYP_MODEL_MULTI = 1, 2
HYP_FLUX_RUSANOV, HYP_FLUX_LXF, HYP_FLUX_HLL = 0, 1, 2
HYP_BC_FROZEN, HYP_BC_TRANSMISSIVE = 0, 1
HYP_PREC_FP64, HYP_PREC_MIXED = 0, 1
HYP_RELAX_NONE, HYP_RELAX_PRESSURE, HYP_RELAX_MECHANICAL = 0, 1, 2
HYP_BATCH_NUM_VARIANTS = 3


class HypError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, code, msg, cell=-1):
        super().__init__(f"[{code}] {msg}")
        self.code, self.cell = code, cell


class NegativeDeterminantError(HypError, ValueError):
    """det(rho A) <= 0: the reference raises DomainError from sqrt (HyperelasticityMPh.jl:114)."""


class NonFiniteError(HypError, ArithmeticError):
    pass


class UnsupportedError(HypError, NotImplementedError):
    pass


_ERRS = {HYP_ERR_NEG_DET: NegativeDeterminantError, HYP_ERR_NONFINITE: NonFiniteError,
         HYP_ERR_UNSUPPORTED: UnsupportedError}
_NAMES = {HYP_ERR_INVALID: "invalid argument", HYP_ERR_CUDA: "CUDA error", HYP_ERR_NEG_DET: "det(rho A) <= 0",
          HYP_ERR_NONFINITE: "non-finite value", HYP_ERR_TIMEOUT: "device wait timed out",
          HYP_ERR_UNSUPPORTED: "unsupported option", HYP_ERR_NO_DEVICE: "no CUDA device"}


class Barton2009C(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("rho0", "c0", "cv", "t0", "b0", "alpha", "beta", "gamma")]


class Hank2016C(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("rho0", "mu", "gamma", "pres_inf", "a")]


class ConfigC(ctypes.Structure):
    _fields_ = [
        ("n_cells", ctypes.c_int64),
        ("model", ctypes.c_int),
        ("flux", ctypes.c_int),
        ("bc", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("x_length", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("eos", Barton2009C * 2),
    ]


_dp = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.c_int64
_SIGS = {
    "hyp_create": ([ctypes.POINTER(ConfigC), ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "hyp_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "hyp_last_error": ([ctypes.c_void_p], ctypes.c_char_p),
    "hyp_error_cell": ([ctypes.c_void_p], ctypes.c_int64),
    "hyp_upload": ([ctypes.c_void_p, _dp, _i64, ctypes.c_int, ctypes.c_double], ctypes.c_int),
    "hyp_download": ([ctypes.c_void_p, _dp, _i64, ctypes.c_int], ctypes.c_int),
    "hyp_step": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_int), _dp], ctypes.c_int),
    "hyp_set_eos": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Barton2009C)], ctypes.c_int),
    "hyp_step_times": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.POINTER(ctypes.c_int), _dp, _dp],
                       ctypes.c_int),
    "hyp_max_wavespeed": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "hyp_get_time": ([ctypes.c_void_p, _dp, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "hyp_set_profiling": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "hyp_last_timing": ([ctypes.c_void_p, _dp, _dp, ctypes.POINTER(ctypes.c_int), _dp, ctypes.POINTER(ctypes.c_int)],
                        ctypes.c_int),
    "hyp_set_mixed_kernel": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "hyp_set_wait_limit": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "hyp_step_noalloc_f64": ([ctypes.POINTER(ConfigC), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                              ctypes.c_double, ctypes.c_void_p, _dp, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "hyp_set_relaxation": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "hyp_eval_relax": ([ctypes.POINTER(ConfigC), ctypes.c_int, _dp, _dp, _i64], ctypes.c_int),
    "hyp_set_slab": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "hyp_slab_local_max": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "hyp_slab_step": ([ctypes.c_void_p, ctypes.c_double, _dp], ctypes.c_int),
    "hyp_cell_record_size": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "hyp_get_cells": ([ctypes.c_void_p, _i64, _i64, ctypes.c_void_p], ctypes.c_int),
    "hyp_set_cells": ([ctypes.c_void_p, _i64, _i64, ctypes.c_void_p], ctypes.c_int),
    "hyp_batch_create": ([ctypes.POINTER(ConfigC), ctypes.POINTER(ctypes.c_int64), ctypes.c_int,
                          ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "hyp_batch_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "hyp_batch_last_error": ([ctypes.c_void_p], ctypes.c_char_p),
    "hyp_batch_upload": ([ctypes.c_void_p, _dp, ctypes.c_double], ctypes.c_int),
    "hyp_batch_download": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "hyp_batch_step": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_double], ctypes.c_int),
    "hyp_batch_status": ([ctypes.c_void_p, _dp, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "hyp_batch_last_ms": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "hyp_batch_autotune": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), _dp], ctypes.c_int),
    "hyp_batch_set_variant": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "hyp_adjoint_record": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp], ctypes.c_int),
    "hyp_adjoint": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _dp], ctypes.c_int),
    "hyp_adjoint_timing": ([ctypes.c_void_p, _dp, _dp, _dp], ctypes.c_int),
    "hyp_density_misfit": ([ctypes.c_void_p, _dp, _dp, ctypes.c_void_p], ctypes.c_int),
    "hyp_snapshot": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "hyp_save_snapshot": ([ctypes.c_void_p, ctypes.c_char_p], ctypes.c_int),
    "hyp_load_snapshot": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_double], ctypes.c_int),
    "hyp_run_logged": ([ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, _i64,
                        ctypes.POINTER(ctypes.c_int), _dp], ctypes.c_int),
    "hyp_initial_states": ([ctypes.POINTER(ConfigC), ctypes.c_int, _dp, _dp], ctypes.c_int),
    "hyp_init_riemann": ([ctypes.c_void_p, _dp, _dp], ctypes.c_int),
    "hyp_init_tanh": ([ctypes.c_void_p, _dp, _dp, ctypes.c_double], ctypes.c_int),
    "hyp_measure_peaks": ([ctypes.c_int, _i64, _dp], ctypes.c_int),
    "hyp_measure_layouts": ([ctypes.c_int, _i64, _dp], ctypes.c_int),
    "hyp_host_alloc": ([ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "hyp_host_free": ([ctypes.c_void_p], ctypes.c_int),
    "hyp_eval_finger": ([_dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_invariants": ([_dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_energy": ([ctypes.POINTER(Barton2009C), _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_entropy": ([ctypes.POINTER(Barton2009C), _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_stress": ([ctypes.POINTER(Barton2009C), _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_acoustic": ([ctypes.POINTER(Barton2009C), _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_acoustic_dir": ([ctypes.POINTER(Barton2009C), _dp, _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_stress_den": ([ctypes.POINTER(Barton2009C), _dp, _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_acoustic_prim": ([ctypes.POINTER(Barton2009C), _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_hank2016_energy": ([ctypes.POINTER(Hank2016C), _dp, _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_hank2016_pressure": ([ctypes.POINTER(Hank2016C), _dp, _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_hank2016_stress": ([ctypes.POINTER(Hank2016C), _dp, _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_cons2prim": ([ctypes.POINTER(ConfigC), _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_prim2cons": ([ctypes.POINTER(ConfigC), _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_prim2cons_vjp": ([ctypes.POINTER(ConfigC), _dp, _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_flux": ([ctypes.POINTER(ConfigC), _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_eigvals": ([ctypes.POINTER(ConfigC), _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_eigvals_dir": ([ctypes.POINTER(ConfigC), _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_lxf": ([ctypes.POINTER(ConfigC), _dp, _dp, _dp, _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_noncons": ([ctypes.POINTER(ConfigC), _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_hll": ([ctypes.POINTER(ConfigC), _dp, _dp, _dp, _dp, _i64], ctypes.c_int),
    "hyp_eval_hll_eigvals": ([ctypes.POINTER(ConfigC), _dp, _dp, _dp, _dp, _dp, _dp, _i64], ctypes.c_int),
}

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load the library (building it first if it is absent). Raises if it cannot be built or loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"libhyperelastic_cuda.so not built ({path}); call hyperelasticsolver_gb300.build()")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (args, res) in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def exported_symbols():
    return list(_SIGS)


def check(rc, ctx=None, what=""):
    if rc == HYP_OK:
        return
    L = load()
    msg = L.hyp_last_error(ctx).decode() if ctx else ""
    cell = L.hyp_error_cell(ctx) if ctx else -1
    text = f"{what}: {_NAMES.get(rc, 'error')}" + (f" ({msg})" if msg else "")
    raise _ERRS.get(rc, HypError)(rc, text, cell)


def ptr(a):
    return a.ctypes.data_as(_dp)


def soa(x, k):
    """(n, k) or (k,) array -> contiguous SoA (k, n), n, single-item flag."""
    x = np.asarray(x, dtype=np.float64)
    single = x.ndim == 1
    x = x.reshape(-1, k)
    return np.ascontiguousarray(x.T), x.shape[0], single


def unsoa(buf, single):
    r = np.ascontiguousarray(buf.T)
    return r[0] if single else r


class PinnedArray:
    """A numpy view of page-locked host memory from hyp_host_alloc (freed by close())."""

    def __init__(self, shape):
        n = int(np.prod(shape))
        self._p = ctypes.c_void_p()
        check(load().hyp_host_alloc(n * 8, ctypes.byref(self._p)), what="hyp_host_alloc")
        buf = (ctypes.c_double * n).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=np.float64).reshape(shape)

    def close(self):
        if self._p:
            self.array = None
            load().hyp_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

"""The explicit time loop of main.jl:202-241 on the GPU (one context = one problem)."""
import ctypes
import glob
import math
import os

import numpy as np

from . import _lib as L
from . import _model as M

_MODELS = {"single": L.HYP_MODEL_SINGLE, "multi": L.HYP_MODEL_MULTI}
_FLUXES = {"rusanov": L.HYP_FLUX_RUSANOV, "lxf": L.HYP_FLUX_LXF, "hll": L.HYP_FLUX_HLL}
_BCS = {"frozen": L.HYP_BC_FROZEN, "transmissive": L.HYP_BC_TRANSMISSIVE}
_PRECS = {"fp64": L.HYP_PREC_FP64, "mixed": L.HYP_PREC_MIXED}


class Solver:
    """Device-resident solver state for one 1D problem.

    Parameters mirror the reference driver's globals (main.jl:133-152):
    eos (one Barton2009, or a pair for the two-phase model), nx, X, cfl, and
    the flux choice of main.jl:223-225. State arrays are SoA (nvar, nx)."""

    def __init__(self, eos, nx, model="single", flux="rusanov", bc="frozen", precision="fp64", X=1.0, cfl=0.5,
                 relax=None):
        self.model = _MODELS[model]
        self.nvar = M.nvar(self.model)
        self.nx = int(nx)
        self.cfg = M.config(eos, self.model, nx, _FLUXES[flux], _BCS[bc], _PRECS[precision], X, cfl)
        lib = L.load()
        h = ctypes.c_void_p()
        L.check(lib.hyp_create(self.cfg, ctypes.byref(h)), what="hyp_create")
        self._h = h
        if relax is not None:
            self.set_relaxation(relax)

    def set_relaxation(self, mode):
        """Two-phase relaxation after each step: "pressure", "mechanical" (velocity, then
        pressure), or None (the reference's model, the default). An extension: the
        reference has no relaxation terms."""
        m = {None: L.HYP_RELAX_NONE, "none": L.HYP_RELAX_NONE, "pressure": L.HYP_RELAX_PRESSURE,
             "mechanical": L.HYP_RELAX_MECHANICAL}[mode]
        L.check(L.load().hyp_set_relaxation(self._h, m), self._h, "hyp_set_relaxation")

    def close(self):
        if getattr(self, "_h", None):
            L.load().hyp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, Q, t0=0.0):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        if Q.shape != (self.nvar, self.nx):
            raise ValueError(f"state must be SoA {(self.nvar, self.nx)}, got {Q.shape}")
        L.check(L.load().hyp_upload(self._h, L.ptr(Q), self.nx, self.nvar, float(t0)), self._h, "hyp_upload")

    def download(self, out=None):
        out = np.empty((self.nvar, self.nx)) if out is None else out
        L.check(L.load().hyp_download(self._h, L.ptr(out), self.nx, self.nvar), self._h, "hyp_download")
        return out

    def step(self, max_steps=0, t_end=math.inf):
        """Advance like `while t < T` (main.jl:202); returns (steps taken, t)."""
        s = ctypes.c_int(0)
        t = ctypes.c_double(0.0)
        L.check(L.load().hyp_step(self._h, int(max_steps), float(t_end), ctypes.byref(s), ctypes.byref(t)),
                self._h, "hyp_step")
        return s.value, t.value

    def set_eos(self, eos, phase=0):
        """Replace the Barton2009 parameters of one phase (1: two-phase contexts only);
        the state and time are kept (the reference passes eos to every call, main.jl:134)."""
        c = eos.c()
        L.check(L.load().hyp_set_eos(self._h, int(phase), ctypes.byref(c)), self._h, "hyp_set_eos")
        self.cfg.eos[int(phase)] = c
        if self.model == L.HYP_MODEL_SINGLE:
            self.cfg.eos[1] = c

    def step_times(self, max_steps, t_end=math.inf):
        """step() that also returns the time and dt of every step taken (the Step / t /
        dt line main.jl:229-237 logs), read back once at the end: (t, dt) arrays."""
        t0 = self.time()[0]
        hist = np.empty(max(int(max_steps), 1))
        s = ctypes.c_int(0)
        t = ctypes.c_double(0.0)
        L.check(L.load().hyp_step_times(self._h, int(max_steps), float(t_end), ctypes.byref(s), ctypes.byref(t),
                                        L.ptr(hist)), self._h, "hyp_step_times")
        th = hist[:s.value].copy()
        return th, np.diff(np.concatenate(([t0], th)))

    def max_wavespeed(self):
        v = ctypes.c_double(0.0)
        L.check(L.load().hyp_max_wavespeed(self._h, ctypes.byref(v)), self._h, "hyp_max_wavespeed")
        return v.value

    def time(self):
        t = ctypes.c_double(0.0)
        s = ctypes.c_int64(0)
        L.check(L.load().hyp_get_time(self._h, ctypes.byref(t), ctypes.byref(s)), self._h, "hyp_get_time")
        return t.value, s.value

    MIXED_KERNELS = {"tile": 0, "tma": 1, "pair": 2}

    def set_mixed_kernel(self, kernel):
        """Mixed precision kernel family: "tile" (one block per tile, the single-phase
        default; two-phase: scalar FP32 faces), "tma" (single-phase: persistent,
        TMA-prefetched tiles) or "pair" (two cells -- two-phase: the two phases, the
        two-phase default -- in the lanes of packed FP32 pairs)."""
        if kernel not in self.MIXED_KERNELS:
            raise ValueError("kernel must be one of " + ", ".join(self.MIXED_KERNELS))
        L.check(L.load().hyp_set_mixed_kernel(self._h, self.MIXED_KERNELS[kernel]), self._h, "hyp_set_mixed_kernel")

    def set_wait_limit(self, tries):
        """Poll budget of the TMA kernel's device waits; 0 makes each wait time out at once."""
        L.check(L.load().hyp_set_wait_limit(self._h, int(tries)), self._h, "hyp_set_wait_limit")

    def set_profiling(self, on):
        L.check(L.load().hyp_set_profiling(self._h, int(bool(on))), self._h, "hyp_set_profiling")

    def timing(self):
        a, b, d = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        nc, nu = ctypes.c_int(), ctypes.c_int()
        L.check(L.load().hyp_last_timing(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(nc), ctypes.byref(d),
                                         ctypes.byref(nu)), self._h, "hyp_last_timing")
        return {"ms_total": a.value, "ms_cell": b.value, "n_cell": nc.value, "ms_update": d.value,
                "n_update": nu.value}

    # ---- initial conditions on the device (main.jl:99-123) ----
    def init_riemann(self, Ql, Qr):
        """initial_condition(Ql, Qr, nx) (main.jl:99-106) built on the device as the state at t = 0."""
        ql = np.ascontiguousarray(Ql, dtype=np.float64)
        qr = np.ascontiguousarray(Qr, dtype=np.float64)
        if ql.shape != (self.nvar,) or qr.shape != (self.nvar,):
            raise ValueError(f"states must have {self.nvar} values")
        L.check(L.load().hyp_init_riemann(self._h, L.ptr(ql), L.ptr(qr)), self._h, "hyp_init_riemann")

    def init_tanh(self, Ql, Qr, eps=0.2):
        """initial_condition_tanh(eos, Ql, Qr, nx, eps) (main.jl:110-123), two phases, on the device."""
        ql = np.ascontiguousarray(Ql, dtype=np.float64)
        qr = np.ascontiguousarray(Qr, dtype=np.float64)
        if ql.shape != (30,) or qr.shape != (30,):
            raise ValueError("two-phase states have 30 values")
        L.check(L.load().hyp_init_tanh(self._h, L.ptr(ql), L.ptr(qr), float(eps)), self._h, "hyp_init_tanh")

    # ---- snapshots and restart (main.jl:62-95, 174-198, 233-237) ----
    def snapshot(self):
        """Primitive states of the current state, (15 or 30, nx): per phase alpha, rho, u(3), S, A(9)."""
        cols = 15 if self.nvar == 14 else 30
        P = np.empty((cols, self.nx))
        L.check(L.load().hyp_snapshot(self._h, L.ptr(P)), self._h, "hyp_snapshot")
        return P

    def save_snapshot(self, path):
        """Write the current state as the reference's save_data file (tab-separated prims)."""
        L.check(L.load().hyp_save_snapshot(self._h, os.fsencode(path)), self._h, "hyp_save_snapshot")

    def load_snapshot(self, path, t0=0.0):
        """Make a save_data file's state the current state at time t0 (read_data + prim2cons)."""
        L.check(L.load().hyp_load_snapshot(self._h, os.fsencode(path), float(t0)), self._h, "hyp_load_snapshot")

    def run_logged(self, directory, t_end=math.inf, max_steps=0, log_freq=100, first_step=0):
        """The main.jl loop with logging: writes directory/sol_%06i.csv for the current state and
        after every step whose number is a multiple of log_freq. Returns (steps taken, t)."""
        sd = ctypes.c_int(0)
        t = ctypes.c_double(0.0)
        L.check(L.load().hyp_run_logged(self._h, float(t_end), int(max_steps), int(log_freq), os.fsencode(directory),
                                        int(first_step), ctypes.byref(sd), ctypes.byref(t)), self._h, "hyp_run_logged")
        return sd.value, t.value

    # ---- adjoint (single-phase FP64 Rusanov) ----
    def record(self, n_steps, ckpt_every=50):
        """n_steps steps (as step(n_steps)) that keep the state every ckpt_every
        steps for adjoint(); returns the new time."""
        t = ctypes.c_double(0.0)
        L.check(L.load().hyp_adjoint_record(self._h, int(n_steps), int(ckpt_every), ctypes.byref(t)), self._h,
                "hyp_adjoint_record")
        return t.value

    def adjoint(self, dQ_final):
        """Pullback of the recorded run: dL/dQ of its initial state (nvar, nx) and
        dL/d(b0sq, k0), from dL/dQ of the current (final) state."""
        g = np.ascontiguousarray(dQ_final, dtype=np.float64)
        if g.shape != (self.nvar, self.nx):
            raise ValueError(f"dQ_final must be SoA {(self.nvar, self.nx)}, got {g.shape}")
        out = np.empty((self.nvar, self.nx))
        de = np.zeros(2)
        L.check(L.load().hyp_adjoint(self._h, g.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p),
                                     L.ptr(de)), self._h, "hyp_adjoint")
        return out, de

    def adjoint_timing(self):
        a, b, d = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        L.check(L.load().hyp_adjoint_timing(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(d)), self._h,
                "hyp_adjoint_timing")
        return {"ms_record": a.value, "ms_recompute": b.value, "ms_adjoint": d.value}

    def density_misfit(self, target, grad=True):
        """L = 1/2 sum (rho_i - target_i)^2 of the current state (rho = sqrt(det(rho A)/rho0))
        and, with grad, dL/dQ (nvar, nx)."""
        tg = np.ascontiguousarray(target, dtype=np.float64)
        if tg.shape != (self.nx,):
            raise ValueError(f"target must have shape ({self.nx},)")
        loss = ctypes.c_double(0.0)
        g = np.empty((self.nvar, self.nx)) if grad else None
        L.check(L.load().hyp_density_misfit(self._h, L.ptr(tg), ctypes.byref(loss),
                                            g.ctypes.data_as(ctypes.c_void_p) if grad else None), self._h,
                "hyp_density_misfit")
        return (loss.value, g) if grad else loss.value


class Batch:
    """Many independent single-phase problems of uneven size, advanced together.

    `sizes` are the problems' cell counts; each problem lives on [0, X] with
    dx = X / N_p and its own CFL time step and time (main.jl:202-227 per problem).
    States are SoA (14, total) with problem p in columns offsets[p]:offsets[p+1]."""

    def __init__(self, eos, sizes, flux="rusanov", bc="frozen", precision="mixed", X=1.0, cfl=0.5):
        sizes = np.asarray(sizes, dtype=np.int64)
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.n_problems = len(sizes)
        self.total = int(self.offsets[-1])
        self.cfg = M.config(eos, L.HYP_MODEL_SINGLE, self.total, _FLUXES[flux], _BCS[bc], _PRECS[precision], X, cfl)
        h = ctypes.c_void_p()
        off = self.offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        rc = L.load().hyp_batch_create(self.cfg, off, self.n_problems, ctypes.byref(h))
        L.check(rc, what="hyp_batch_create")
        self._h = h

    def _check(self, rc, what):
        if rc != L.HYP_OK:
            msg = L.load().hyp_batch_last_error(self._h).decode()
            raise L._ERRS.get(rc, L.HypError)(rc, f"{what}: {L._NAMES.get(rc, 'error')} ({msg})")

    def close(self):
        if getattr(self, "_h", None):
            L.load().hyp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, Q, t0=0.0):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        if Q.shape != (14, self.total):
            raise ValueError(f"batch state must be SoA (14, {self.total})")
        self._check(L.load().hyp_batch_upload(self._h, L.ptr(Q), float(t0)), "hyp_batch_upload")

    def download(self, out=None):
        out = np.empty((14, self.total)) if out is None else out
        self._check(L.load().hyp_batch_download(self._h, L.ptr(out)), "hyp_batch_download")
        return out

    def step(self, n_steps, t_end=math.inf):
        self._check(L.load().hyp_batch_step(self._h, int(n_steps), float(t_end)), "hyp_batch_step")

    def status(self):
        t = np.empty(self.n_problems)
        s = np.empty(self.n_problems, dtype=np.int64)
        self._check(L.load().hyp_batch_status(self._h, L.ptr(t), s.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))),
                    "hyp_batch_status")
        return t, s

    def last_ms(self):
        v = ctypes.c_double()
        self._check(L.load().hyp_batch_last_ms(self._h, ctypes.byref(v)), "hyp_batch_last_ms")
        return v.value

    def autotune(self, trial_steps=10):
        chosen = ctypes.c_int(-1)
        ms = np.zeros(L.HYP_BATCH_NUM_VARIANTS)
        self._check(L.load().hyp_batch_autotune(self._h, int(trial_steps), ctypes.byref(chosen), L.ptr(ms)),
                    "hyp_batch_autotune")
        return chosen.value, ms

    def set_variant(self, v):
        self._check(L.load().hyp_batch_set_variant(self._h, int(v)), "hyp_batch_set_variant")

    def problem(self, Q, p):
        """Columns of problem p in a SoA batch state."""
        return Q[:, self.offsets[p]:self.offsets[p + 1]]


def last_snapshot(directory, dt, clean=False):
    """The restart point of main.jl:173-187: the last sol_*.csv in `directory`, its step
    number and the time step_number * dt; (path, step, t). None where the reference
    starts afresh: an empty directory, or one holding result.csv (a finished run),
    whose sol_*.csv and result.csv files are then removed if clean is true (the
    reference removes every file of its data directory)."""
    files = sorted(glob.glob(os.path.join(directory, "sol_*.csv")))
    result = os.path.join(directory, "result.csv")
    if os.path.exists(result):
        if clean:
            for f in files + [result]:
                os.remove(f)
        return None
    if not files:
        return None
    step = int(os.path.basename(files[-1]).split(".")[0].split("_")[1])
    return files[-1], step, step * dt

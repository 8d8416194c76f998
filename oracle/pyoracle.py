"""ctypes binding of the C++ oracle (test infrastructure only; see package docstring).

Every function takes and returns numpy arrays with one row per item
(shape ``(n, k)``); the C side is structure-of-arrays and the binding transposes.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libhyp_oracle.so")

MODEL_SINGLE, MODEL_MULTI = 1, 2
FLUX_RUSANOV, FLUX_LXF, FLUX_HLL = 0, 1, 2
BC_FROZEN, BC_TRANSMISSIVE = 0, 1


class Eos(ctypes.Structure):
    """Barton2009 primary parameters (EquationsOfState.jl:71-116)."""

    _fields_ = [(n, ctypes.c_double) for n in ("rho0", "c0", "cv", "t0", "b0", "alpha", "beta", "gamma")]


class Hank(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("rho0", "mu", "gamma", "pres_inf", "a")]


def hank2016(rho0=2.7, mu=26e9, gamma=3.4, pres_inf=21.5e9, a=0.5):
    return Hank(rho0, mu, gamma, pres_inf, a)


def _hank(fname, h, x, y, M, k_in, k_out):
    m, n, single = _soa(M, k_in)
    x, y = _vec(x, n), _vec(y, n)
    out = np.empty((k_out, n))
    getattr(lib(), fname)(ctypes.byref(h), _ptr(x), _ptr(y), _ptr(m), _ptr(out), n)
    return (out[0, 0] if single else out[0]) if k_out == 1 else _out(out, single)


def hank_energy(h, den, pres, G):
    return _hank("hyo_hank_energy", h, den, pres, G, 9, 1)


def hank_pressure(h, den, e_int, inv):
    return _hank("hyo_hank_pressure", h, den, e_int, inv, 3, 1)


def hank_stress(h, den, pres, F):
    return _hank("hyo_hank_stress", h, den, pres, F, 9, 9)


def barton2009(rho0=8.93, c0=4.6, cv=3.9e-4, t0=300.0, b0=2.1, alpha=1.0, beta=3.0, gamma=2.0):
    """Default arguments as the reference constructor (EquationsOfState.jl:90)."""
    return Eos(rho0, c0, cv, t0, b0, alpha, beta, gamma)


class Problem(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int),
        ("flux", ctypes.c_int),
        ("bc", ctypes.c_int),
        ("nx", ctypes.c_int),
        ("X", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("eos", Eos * 2),
        ("relax", ctypes.c_int),
    ]


def problem(model=MODEL_SINGLE, flux=FLUX_RUSANOV, bc=BC_FROZEN, nx=3, X=1.0, cfl=0.5, eos=None, relax=0):
    eos = eos if eos is not None else (barton2009(), barton2009())
    p = Problem()
    p.model, p.flux, p.bc, p.nx, p.X, p.cfl, p.relax = model, flux, bc, nx, X, cfl, relax
    p.eos[0] = eos[0]
    p.eos[1] = eos[1]
    return p


def build(quiet=True):
    """Compile the oracle with its Makefile (g++, OpenMP)."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        i64 = ctypes.c_int64
        ep = ctypes.POINTER(Eos)
        pp = ctypes.POINTER(Problem)
        sig = {
            "hyo_finger": [dp, dp, i64],
            "hyo_invariants": [dp, dp, i64],
            "hyo_energy": [ep, dp, dp, dp, i64],
            "hyo_entropy": [ep, dp, dp, dp, i64],
            "hyo_stress": [ep, dp, dp, dp, i64],
            "hyo_acoustic": [ep, dp, dp, dp, i64],
            "hyo_eig3_moduli": [dp, dp, i64],
            "hyo_eig3_sorted": [dp, dp, i64],
            "hyo_acoustic_dir": [ep, dp, dp, dp, dp, i64],
            "hyo_stress_den": [ep, dp, dp, dp, dp, i64],
            "hyo_acoustic_prim": [ep, dp, dp, dp, i64],
            "hyo_speeds_dir": [pp, dp, dp, dp, i64],
            "hyo_relax": [pp, dp, dp, ctypes.POINTER(ctypes.c_int), i64],
            "hyo_cons2prim": [pp, dp, dp, i64],
            "hyo_prim2cons": [pp, dp, dp, i64],
            "hyo_flux": [pp, dp, dp, i64],
            "hyo_speeds": [pp, dp, dp, i64],
            "hyo_noncons": [pp, dp, dp, i64],
            "hyo_lxf": [pp, dp, dp, dp, dp, dp, dp, i64],
            "hyo_hll": [pp, dp, dp, dp, dp, dp, dp, i64],
            "hyo_run": [pp, dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                        ctypes.POINTER(ctypes.c_int), dp, dp],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        L.hyo_run_dts.argtypes = [pp, dp, ctypes.c_int, dp, ctypes.c_int]
        L.hyo_run_dts.restype = ctypes.c_int
        L.hyo_quadrature.argtypes = [ctypes.c_int, dp, dp]
        L.hyo_quadrature.restype = None
        L.hyo_max_speed.argtypes = [pp, dp, ctypes.c_int]
        L.hyo_max_speed.restype = ctypes.c_double
        hp = ctypes.POINTER(Hank)
        for name in ("hyo_hank_energy", "hyo_hank_pressure", "hyo_hank_stress"):
            getattr(L, name).argtypes = [hp, dp, dp, dp, dp, ctypes.c_int64]
            getattr(L, name).restype = ctypes.c_int
        L.hyo_misfit_grad_dual.argtypes = [pp, dp, dp, ctypes.c_int, dp, ctypes.c_int, dp, dp]
        L.hyo_misfit_grad_dual.restype = ctypes.c_int
        _lib = L
    return _lib


def _soa(x, k):
    x = np.asarray(x, dtype=np.float64)
    single = x.ndim == 1
    x = x.reshape(-1, k)
    return np.ascontiguousarray(x.T), x.shape[0], single


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _out(buf, single):
    r = np.ascontiguousarray(buf.T)
    return r[0] if single else r


def _vec(x, n):
    x = np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (n,)))
    return x


def finger(A):
    a, n, s = _soa(A, 9)
    g = np.empty_like(a)
    lib().hyo_finger(_ptr(a), _ptr(g), n)
    return _out(g, s)


def invariants(G):
    g, n, s = _soa(G, 9)
    r = np.empty((3, n))
    lib().hyo_invariants(_ptr(g), _ptr(r), n)
    return _out(r, s)


def energy(eos, S, G):
    g, n, s = _soa(G, 9)
    S = _vec(S, n)
    r = np.empty((1, n))
    lib().hyo_energy(ctypes.byref(eos), _ptr(S), _ptr(g), _ptr(r), n)
    return r[0, 0] if s else r[0]


def entropy(eos, e, G):
    g, n, s = _soa(G, 9)
    e = _vec(e, n)
    r = np.empty((1, n))
    lib().hyo_entropy(ctypes.byref(eos), _ptr(e), _ptr(g), _ptr(r), n)
    return r[0, 0] if s else r[0]


def stress(eos, S, F):
    f, n, s = _soa(F, 9)
    S = _vec(S, n)
    r = np.empty((9, n))
    lib().hyo_stress(ctypes.byref(eos), _ptr(S), _ptr(f), _ptr(r), n)
    return _out(r, s)


def _dirs(d, n):
    """Directions as SoA [3][n] from one 3-vector or an (n, 3) array."""
    d = np.asarray(d, dtype=np.float64)
    d = np.broadcast_to(d.reshape(-1, 3), (n, 3)) if d.size == 3 else d.reshape(n, 3)
    return np.ascontiguousarray(d.T)


def acoustic(eos, S, F, n_dir=None):
    """Acoustic tensor (EquationsOfState.jl:223-246), column-major 9-vector; direction
    n = e1 by default, else one 3-vector or one per item."""
    f, n, s = _soa(F, 9)
    S = _vec(S, n)
    r = np.empty((9, n))
    if n_dir is None:
        lib().hyo_acoustic(ctypes.byref(eos), _ptr(S), _ptr(f), _ptr(r), n)
    else:
        lib().hyo_acoustic_dir(ctypes.byref(eos), _ptr(S), _ptr(f), _ptr(_dirs(n_dir, n)), _ptr(r), n)
    return _out(r, s)


def stress_den(eos, den, e_int, F):
    """stress(eos, den, e_int, F) (EquationsOfState.jl:162-176)."""
    f, n, s = _soa(F, 9)
    den, e_int = _vec(den, n), _vec(e_int, n)
    r = np.empty((9, n))
    lib().hyo_stress_den(ctypes.byref(eos), _ptr(den), _ptr(e_int), _ptr(f), _ptr(r), n)
    return _out(r, s)


def acoustic_prim(eos, P, n_dir):
    """acoustic(eos, P, n) (EquationsOfState.jl:192-221), P one phase's 15 primitives."""
    p, n, s = _soa(P, 15)
    r = np.empty((9, n))
    lib().hyo_acoustic_prim(ctypes.byref(eos), _ptr(p), _ptr(_dirs(n_dir, n)), _ptr(r), n)
    return _out(r, s)


def eig3_sorted(M):
    """Eigenvalue moduli in Julia's eigvals order (ascending real part)."""
    m, n, s = _soa(M, 9)
    r = np.empty((3, n))
    lib().hyo_eig3_sorted(_ptr(m), _ptr(r), n)
    return _out(r, s)


def eig3_moduli(M):
    m, n, s = _soa(M, 9)
    r = np.empty((3, n))
    lib().hyo_eig3_moduli(_ptr(m), _ptr(r), n)
    return _out(r, s)


def _model_call(fname, pb, Q, k_in, k_out):
    q, n, s = _soa(Q, k_in)
    r = np.empty((k_out, n))
    rc = getattr(lib(), fname)(ctypes.byref(pb), _ptr(q), _ptr(r), n)
    if rc != 0:
        raise ValueError(f"{fname} failed ({rc})")
    return _out(r, s)


def nvar(pb):
    return 14 if pb.model == MODEL_SINGLE else 30


def cons2prim(pb, Q):
    return _model_call("hyo_cons2prim", pb, Q, nvar(pb), nvar(pb))


def prim2cons(pb, P):
    return _model_call("hyo_prim2cons", pb, P, nvar(pb), nvar(pb))


def flux(pb, Q):
    return _model_call("hyo_flux", pb, Q, nvar(pb), nvar(pb))


def speeds(pb, Q, n_dir=None):
    """get_eigvals (HyperelasticityMPh.jl:252-266): n = e1 by default."""
    if n_dir is None:
        return _model_call("hyo_speeds", pb, Q, nvar(pb), 6 if pb.model == MODEL_SINGLE else 12)
    q, n, s = _soa(Q, nvar(pb))
    r = np.empty((6 if pb.model == MODEL_SINGLE else 12, n))
    lib().hyo_speeds_dir(ctypes.byref(pb), _ptr(q), _ptr(_dirs(n_dir, n)), _ptr(r), n)
    return _out(r, s)


def relax(pb, Q):
    """Two-phase pressure relaxation of cells (an extension; see hyp_oracle.hpp), the
    velocities relaxed first when pb.relax == 2.
    Returns (Q', status per cell: 0, or 8 when Newton did not converge)."""
    q, n, s = _soa(Q, 30)
    r = np.empty_like(q)
    st = np.zeros(n, dtype=np.int32)
    lib().hyo_relax(ctypes.byref(pb), _ptr(q), _ptr(r), st.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n)
    return _out(r, s), (st[0] if s else st)


def noncons(pb, Q):
    return _model_call("hyo_noncons", pb, Q, 30, 30)


def lxf(pb, Ql, Qr, lam):
    l, n, s = _soa(Ql, nvar(pb))
    r, _, _ = _soa(Qr, nvar(pb))
    lam = _vec(lam, n)
    c, m, p = (np.empty_like(l) for _ in range(3))
    lib().hyo_lxf(ctypes.byref(pb), _ptr(l), _ptr(r), _ptr(lam), _ptr(c), _ptr(m), _ptr(p), n)
    return _out(c, s), _out(m, s), _out(p, s)


def hll(pb, Ql, Qr, spdL, spdR):
    l, n, s = _soa(Ql, 30)
    r, _, _ = _soa(Qr, 30)
    sl, _, _ = _soa(spdL, 12)
    sr, _, _ = _soa(spdR, 12)
    m, p = np.empty_like(l), np.empty_like(l)
    lib().hyo_hll(ctypes.byref(pb), _ptr(l), _ptr(r), _ptr(sl), _ptr(sr), _ptr(m), _ptr(p), n)
    return _out(m, s), _out(p, s)


def quadrature(kind):
    """kind 0: Gauss-Legendre 6 on [0,1]; kind 1: Gauss-Lobatto 6 on [0,1]."""
    x, w = np.empty(6), np.empty(6)
    lib().hyo_quadrature(kind, _ptr(x), _ptr(w))
    return x, w


def max_speed(pb, Q_soa, nthreads=0):
    Q_soa = np.ascontiguousarray(Q_soa, dtype=np.float64)
    pb.nx = Q_soa.shape[1]
    return lib().hyo_max_speed(ctypes.byref(pb), _ptr(Q_soa), nthreads or os.cpu_count())


def run(pb, Q_soa, max_steps=0, t_end=float("inf"), t0=0.0, nthreads=0, literal=False):
    """Time loop of main.jl:202-227 on a SoA state ``(nvar, nx)``.

    Returns ``(Q, steps, t, dt_last)``; Q is a new array."""
    Q = np.array(Q_soa, dtype=np.float64, order="C", copy=True)
    pb.nx = Q.shape[1]
    steps = ctypes.c_int(0)
    t = ctypes.c_double(t0)
    dt = ctypes.c_double(0.0)
    rc = lib().hyo_run(ctypes.byref(pb), _ptr(Q), int(max_steps), float(t_end), int(nthreads or os.cpu_count()),
                       int(bool(literal)), ctypes.byref(steps), ctypes.byref(t), ctypes.byref(dt))
    if rc != 0:
        raise ValueError(f"hyo_run failed ({rc})")
    return Q, steps.value, t.value, dt.value


def run_dts(pb, Q_soa, dts, nthreads=0):
    """Advance with prescribed time steps (one per step). Returns a new SoA array."""
    Q = np.array(Q_soa, dtype=np.float64, order="C", copy=True)
    pb.nx = Q.shape[1]
    d = np.ascontiguousarray(dts, dtype=np.float64)
    rc = lib().hyo_run_dts(ctypes.byref(pb), _ptr(Q), len(d), _ptr(d), int(nthreads or os.cpu_count()))
    if rc != 0:
        raise ValueError(f"hyo_run_dts failed ({rc})")
    return Q


def misfit_grad_dual(pb, prim_left, prim_right, n_steps, target, nthreads=1):
    """Forward-mode (15 partials) value and gradient of L = 1/2 sum (rho_i - target_i)^2
    after n_steps of the single-phase two-state problem (cells i < nx/2 left), with
    respect to the left state (rho, u(3), A(9) column-major) and the moduli (b0sq, k0).
    Every scalar of the oracle run is a dual number, so the reference's nested-dual
    stress and acoustic tensor carry the outer partials too. Returns (L, grad(15))."""
    tg = np.ascontiguousarray(target, dtype=np.float64)
    pb.nx = len(tg)
    pl = np.ascontiguousarray(prim_left, dtype=np.float64)
    pr = np.ascontiguousarray(prim_right, dtype=np.float64)
    loss = np.zeros(1)
    g = np.zeros(15)
    rc = lib().hyo_misfit_grad_dual(ctypes.byref(pb), _ptr(pl), _ptr(pr), int(n_steps), _ptr(tg), int(nthreads),
                                    _ptr(loss), _ptr(g))
    if rc != 0:
        raise ValueError(f"hyo_misfit_grad_dual failed ({rc})")
    return loss[0], g

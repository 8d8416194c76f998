"""EquationsOfState mirror (reference: EquationsOfState.jl) over the GPU C ABI.

Functions accept one item (shape (9,)) or a batch (shape (n, 9)) and evaluate it
with the same device code as the solver step.
"""
import numpy as np

from . import _lib as L
from . import _model as M


class Barton2009:
    """Barton2009 EOS parameters (EquationsOfState.jl:71-116), same keyword names and defaults."""

    def __init__(self, _rho0=8.93, _c0=4.6, _cv=3.9e-4, _t0=300, _b0=2.1, _alpha=1, _beta=3, _gamma=2):
        self.rho0, self.c0, self.cv, self.t0 = float(_rho0), float(_c0), float(_cv), float(_t0)
        self.b0, self.alpha, self.beta, self.gamma = float(_b0), float(_alpha), float(_beta), float(_gamma)
        self.b0sq = self.b0 ** 2                               # :111
        self.k0 = self.c0 ** 2 - (4 / 3) * self.b0 ** 2        # :112

    def c(self):
        return L.Barton2009C(self.rho0, self.c0, self.cv, self.t0, self.b0, self.alpha, self.beta, self.gamma)

    def __repr__(self):
        return (f"Barton2009(rho0={self.rho0}, c0={self.c0}, cv={self.cv}, t0={self.t0}, b0={self.b0}, "
                f"alpha={self.alpha}, beta={self.beta}, gamma={self.gamma})")


class Hank2016:
    """Hank2016 EOS parameters (EquationsOfState.jl:305-326), same names and defaults.
    The reference defines energy, pressure and stress for it; its time step uses Barton2009."""

    def __init__(self, rho0=2.7, mu=26e9, gamma=3.4, pres_inf=21.5e9, a=0.5):
        self.rho0, self.mu, self.gamma, self.pres_inf, self.a = (float(v) for v in (rho0, mu, gamma, pres_inf, a))

    def c(self):
        return L.Hank2016C(self.rho0, self.mu, self.gamma, self.pres_inf, self.a)

    def __repr__(self):
        return f"Hank2016(rho0={self.rho0}, mu={self.mu}, gamma={self.gamma}, pres_inf={self.pres_inf}, a={self.a})"


EoS = Barton2009


def _scalar_vec(x, n):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), (n,)))


def _eval(fname, eos, s, M, k_out):
    m, n, single = L.soa(M, 9)
    s = _scalar_vec(s, n)
    out = np.empty((k_out, n))
    e = eos.c()
    L.check(getattr(L.load(), fname)(e, L.ptr(s), L.ptr(m), L.ptr(out), n), what=fname)
    if k_out == 1:
        return out[0, 0] if single else out[0]
    return L.unsoa(out, single)


def _eval_hank(fname, eos, x, y, M, k_in, k_out):
    m, n, single = L.soa(M, k_in)
    x, y = _scalar_vec(x, n), _scalar_vec(y, n)
    out = np.empty((k_out, n))
    L.check(getattr(L.load(), fname)(eos.c(), L.ptr(x), L.ptr(y), L.ptr(m), L.ptr(out), n), what=fname)
    if k_out == 1:
        return out[0, 0] if single else out[0]
    return L.unsoa(out, single)


def energy(eos, *args):
    """Internal energy: energy(eos::Barton2009, S, G) (EquationsOfState.jl:118-137) or
    energy(eos::Hank2016, den, pres, G) (EquationsOfState.jl:321-336)."""
    if isinstance(eos, Hank2016):
        den, pres, G = args
        return _eval_hank("hyp_eval_hank2016_energy", eos, den, pres, G, 9, 1)
    S, G = args
    return _eval("hyp_eval_energy", eos, S, G, 1)


def pressure(eos, den, e_int, i):
    """pressure(eos::Hank2016, den, e_int, i) (EquationsOfState.jl:338-352); i: invariants (3,) or (n, 3)."""
    if not isinstance(eos, Hank2016):
        raise NotImplementedError("the reference defines pressure for Hank2016 only")
    return _eval_hank("hyp_eval_hank2016_pressure", eos, den, e_int, i, 3, 1)


def entropy(eos, e_int, G):
    """Entropy from internal energy, argument clamped at 1e-6 (EquationsOfState.jl:139-156)."""
    return _eval("hyp_eval_entropy", eos, e_int, G, 1)


def stress(eos, *args):
    """Cauchy stress, column-major 9-vector (or (n, 9)), by the reference's methods:
    stress(eos::Barton2009, ent, F) = -2 rho G dE/dG, rho = rho0/det F
    (EquationsOfState.jl:179-190); stress(eos::Barton2009, den, e_int, F), the entropy from
    e_int and den as given (EquationsOfState.jl:162-176); stress(eos::Hank2016, den,
    pressure, distortion) = -2 den G dE/dG with G = finger(inv(F)) (EquationsOfState.jl:354-361)."""
    if isinstance(eos, Hank2016):
        den, pres, F = args
        return _eval_hank("hyp_eval_hank2016_stress", eos, den, pres, F, 9, 9)
    if len(args) == 3:
        den, e_int, F = args
        m, n, single = L.soa(F, 9)
        den, e_int = _scalar_vec(den, n), _scalar_vec(e_int, n)
        out = np.empty((9, n))
        L.check(L.load().hyp_eval_stress_den(eos.c(), L.ptr(den), L.ptr(e_int), L.ptr(m), L.ptr(out), n),
                what="hyp_eval_stress_den")
        return L.unsoa(out, single)
    ent, F = args
    return _eval("hyp_eval_stress", eos, ent, F, 9)


def _mat3(r):
    return r.reshape(3, 3, order="F") if r.ndim == 1 else r.reshape(-1, 3, 3).transpose(0, 2, 1)


def acoustic(eos, *args):
    """Acoustic tensor as a 3x3 matrix (or (m, 3, 3)), by the reference's methods:
    acoustic(eos, ent, F, n=[1,0,0]) (EquationsOfState.jl:223-246), the entropy held;
    acoustic(eos, P, n) with P one phase's primitives [alpha, rho, u(3), S, A(9)]
    (EquationsOfState.jl:192-221), the internal energy and alpha*rho held. n: one
    direction (3,) or one per item (m, 3)."""
    if len(args) == 2 and np.asarray(args[0]).shape[-1:] == (15,) and np.asarray(args[1]).shape[-1:] == (3,):
        P, n_dir = args
        p, n, single = L.soa(P, 15)
        out = np.empty((9, n))
        L.check(L.load().hyp_eval_acoustic_prim(eos.c(), L.ptr(p), L.ptr(M.dirs(n_dir, n)), L.ptr(out), n),
                what="hyp_eval_acoustic_prim")
        return _mat3(L.unsoa(out, single))
    ent, F = args[0], args[1]
    n_dir = args[2] if len(args) > 2 else (1, 0, 0)
    if M.is_e1(n_dir):
        return _mat3(_eval("hyp_eval_acoustic", eos, ent, F, 9))
    m, n, single = L.soa(F, 9)
    ent = _scalar_vec(ent, n)
    out = np.empty((9, n))
    L.check(L.load().hyp_eval_acoustic_dir(eos.c(), L.ptr(ent), L.ptr(m), L.ptr(M.dirs(n_dir, n)), L.ptr(out), n),
            what="hyp_eval_acoustic_dir")
    return _mat3(L.unsoa(out, single))

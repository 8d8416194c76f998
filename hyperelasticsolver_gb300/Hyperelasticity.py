"""Single-phase model over the GPU C ABI: 14 values per cell (rho, rho u(3), rho E, rho A(9)).

The reference's single-phase module (Hyperelasticity.jl) does not run against its
current EOS API; its solver restates single-phase hyperelasticity as the per-phase
functions of HyperelasticityMPh.jl with volume fraction alpha == 1, which is what
these functions evaluate. Primitive layout: (rho, u(3), S, A(9)).
"""
import numpy as np

from . import _lib as L
from . import _model as M


def _cfg(eos):
    return M.config(eos, L.HYP_MODEL_SINGLE)


def prim2cons(eos, P):
    """(rho, u, S, A) -> (rho, rho u, rho E, rho A) (HyperelasticityMPh.jl:66-87 at alpha = 1)."""
    return M.call("hyp_eval_prim2cons", _cfg(eos), P, 14, 14)


def prim2cons_vjp(eos, P, Qbar):
    """Pullback of prim2cons: ((dQ/dP)^T Qbar per state, sum over states of (dL/d b0sq, dL/d k0))."""
    p, n, single = L.soa(P, 14)
    qb, n2, _ = L.soa(Qbar, 14)
    if n2 != n:
        raise ValueError("P and Qbar hold different numbers of states")
    pb = np.empty((14, n))
    eb = np.zeros(2)
    L.check(L.load().hyp_eval_prim2cons_vjp(_cfg(eos), L.ptr(p), L.ptr(qb), L.ptr(pb), L.ptr(eb), n),
            what="hyp_eval_prim2cons_vjp")
    return L.unsoa(pb, single), eb


def cons2prim(eos, Q):
    """(HyperelasticityMPh.jl:106-133 at alpha = 1); rho = sqrt(det(rho A)/rho0)."""
    return M.call("hyp_eval_cons2prim", _cfg(eos), Q, 14, 14)


def flux(eos, Q):
    """Physical x-flux (HyperelasticityMPh.jl:146-175 at alpha = 1)."""
    return M.call("hyp_eval_flux", _cfg(eos), Q, 14, 14)


def get_eigvals(eos, Q, n=(1, 0, 0)):
    """u.n + sqrt|mu_k| then u.n - sqrt|mu_k| (HyperelasticityMPh.jl:258-266), 6 speeds, mu_k
    the eigenvalues of acoustic(eos, S, A, n) in Julia's eigvals order (ascending real
    part). n: one direction (3,) or one per state (m, 3)."""
    return M.eigvals_call(_cfg(eos), Q, 14, 6, n)

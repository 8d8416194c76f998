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


# ---- the 13-value layout of the reference's single-phase module ------------
# Hyperelasticity.jl:25-114 stores a cell as 13 values: rho u (3), rho F row-major
# (Q[3i + j] = rho F[i, j], 1-based, :82-86), rho E; its density is
# sqrt(det(rho F) / rho0) (EquationsOfState.jl:259-264). That module calls EOS methods
# the reference no longer defines (density and stress without the eos argument), so it
# cannot run there; these functions give its names a working form, with the eos passed
# in, by converting to the 14-value layout above and back.
_ROW_TO_COL = np.array([3 * (k % 3) + k // 3 for k in range(9)])  # col-major slot c <- row-major slot


def q13_to_q14(eos, Q13):
    """(n, 13) or (13,) -> (n, 14): rho = sqrt(det(rho F)/rho0) prepended, rho F column-major."""
    q = np.atleast_2d(np.asarray(Q13, dtype=np.float64))
    rF_row = q[:, 3:12]
    rF = rF_row.reshape(-1, 3, 3)  # [i][j] = rho F[i, j]
    den = np.sqrt(np.linalg.det(rF) / eos.rho0)
    out = np.empty((q.shape[0], 14))
    out[:, 0] = den
    out[:, 1:4] = q[:, 0:3]
    out[:, 4] = q[:, 12]
    out[:, 5:14] = rF_row[:, _ROW_TO_COL]
    return out[0] if np.ndim(Q13) == 1 else out


def q14_to_q13(Q14):
    """(n, 14) or (14,) -> (n, 13): rho dropped, rho A written row-major."""
    q = np.atleast_2d(np.asarray(Q14, dtype=np.float64))
    out = np.empty((q.shape[0], 13))
    out[:, 0:3] = q[:, 1:4]
    out[:, 3:12][:, _ROW_TO_COL] = q[:, 5:14]
    out[:, 12] = q[:, 4]
    return out[0] if np.ndim(Q14) == 1 else out


def cons2prim13(eos, Q13):
    """cons2prim of Hyperelasticity.jl:25-36 with the eos: (den, vel (n, 3), F (n, 3, 3), e_int)."""
    q14 = np.atleast_2d(q13_to_q14(eos, Q13))
    den = q14[:, 0]
    vel = q14[:, 1:4] / den[:, None]
    F = (q14[:, 5:14] / den[:, None]).reshape(-1, 3, 3).transpose(0, 2, 1)
    e_int = q14[:, 4] / den - 0.5 * np.sum(vel * vel, axis=1)
    if np.ndim(Q13) == 1:
        return den[0], vel[0], F[0], e_int[0]
    return den, vel, F, e_int


def prim2cons13(eos, vel, F, S):
    """prim2cons of Hyperelasticity.jl:70-93 with the eos: vel (3,) / (n, 3), F (3, 3) / (n, 3, 3), S."""
    single = np.ndim(vel) == 1
    vel = np.atleast_2d(np.asarray(vel, dtype=np.float64))
    F = np.asarray(F, dtype=np.float64).reshape(-1, 3, 3)
    S = np.broadcast_to(np.asarray(S, dtype=np.float64), (F.shape[0],))
    P = np.empty((F.shape[0], 14))
    P[:, 0] = eos.rho0 / np.linalg.det(F)  # :78
    P[:, 1:4] = vel
    P[:, 4] = S
    P[:, 5:14] = F.transpose(0, 2, 1).reshape(-1, 9)  # column-major
    out = q14_to_q13(prim2cons(eos, P))
    return out[0] if single else out


def flux13(eos, Q13):
    """flux of Hyperelasticity.jl:99-114 with the eos, 13 values: the rho F rows follow the
    14-value flux (row 1 identically zero, :106), energy last."""
    f14 = np.atleast_2d(flux(eos, np.atleast_2d(q13_to_q14(eos, Q13))))
    out = q14_to_q13(f14)
    return out[0] if np.ndim(Q13) == 1 else out

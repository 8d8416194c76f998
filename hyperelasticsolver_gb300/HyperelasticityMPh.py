"""HyperelasticityMPh mirror (reference: HyperelasticityMPh.jl): two-phase model, 30 values per cell.

`eos` is a pair of Barton2009 (main.jl:134). Inputs are one cell (shape (30,)) or a batch (n, 30).
"""
import numpy as np

from . import _lib as L
from . import _model as M


def _cfg(eos):
    return M.config(eos, L.HYP_MODEL_MULTI)


def prim2cons_mph(eos, P):
    """Primitive [alpha, rho, u(3), S, A(9)] x 2 -> conservative (HyperelasticityMPh.jl:63-90)."""
    return M.call("hyp_eval_prim2cons", _cfg(eos), P, 30, 30)


def cons2prim_mph(eos, Q):
    """Conservative -> primitive; density from det(alpha rho A) (HyperelasticityMPh.jl:99-133)."""
    return M.call("hyp_eval_cons2prim", _cfg(eos), Q, 30, 30)


def flux_mph(eos, Q):
    """Physical x-flux of both phases (HyperelasticityMPh.jl:140-175)."""
    return M.call("hyp_eval_flux", _cfg(eos), Q, 30, 30)


def get_eigvals(eos, Q, n=(1, 0, 0)):
    """Wave speeds u.n +- sqrt|eig(acoustic)| of both phases (HyperelasticityMPh.jl:252-266):
    per phase the three u.n + c_k, then the three u.n - c_k, in Julia's eigvals order
    (ascending real part of the eigenvalue). n: one direction (3,) or one per state."""
    return M.eigvals_call(_cfg(eos), Q, 30, 12, n)


def noncons_flux(eos, Q):
    """Non-conservative matrix B(Q), 30x30 (HyperelasticityMPh.jl:178-250): only column 1
    (phase-1 rows) and column 16 (phase-2 rows) are non-zero. Returns (30, 30) or (n, 30, 30)."""
    bcol = M.call("hyp_eval_noncons", _cfg(eos), Q, 30, 30)
    b = np.atleast_2d(bcol)
    B = np.zeros((b.shape[0], 30, 30))
    B[:, :15, 0] = b[:, :15]
    B[:, 15:, 15] = b[:, 15:]
    return B[0] if bcol.ndim == 1 else B


def initial_states(eos, testcase):
    """Left/right conservative states of the Riemann test cases 1-7 and 10
    (HyperelasticityMPh.jl:275-426), built by hyp_initial_states."""
    Ql, Qr = np.empty(30), np.empty(30)
    L.check(L.load().hyp_initial_states(_cfg(eos), int(testcase), L.ptr(Ql), L.ptr(Qr)),
            what=f"initial_states({testcase})")
    return Ql, Qr


def relax_pressure(eos, Q, velocity=False):
    """Instantaneous pressure relaxation of two-phase cells (hyp_eval_relax): volume
    fractions moved until both phases' mean-stress pressures agree, energies by
    de = -p* dv, distortions scaled in their volumetric part; velocity=True relaxes the
    velocities to the mixture velocity first. An extension (the reference has no
    relaxation terms); cells with a phase below 1e-5 come back as they are, a cell whose
    Newton iteration does not converge as NaN."""
    x, n, single = L.soa(Q, 30)
    out = np.empty((30, n))
    mode = L.HYP_RELAX_MECHANICAL if velocity else L.HYP_RELAX_PRESSURE
    L.check(L.load().hyp_eval_relax(_cfg(eos), mode, L.ptr(x), L.ptr(out), n), what="hyp_eval_relax")
    return L.unsoa(out, single)

"""NumFluxes mirror (reference: NumFluxes.jl) over the GPU C ABI."""
import numpy as np

from . import _lib as L
from . import _model as M


def hll(eos, Q_l, Q_r, eigvals=None):
    """Two-phase path-conservative HLL (NumFluxes.jl:70-132): returns (zeros(30), D-, D+).

    eigvals = [eig_l, eig_r], each 12 speeds (or (n, 12)): s_l = min(0, min speed of the
    face midpoint, minimum(eig_l)) and s_r = max(0, max speed of the midpoint,
    maximum(eig_r)) (NumFluxes.jl:90-91), as the reference uses them. main.jl:225 passes
    the two cells' own get_eigvals; eigvals=None computes exactly those."""
    cfg = M.config(eos, L.HYP_MODEL_MULTI, flux=L.HYP_FLUX_HLL)
    l, n, single = L.soa(Q_l, 30)
    r, _, _ = L.soa(Q_r, 30)
    dm, dp = np.empty((30, n)), np.empty((30, n))
    if eigvals is None:
        L.check(L.load().hyp_eval_hll(cfg, L.ptr(l), L.ptr(r), L.ptr(dm), L.ptr(dp), n), what="hll")
    else:
        el, n_l, _ = L.soa(eigvals[0], 12)
        er, n_r, _ = L.soa(eigvals[1], 12)
        if n_l != n or n_r != n:
            raise ValueError("eigvals must hold 12 speeds per face for each side")
        L.check(L.load().hyp_eval_hll_eigvals(cfg, L.ptr(l), L.ptr(r), L.ptr(el), L.ptr(er), L.ptr(dm), L.ptr(dp), n),
                what="hll")
    zero = np.zeros(30) if single else np.zeros((n, 30))
    return zero, L.unsoa(dm, single), L.unsoa(dp, single)


def lxf(eos, Q_l, Q_r, lam):
    """Lax-Friedrichs / Rusanov face flux (NumFluxes.jl:25-60).

    Returns (cons, D-, D+): cons = 0.5 (f(Q_l) + f(Q_r)) - 0.5 lam (Q_r - Q_l). `eos` a
    Barton2009 selects the single-phase model (14 values), whose path-conservative parts
    are zero; a pair of them the two-phase model (30 values), with D- = D+ = half the
    6-point Gauss-Lobatto path integral of the non-conservative matrix."""
    two = isinstance(eos, (tuple, list))
    nv = 30 if two else 14
    cfg = M.config(eos, L.HYP_MODEL_MULTI if two else L.HYP_MODEL_SINGLE,
                   flux=L.HYP_FLUX_LXF) if two else M.config(eos, L.HYP_MODEL_SINGLE)
    l, n, single = L.soa(Q_l, nv)
    r, _, _ = L.soa(Q_r, nv)
    lam = np.ascontiguousarray(np.broadcast_to(np.asarray(lam, dtype=np.float64), (n,)))
    cons, dm, dp = (np.empty((nv, n)) for _ in range(3))
    L.check(L.load().hyp_eval_lxf(cfg, L.ptr(l), L.ptr(r), L.ptr(lam), L.ptr(cons), L.ptr(dm), L.ptr(dp), n),
            what="lxf")
    return L.unsoa(cons, single), L.unsoa(dm, single), L.unsoa(dp, single)

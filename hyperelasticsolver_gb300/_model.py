"""Shared helpers of the model-level mirrors: config structs and batched calls."""
import numpy as np

from . import _lib as L


def config(eos, model, n_cells=3, flux=L.HYP_FLUX_RUSANOV, bc=L.HYP_BC_FROZEN, precision=L.HYP_PREC_FP64,
           x_length=1.0, cfl=0.5):
    """Build a ConfigC. `eos` is one Barton2009 (single phase) or a pair (two phases, main.jl:134)."""
    pair = eos if isinstance(eos, (tuple, list)) else (eos, eos)
    c = L.ConfigC()
    c.n_cells, c.model, c.flux, c.bc, c.precision = int(n_cells), model, flux, bc, precision
    c.x_length, c.cfl = float(x_length), float(cfl)
    c.eos[0] = pair[0].c()
    c.eos[1] = pair[1].c()
    return c


def nvar(model):
    return 14 if model == L.HYP_MODEL_SINGLE else 30


def call(fname, cfg, X, k_in, k_out):
    x, n, single = L.soa(X, k_in)
    out = np.empty((k_out, n))
    L.check(getattr(L.load(), fname)(cfg, L.ptr(x), L.ptr(out), n), what=fname)
    return L.unsoa(out, single)


def dirs(d, n):
    """Directions as SoA [3][n] from one 3-vector or an (n, 3) array."""
    d = np.asarray(d, dtype=np.float64)
    d = np.broadcast_to(d.reshape(1, 3), (n, 3)) if d.size == 3 else d.reshape(n, 3)
    return np.ascontiguousarray(d.T)


def is_e1(d):
    d = np.asarray(d, dtype=np.float64)
    return d.size == 3 and bool(np.all(d.reshape(3) == (1.0, 0.0, 0.0)))


def eigvals_call(cfg, Q, nv, ns, n_dir):
    """get_eigvals over states Q along n_dir (one 3-vector or one per state)."""
    if is_e1(n_dir):
        return call("hyp_eval_eigvals", cfg, Q, nv, ns)
    q, n, single = L.soa(Q, nv)
    out = np.empty((ns, n))
    L.check(L.load().hyp_eval_eigvals_dir(cfg, L.ptr(q), L.ptr(dirs(n_dir, n)), L.ptr(out), n),
            what="hyp_eval_eigvals_dir")
    return L.unsoa(out, single)

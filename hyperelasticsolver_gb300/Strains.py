"""Strains mirror (reference: Strains.jl) over the GPU C ABI."""
import numpy as np

from . import _lib as L


def finger(a):
    """Finger tensor G = inv(A A^T) of a column-major 9-vector (Strains.jl:26-32)."""
    x, n, single = L.soa(a, 9)
    out = np.empty_like(x)
    L.check(L.load().hyp_eval_finger(L.ptr(x), L.ptr(out), n), what="finger")
    return L.unsoa(out, single)


def invariants(g):
    """(tr G, (tr(G)^2 - tr(G^2))/2, det G) (Strains.jl:46-52)."""
    x, n, single = L.soa(g, 9)
    out = np.empty((3, n))
    L.check(L.load().hyp_eval_invariants(L.ptr(x), L.ptr(out), n), what="invariants")
    return L.unsoa(out, single)

"""Mirror symmetry at full size, a size-independent parity property: the step is
built from operations that commute with x -> -x (reverse the cells, negate rho u1
and the entries of rho A with exactly one index along x), so the run of the
mirrored state is the mirror of the run, bitwise: IEEE negation, fused
multiply-add and round-to-nearest are sign-symmetric, each face is evaluated with
one rounding sequence, and the max picks the same value. Checked on the 64-segment
workload up to 2^24 cells, FP64 and mixed precision, frozen and transmissive ends;
the two-phase step at 2^22 cells to rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLIP = [1, 6, 7, 8, 11]  # rho u1; rho A (1,0), (2,0), (0,1), (0,2) column-major


def mirror(Q):
    M = Q[:, ::-1].copy()
    M[FLIP] *= -1.0
    return np.ascontiguousarray(M)


@pytest.mark.parametrize("precision,bc,n,kernel", [("fp64", "frozen", 1 << 20, None),
                                                   ("mixed", "frozen", 1 << 24, "tile"),
                                                   ("mixed", "transmissive", 1 << 20, "tile"),
                                                   ("mixed", "frozen", 1 << 22, "pair"),
                                                   ("fp64", "transmissive", 4097, None)])
def test_mirrored_run_is_the_mirror_of_the_run(hyp, precision, bc, n, kernel):
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    eos = hyp.Barton2009()
    Q0 = segment_fill(H.prim2cons(eos, segment_states(eos, 64)), n)
    out = []
    for q in (Q0, mirror(Q0)):
        with hyp.Solver(eos, n, precision=precision, bc=bc) as s:
            if kernel:
                s.set_mixed_kernel(kernel)
            s.upload(q)
            k, t = s.step(max_steps=40)
            out.append((s.download(), t))
    (Qa, ta), (Qb, tb) = out
    assert ta == tb
    d = np.abs(mirror(Qa) - Qb)
    scale = np.maximum(np.max(np.abs(Qa), axis=1, keepdims=True), 1e-30)
    print(f"mirror {precision} {kernel} {bc} {n}: max rel {np.max(d / scale):.1e}, bitwise {np.array_equal(mirror(Qa), Qb)}")
    assert np.array_equal(mirror(Qa), Qb)


FLIP2 = [2, 7, 8, 9, 12]  # per phase: alpha rho u1; alpha rho A (1,0), (2,0), (0,1), (0,2)


def mirror2(Q):
    M = Q[:, ::-1].copy()
    M[FLIP2 + [k + 15 for k in FLIP2]] *= -1.0
    return np.ascontiguousarray(M)


# observed: FP64 3.4e-15; mixed 1.7e-7 (HLL) and 6.8e-7 (LxF) of each variable's scale
@pytest.mark.parametrize("precision,flux,tol,kernel", [("fp64", "hll", 1e-13, None), ("mixed", "hll", 5e-6, "tile"),
                                                       ("mixed", "lxf", 5e-6, "tile"), ("mixed", "hll", 5e-6, "pair"),
                                                       ("mixed", "lxf", 5e-6, "pair")])
def test_twophase_mirrored_run_at_full_size(hyp, precision, flux, tol, kernel):
    """The two-phase step at the 2^22-cell interface workload also commutes with
    x -> -x, to rounding rather than bitwise: the HLL state Q_hll = (s_R Q_R - s_L Q_L
    - ...)/(s_R - s_L) and the path integrals evaluate their mirrored operands in a
    different order, so multiply-add contraction can differ in the last bit."""
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    eos = (hyp.Barton2009(), hyp.Barton2009(_b0=2.1 * np.sqrt(0.1)))
    n = 1 << 22
    Q0 = np.ascontiguousarray(HM.prim2cons_mph(eos, mph_interface_prims(eos[0], n)).T)
    out = []
    for q in (Q0, mirror2(Q0)):
        with hyp.Solver(eos, n, model="multi", flux=flux, precision=precision) as s:
            if kernel:
                s.set_mixed_kernel(kernel)
            s.upload(q)
            k, t = s.step(max_steps=40)
            assert k == 40
            out.append((s.download(), t))
    (Qa, ta), (Qb, tb) = out
    # mixed: each step's dt comes from an FP32 max wave speed, itself mirrored only to rounding
    assert abs(ta - tb) <= (1e-14 if precision == "fp64" else 1e-6) * ta
    scale = np.maximum(np.max(np.abs(Qa), axis=1, keepdims=True), 1e-30)
    err = np.max(np.abs(mirror2(Qa) - Qb) / scale)
    print(f"two-phase mirror {precision} {kernel} {flux} 2^22: max rel {err:.1e}")
    assert err <= tol

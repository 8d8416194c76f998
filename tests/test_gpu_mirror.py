"""Mirror symmetry at full size, a size-independent parity property: the step is
built from operations that commute with x -> -x (reverse the cells, negate rho u1
and the entries of rho A with exactly one index along x), so the run of the
mirrored state is the mirror of the run, bitwise: IEEE negation, fused
multiply-add and round-to-nearest are sign-symmetric, each face is evaluated with
one rounding sequence, and the max picks the same value. Checked on the 64-segment
workload up to 2^24 cells, FP64 and mixed precision, frozen and transmissive ends."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLIP = [1, 6, 7, 8, 11]  # rho u1; rho A (1,0), (2,0), (0,1), (0,2) column-major


def mirror(Q):
    M = Q[:, ::-1].copy()
    M[FLIP] *= -1.0
    return np.ascontiguousarray(M)


@pytest.mark.parametrize("precision,bc,n", [("fp64", "frozen", 1 << 20), ("mixed", "frozen", 1 << 24),
                                            ("mixed", "transmissive", 1 << 20), ("fp64", "transmissive", 4097)])
def test_mirrored_run_is_the_mirror_of_the_run(hyp, precision, bc, n):
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    eos = hyp.Barton2009()
    Q0 = segment_fill(H.prim2cons(eos, segment_states(eos, 64)), n)
    out = []
    for q in (Q0, mirror(Q0)):
        with hyp.Solver(eos, n, precision=precision, bc=bc) as s:
            s.upload(q)
            k, t = s.step(max_steps=40)
            out.append((s.download(), t))
    (Qa, ta), (Qb, tb) = out
    assert ta == tb
    d = np.abs(mirror(Qa) - Qb)
    scale = np.maximum(np.max(np.abs(Qa), axis=1, keepdims=True), 1e-30)
    print(f"mirror {precision} {bc} {n}: max rel {np.max(d / scale):.1e}, bitwise {np.array_equal(mirror(Qa), Qb)}")
    assert np.array_equal(mirror(Qa), Qb)

"""The smallest problems of every stepping path (GPU): three to five cells (the C ABI
takes at least three, the reference's two frozen ends and one interior cell,
main.jl:219-221), where every face is a boundary face or next to one, against the
oracle (FP64) or the FP64 step (mixed precision). Fewer cells are refused before
any device work (tests/test_capi_abi.py)."""
import numpy as np
import pytest

from helpers import RTOL_FP64, assert_close_soa

pytestmark = pytest.mark.gpu

MIXED_REL = 1e-6  # mixed-precision step against the FP64 step, per variable, relative to its scale
# two phases: the FP32 interface terms across a full-strength jump (test case 7 on three
# to five cells, so every face carries the jump) give ~1e-6 of a variable's scale
MIXED_REL_JUMP = 1e-5


def riemann_1ph(orc, nx, flux, bc):
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300._cases import riemann_1ph as states, initial_condition
    pb = orc.problem(nx=nx, cfl=0.5, flux=orc.FLUX_LXF if flux == "lxf" else orc.FLUX_RUSANOV,
                     bc=orc.BC_TRANSMISSIVE if bc == "transmissive" else orc.BC_FROZEN)
    Pl, Pr = states(h.Barton2009())
    return initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx), pb


def scaled_err(a, b):
    """Per-variable max |a - b| relative to the variable's largest magnitude."""
    scale = np.maximum(np.max(np.abs(b), axis=1, keepdims=True), 1e-30)
    return np.max(np.abs(a - b) / scale, axis=1)


def close_to_scale(a, b, rel):
    e = scaled_err(a, b)
    print("per-variable scaled error", np.array2string(e, precision=1, max_line_width=400))
    return float(np.max(e)) <= rel


@pytest.mark.parametrize("bc", ["frozen", "transmissive"])
@pytest.mark.parametrize("flux", ["rusanov", "lxf"])
@pytest.mark.parametrize("nx", [3, 4, 5])
def test_single_phase_fp64_tiny(hyp, orc, nx, flux, bc):
    Q0, pb = riemann_1ph(orc, nx, flux, bc)
    Qo, so, to, _ = orc.run(pb, Q0, max_steps=6)
    with hyp.Solver(hyp.Barton2009(), nx, flux=flux, bc=bc, cfl=0.5) as s:
        s.upload(Q0)
        n, t = s.step(max_steps=6)
        assert n == 6 and abs(t - to) <= RTOL_FP64 * to
        Q = s.download()
    assert_close_soa(Q, Qo, RTOL_FP64, f"{flux}/{bc}/N={nx}")
    if bc == "frozen":
        assert np.array_equal(Q[:, [0, -1]], Q0[:, [0, -1]])


@pytest.mark.parametrize("bc", ["frozen", "transmissive"])
@pytest.mark.parametrize("nx", [3, 4, 5])
def test_single_phase_mixed_tiny(hyp, orc, nx, bc):
    Q0, _ = riemann_1ph(orc, nx, "rusanov", bc)
    out = {}
    for prec in ("fp64", "mixed"):
        with hyp.Solver(hyp.Barton2009(), nx, bc=bc, precision=prec, cfl=0.5) as s:
            s.upload(Q0)
            n, t = s.step(max_steps=6)
            assert n == 6
            out[prec] = (s.download(), t)
    assert abs(out["mixed"][1] - out["fp64"][1]) <= 1e-6 * out["fp64"][1]
    assert close_to_scale(out["mixed"][0], out["fp64"][0], MIXED_REL)


def oracle_pb2(orc, nx, flux):
    from test_gpu_mph import oracle_pb
    return oracle_pb(orc, nx=nx, cfl=0.5, flux=orc.FLUX_LXF if flux == "lxf" else orc.FLUX_HLL)


@pytest.mark.parametrize("flux", ["hll", "lxf"])
@pytest.mark.parametrize("nx", [3, 4, 5])
def test_two_phase_tiny(hyp, orc, nx, flux):
    from hyperelasticsolver_gb300._cases import mph_case, initial_condition
    from test_gpu_mph import eos_pair
    pb = oracle_pb2(orc, nx, flux)
    Pl, Pr = mph_case(7)
    Q0 = initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx)
    Qo, so, to, _ = orc.run(pb, Q0, max_steps=5)
    out = {}
    for prec in ("fp64", "mixed"):
        with hyp.Solver(eos_pair(hyp), nx, model="multi", flux=flux, precision=prec, cfl=0.5) as s:
            s.upload(Q0)
            n, t = s.step(max_steps=5)
            assert n == 5
            out[prec] = (s.download(), t)
    assert abs(out["fp64"][1] - to) <= RTOL_FP64 * to
    assert_close_soa(out["fp64"][0], Qo, RTOL_FP64, f"two-phase {flux} N={nx}")
    assert abs(out["mixed"][1] - to) <= 1e-6 * to
    assert close_to_scale(out["mixed"][0], Qo, MIXED_REL_JUMP)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_of_tiny_problems(hyp, orc, precision):
    """Three- to five-cell problems between larger ones: each steps as it does alone."""
    from test_gpu_batch import make_batch_state
    sizes = np.array([3, 300, 4, 5, 3, 255, 256, 3], dtype=np.int64)
    Q0 = make_batch_state(orc, sizes, seed=21)
    with hyp.Batch(hyp.Barton2009(), sizes, precision=precision) as b:
        b.upload(Q0)
        b.step(12)
        Qb = b.download()
        tb, sb = b.status()
    assert np.all(sb == 12)
    for p, n in enumerate(sizes):
        o = int(np.sum(sizes[:p]))
        with hyp.Solver(hyp.Barton2009(), int(n), precision=precision) as s:
            s.upload(np.ascontiguousarray(Q0[:, o:o + n]))
            s.step(max_steps=12)
            Qs = s.download()
        if precision == "fp64":
            assert_close_soa(Qb[:, o:o + n], Qs, RTOL_FP64, f"problem {p} ({n} cells)")
        else:
            assert close_to_scale(Qb[:, o:o + n], Qs, MIXED_REL), f"problem {p} ({n} cells)"


"""Initial conditions built on the device: the two-phase Riemann test cases
(HyperelasticityMPh.jl:275-426), the two-state fill (main.jl:99-106) and the tanh
volume-fraction profile (main.jl:110-123), against the host / oracle constructions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

B0_SOFT = 2.1 * np.sqrt(0.1)


def pair(hyp):
    return (hyp.Barton2009(), hyp.Barton2009(_b0=B0_SOFT))


def oracle_pb(orc):
    return orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, nx=3,
                       eos=(orc.barton2009(), orc.barton2009(b0=B0_SOFT)))


@pytest.mark.parametrize("testcase", [1, 2, 3, 4, 5, 6, 7, 10])
def test_initial_states_match_the_reference_cases(hyp, orc, testcase):
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    from hyperelasticsolver_gb300._cases import mph_case
    Ql, Qr = HM.initial_states(pair(hyp), testcase)
    Pl, Pr = mph_case(testcase)
    pb = oracle_pb(orc)
    np.testing.assert_allclose(Ql, orc.prim2cons(pb, Pl), rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(Qr, orc.prim2cons(pb, Pr), rtol=1e-14, atol=1e-15)


def test_unknown_testcase_is_an_error(hyp):
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    with pytest.raises(hyp._lib.HypError):
        HM.initial_states(pair(hyp), 8)


@pytest.mark.parametrize("model,precision", [("single", "fp64"), ("single", "mixed"), ("multi", "fp64"),
                                             ("multi", "mixed")])
def test_init_riemann_equals_the_uploaded_fill(hyp, model, precision):
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM, Hyperelasticity as H
    from hyperelasticsolver_gb300._cases import initial_condition, riemann_1ph
    nx = 1001
    if model == "single":
        eos = hyp.Barton2009()
        Pl, Pr = riemann_1ph(eos)
        Ql, Qr = H.prim2cons(eos, Pl), H.prim2cons(eos, Pr)
        kw = {}
    else:
        eos = pair(hyp)
        Ql, Qr = HM.initial_states(eos, 6)
        kw = {"model": "multi", "flux": "hll"}
    Q0 = initial_condition(Ql, Qr, nx)
    with hyp.Solver(eos, nx, precision=precision, **kw) as a, hyp.Solver(eos, nx, precision=precision, **kw) as b:
        a.init_riemann(Ql, Qr)
        b.upload(Q0)
        assert np.array_equal(a.download(), b.download())
        assert a.time() == (0.0, 0)
        a.step(max_steps=5)
        b.step(max_steps=5)
        assert np.array_equal(a.download(), b.download())


def test_init_tanh_matches_the_host_construction(hyp, orc):
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    nx, eps = 96, 0.2
    eos = pair(hyp)
    Ql, Qr = HM.initial_states(eos, 6)
    pb = oracle_pb(orc)
    Pl, Pr = orc.cons2prim(pb, Ql), orc.cons2prim(pb, Qr)
    rows = []
    for i in range(nx):  # main.jl:110-123
        x = (i + 0.5) / nx
        P = (Pl if x < 0.5 else Pr).copy()
        P[0] = 0.2 / 2 * (np.tanh(4 * (x - 0.5) / eps) + 1) + 0.4
        P[15] = 1 - P[0]
        rows.append(P)
    ref = orc.prim2cons(pb, np.array(rows)).T
    with hyp.Solver(eos, nx, model="multi", flux="hll") as s:
        s.init_tanh(Ql, Qr, eps)
        Q = s.download()
    scale = np.maximum(np.max(np.abs(ref), axis=1, keepdims=True), 1e-30)
    assert np.max(np.abs(Q - ref) / scale) < 1e-13
    with hyp.Solver(hyp.Barton2009(), nx) as s, pytest.raises(hyp._lib.UnsupportedError):
        s.init_tanh(Ql, Qr)

"""Two-phase instantaneous pressure relaxation on the GPU (hyp_set_relaxation,
hyp_eval_relax) against the oracle's restatement. An extension with no reference to
match (parity unpinned); tolerance RTOL_FP64 = 1e-12 of each variable's scale, or 4x
the oracle's one-ulp spread where a Newton root is less well conditioned."""
import numpy as np
import pytest

from helpers import RTOL_FP64, assert_close_soa, assert_within_sensitivity, ulp_sensitivity
from test_relax_host import _pb, _states, _pressures, B0_SOFT

pytestmark = pytest.mark.gpu


def eos_pair(hyp):
    return (hyp.Barton2009(), hyp.Barton2009(_b0=B0_SOFT))


@pytest.mark.parametrize("velocity", [False, True])
def test_relax_evaluator_matches_oracle(hyp, orc, velocity):
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    Q = _states(orc, 64, seed=21)
    got = HM.relax_pressure(eos_pair(hyp), Q, velocity=velocity)
    pb = _pb(orc, relax=2 if velocity else 1)
    ref, st = orc.relax(pb, Q)
    assert np.all(st == 0) and np.all(np.isfinite(got))
    sens = ulp_sensitivity(lambda q: orc.relax(pb, q)[0], (Q,))
    assert_within_sensitivity(got, ref, sens, RTOL_FP64, "relaxed cells", axis=0)
    p = _pressures(orc, got)
    assert np.max(np.abs(p[:, 0] - p[:, 1]) / np.abs(p).max(axis=1).clip(1e-2)) <= 1e-10


@pytest.mark.parametrize("mode", ["pressure", "mechanical"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("testcase", [4, 6])
def test_step_with_relaxation(hyp, orc, precision, testcase, mode):
    """The reference's two-phase test cases smoothed over 8 cells (so that interface cells
    hold both phases), 30 HLL steps with relaxation after each: FP64 against the oracle
    run with the same relaxation, mixed against FP64 (density L1 per phase <= 1e-6)."""
    from hyperelasticsolver_gb300._cases import mph_case
    nx, steps = 128, 30
    Pl, Pr = mph_case(testcase)
    pb = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, nx=nx, cfl=0.5, relax=2 if mode == "mechanical" else 1,
                     eos=(orc.barton2009(), orc.barton2009(b0=B0_SOFT)))
    x = (np.arange(nx) + 0.5) / nx
    w = 0.5 * (1 - np.tanh((x - 0.5) * nx / 4))[:, None]
    P = w * np.asarray(Pl)[None] + (1 - w) * np.asarray(Pr)[None]
    P[:, 15] = 1.0 - P[:, 0]
    Q0 = np.ascontiguousarray(orc.prim2cons(pb, P).T)
    Qo, so, to, _ = orc.run(pb, Q0, max_steps=steps)
    with hyp.Solver(eos_pair(hyp), nx, model="multi", flux="hll", cfl=0.5, precision=precision,
                    relax=mode) as s:
        s.upload(Q0)
        n, t = s.step(max_steps=steps)
        assert n == steps
        Qg = s.download()
    if precision == "fp64":
        assert abs(t - to) <= RTOL_FP64 * to
        # the device and the oracle stop their Newton iterations at |d alpha| <= 1e-14 from
        # different Jacobians (closed-form dp/de against differenced), so the relaxed cells
        # agree to that stopping tolerance, not to the last bit, and 30 steps carry it on
        assert_close_soa(Qg, Qo, 1e-10, f"relaxed two-phase run, test case {testcase}")
    else:
        from test_gpu_mph import phase_densities, l1_linf
        errs = [l1_linf(a, b)[0] for a, b in zip(phase_densities(Qg), phase_densities(Qo))]
        assert max(errs) <= 1e-6, errs
    # the relaxation changed the run
    with hyp.Solver(eos_pair(hyp), nx, model="multi", flux="hll", cfl=0.5) as s:
        s.upload(Q0)
        s.step(max_steps=steps)
        assert np.max(np.abs(s.download()[0] - Qg[0])) > 1e-6


def test_relaxation_off_is_the_reference_step(hyp, orc):
    """hyp_set_relaxation(NONE) after PRESSURE gives back the reference's step bitwise."""
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    nx = 256
    Q0 = np.ascontiguousarray(HM.prim2cons_mph(eos_pair(hyp), mph_interface_prims(hyp.Barton2009(), nx)).T)
    out = []
    for modes in ((None,), ("pressure", None)):
        with hyp.Solver(eos_pair(hyp), nx, model="multi", flux="hll") as s:
            for m in modes:
                s.set_relaxation(m)
            s.upload(Q0)
            s.step(max_steps=20)
            out.append(s.download())
    assert np.array_equal(out[0], out[1])
    with hyp.Solver(hyp.Barton2009(), 64) as s:
        with pytest.raises(hyp._lib.HypError):
            s.set_relaxation("pressure")  # two-phase only

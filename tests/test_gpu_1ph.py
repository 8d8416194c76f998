"""Parity of the single-phase FP64 CUDA path with the oracle (GPU).

Everything here calls through the C ABI (libhyperelastic_cuda.so) and checks
the result against the CPU oracle on the same inputs, to the FP64 tolerance
RTOL_FP64 = 1e-12 relative (per variable, relative to that variable's
magnitude over the field)."""
import json
import math
import os

import numpy as np
import pytest

from helpers import RTOL_FP64, assert_close, assert_close_soa, assert_within_sensitivity, rel_err, ulp_sensitivity

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_literal.json")


def random_prims(n, rng, strain=0.08, umax=1.0, smax=1e-3):
    out = np.empty((n, 14))
    k = 0
    while k < n:
        F = np.eye(3) + strain * rng.standard_normal((3, 3))
        if np.linalg.det(F) <= 0.2:
            continue
        out[k] = [8.93 / np.linalg.det(F), *rng.uniform(-umax, umax, 3), rng.uniform(0, smax), *F.reshape(-1, order="F")]
        k += 1
    return out


@pytest.fixture(scope="module")
def states(orc):
    rng = np.random.default_rng(2026)
    P = random_prims(400, rng)
    Q = orc.prim2cons(orc.problem(), P)
    return P, Q


def test_tensor_evaluators(hyp, orc):
    from hyperelasticsolver_gb300 import EquationsOfState as E, Strains as S
    rng = np.random.default_rng(1)
    F = np.array([(np.eye(3) + 0.1 * rng.standard_normal((3, 3))).reshape(-1, order="F") for _ in range(300)])
    F = F[np.linalg.det(F.reshape(-1, 3, 3)) > 0.2]
    Sv = rng.uniform(0, 2e-3, len(F))
    eos, oe = hyp.Barton2009(), orc.barton2009()
    G = orc.finger(F)
    assert_close(S.finger(F), G, RTOL_FP64, "finger")
    assert_close(S.invariants(G), orc.invariants(G), RTOL_FP64, "invariants")
    assert_close(E.energy(eos, Sv, G), orc.energy(oe, Sv, G), RTOL_FP64, "energy")
    e_int = orc.energy(oe, Sv, G)
    # entropy: S = cv log((e - W - U)/(cv t0 p^(gamma/2)) + 1) cancels in e - W - U, so it is held to
    # the oracle's own one-ulp spread where that exceeds 1e-12 of the largest |S|
    sens = ulp_sensitivity(lambda a, b: orc.entropy(oe, a, b), (e_int, G))
    assert_within_sensitivity(E.entropy(eos, e_int, G), orc.entropy(oe, e_int, G), sens, RTOL_FP64, "entropy")
    assert_close(E.stress(eos, Sv, F), orc.stress(oe, Sv, F), RTOL_FP64, "stress")
    ac = E.acoustic(eos, Sv, F)
    ref = orc.acoustic(oe, Sv, F).reshape(-1, 3, 3).transpose(0, 2, 1)
    assert_close(ac, ref, RTOL_FP64, "acoustic")


def test_nondefault_exponents(hyp, orc):
    """Barton2009 with non-integer beta, gamma (the alternative parameters of main.jl:133)."""
    from hyperelasticsolver_gb300 import EquationsOfState as E
    kw = dict(_rho0=8.93, _c0=6.22, _cv=9.0e-4, _t0=300, _b0=3.16, _alpha=1, _beta=3.577, _gamma=2.088)
    eos = hyp.Barton2009(**kw)
    oe = orc.barton2009(8.93, 6.22, 9.0e-4, 300, 3.16, 1, 3.577, 2.088)
    rng = np.random.default_rng(4)
    F = np.array([(np.eye(3) + 0.05 * rng.standard_normal((3, 3))).reshape(-1, order="F") for _ in range(100)])
    Sv = rng.uniform(0, 1e-3, len(F))
    assert_close(E.stress(eos, Sv, F), orc.stress(oe, Sv, F), RTOL_FP64, "stress")
    ref = orc.acoustic(oe, Sv, F).reshape(-1, 3, 3).transpose(0, 2, 1)
    assert_close(E.acoustic(eos, Sv, F), ref, RTOL_FP64, "acoustic")


def test_model_evaluators(hyp, orc, states):
    from hyperelasticsolver_gb300 import Hyperelasticity as H, NumFluxes as NF
    P, Q = states
    eos, pb = hyp.Barton2009(), orc.problem()
    assert_close(H.prim2cons(eos, P), Q, RTOL_FP64, "prim2cons")
    Pg = H.cons2prim(eos, Q)
    Po = orc.cons2prim(pb, Q)
    assert_close(np.delete(Pg, 4, axis=1), np.delete(Po, 4, axis=1), RTOL_FP64, "cons2prim")
    # entropy (cancellation in e - W - U): 1e-12 of max |S| or the oracle's one-ulp spread
    sens = ulp_sensitivity(lambda q: orc.cons2prim(pb, q)[:, 4], (Q,))
    assert_within_sensitivity(Pg[:, 4], Po[:, 4], sens, RTOL_FP64, "cons2prim entropy")
    assert_close(H.flux(eos, Q), orc.flux(pb, Q), RTOL_FP64, "flux")
    eg, eo = H.get_eigvals(eos, Q), orc.speeds(pb, Q)
    scale = np.max(np.abs(eo), axis=1, keepdims=True)  # every speed, in the reference's order
    assert np.max(np.abs(eg - eo) / scale) <= RTOL_FP64, "get_eigvals"
    lam = np.maximum(np.max(np.abs(eo), axis=1)[:-1], np.max(np.abs(eo), axis=1)[1:])
    cg, dmg, dpg = NF.lxf(eos, Q[:-1], Q[1:], lam)
    co, _, _ = orc.lxf(pb, Q[:-1], Q[1:], lam)
    assert_close(cg, co, RTOL_FP64, "lxf")
    assert np.all(dmg == 0) and np.all(dpg == 0)


def test_golden_vectors_on_gpu(hyp):
    from hyperelasticsolver_gb300 import EquationsOfState as E, Hyperelasticity as H
    with open(GOLDEN) as fh:
        g = json.load(fh)
    eos = hyp.Barton2009()
    for t in g["tensors"]:
        ac = E.acoustic(eos, t["S"], np.array(t["F"]))
        assert rel_err(ac.reshape(-1, order="F"), t["acoustic"]) < RTOL_FP64
        st = np.array(t["stress"])
        if np.max(np.abs(st)) > 1e-12:
            assert rel_err(E.stress(eos, t["S"], np.array(t["F"])), st) < RTOL_FP64
    for c in g["cells"]:
        Q = np.array(c["Q"][1:])
        assert rel_err(H.flux(eos, Q), c["flux"][1:]) < RTOL_FP64
        sp = np.array(c["speeds"])  # all six, in the reference's order
        assert np.max(np.abs(H.get_eigvals(eos, Q) - sp)) <= RTOL_FP64 * np.max(np.abs(sp))
    r = g["rusanov"]
    Q0 = np.array(r["Q0"]).T.copy()
    with hyp.Solver(eos, Q0.shape[1], cfl=0.5) as s:
        s.upload(Q0)
        steps, t = s.step(max_steps=2)
        assert steps == 2 and abs(t - sum(r["dt"])) < 1e-15 * 10
        assert_close_soa(s.download(), np.array(r["Q2"]).T, RTOL_FP64, "two Rusanov steps")


def c1_state(hyp, orc, nx=1000):
    from hyperelasticsolver_gb300._cases import riemann_1ph, initial_condition
    eos = hyp.Barton2009()
    Pl, Pr = riemann_1ph(eos)
    pb = orc.problem(nx=nx, cfl=0.5)
    return initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx), pb


def test_riemann_problem_200_steps(hyp, orc):
    """Config: N = 1000 on [0,1], interface at 0.5, CFL 0.5, frozen end cells
    (main.jl:219-220); 200 steps at the strict FP64 tolerance."""
    Q0, pb = c1_state(hyp, orc)
    Qo, so, to, _ = orc.run(pb, Q0, max_steps=200)
    with hyp.Solver(hyp.Barton2009(), 1000, cfl=0.5) as s:
        s.upload(Q0)
        steps, t = s.step(max_steps=200)
        assert steps == 200 and abs(t - to) <= RTOL_FP64 * to
        err = assert_close_soa(s.download(), Qo, RTOL_FP64, "Riemann problem, 200 steps")
    print(f"riemann N=1000, 200 steps: max per-variable relative error {err:.2e}")


@pytest.mark.parametrize("flux", ["rusanov", "lxf"])
def test_riemann_problem_nondefault_exponents(hyp, orc, flux):
    """The Riemann problem with non-integer beta, gamma (main.jl:133's alternative
    Barton2009 parameters), whose powers take the exp/log branch of the step kernels:
    FP64 against the oracle after 100 steps; mixed against FP64 (L1 density <= 1e-6)."""
    from hyperelasticsolver_gb300._cases import riemann_1ph, initial_condition
    eos = hyp.Barton2009(_beta=3.577, _gamma=2.088)
    nx = 1000
    pb = orc.problem(nx=nx, cfl=0.5, flux=orc.FLUX_LXF if flux == "lxf" else orc.FLUX_RUSANOV,
                     eos=(orc.barton2009(beta=3.577, gamma=2.088),) * 2)
    Pl, Pr = riemann_1ph(eos)
    Q0 = initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx)
    Qo, _, to, _ = orc.run(pb, Q0, max_steps=100)
    out = {}
    for prec in ("fp64", "mixed"):
        with hyp.Solver(eos, nx, cfl=0.5, flux=flux, precision=prec) as s:
            s.upload(Q0)
            steps, t = s.step(max_steps=100)
            assert steps == 100
            out[prec] = (s.download(), t)
    assert abs(out["fp64"][1] - to) <= RTOL_FP64 * to
    err = assert_close_soa(out["fp64"][0], Qo, RTOL_FP64, f"non-default exponents ({flux})")
    def density(Q):  # sqrt(det(rho A) / rho0), cons2prim's density
        m = Q[5:14]
        return np.sqrt((m[0] * (m[4] * m[8] - m[5] * m[7]) - m[3] * (m[1] * m[8] - m[7] * m[2])
                        + m[6] * (m[1] * m[5] - m[4] * m[2])) / 8.93)
    a, b = density(out["mixed"][0]), density(out["fp64"][0])
    l1 = np.sum(np.abs(a - b)) / np.sum(np.abs(b))
    print(f"riemann non-default exponents ({flux}): FP64 vs oracle {err:.1e}, mixed density L1 {l1:.1e}")
    assert l1 <= 1e-6


def test_riemann_problem_full_run(hyp, orc):
    """The same problem to t_end = 0.3 / max lambda(t=0) (1113 steps). Over that
    many steps the problem itself amplifies rounding: the oracle run on its own
    input perturbed by one ulp moves by ~1e-10 at the contact. The GPU result must
    lie within max(1e-12, 4x that intrinsic sensitivity) of the oracle, per variable."""
    Q0, pb = c1_state(hyp, orc)
    lam0 = orc.max_speed(pb, Q0)
    t_end = 0.3 / lam0
    Qo, so, to, _ = orc.run(pb, Q0, t_end=t_end)
    rng = np.random.default_rng(0)
    Qp = Q0 * (1 + 2.2e-16 * rng.choice([-1, 0, 1], size=Q0.shape))
    Qq, _, _, _ = orc.run(pb, Qp, t_end=t_end)
    scale = np.max(np.abs(Qo), axis=1)
    scale = np.where(scale > 0, scale, np.max(np.abs(Qo)))
    sens = np.max(np.abs(Qq - Qo), axis=1) / scale
    with hyp.Solver(hyp.Barton2009(), 1000, cfl=0.5) as s:
        s.upload(Q0)
        assert abs(s.max_wavespeed() - lam0) <= 1e-14 * lam0
        steps, t = s.step(t_end=t_end)
        assert steps == so, (steps, so)
        assert abs(t - to) <= RTOL_FP64 * to
        err = np.max(np.abs(s.download() - Qo), axis=1) / scale
    bound = np.maximum(RTOL_FP64, 4 * sens)
    print(f"riemann to t_end: {steps} steps; GPU-oracle {np.array2string(err, precision=1)}; "
          f"oracle 1-ulp sensitivity {np.array2string(sens, precision=1)}")
    assert np.all(err <= bound), (err, bound)


@pytest.mark.parametrize("flux,bc,nx,steps", [("rusanov", "transmissive", 257, 40), ("lxf", "frozen", 100, 30),
                                              ("rusanov", "frozen", 3, 10), ("lxf", "transmissive", 5, 10)])
def test_random_states(hyp, orc, flux, bc, nx, steps):
    rng = np.random.default_rng(nx)
    pb = orc.problem(nx=nx, cfl=0.45, flux=orc.FLUX_LXF if flux == "lxf" else orc.FLUX_RUSANOV,
                     bc=orc.BC_TRANSMISSIVE if bc == "transmissive" else orc.BC_FROZEN)
    P = random_prims(nx, rng, strain=0.03, umax=0.3, smax=2e-4)
    Q0 = np.ascontiguousarray(orc.prim2cons(pb, P).T)
    Qo, so, to, _ = orc.run(pb, Q0, max_steps=steps)
    with hyp.Solver(hyp.Barton2009(), nx, flux=flux, bc=bc, cfl=0.45) as s:
        s.upload(Q0)
        n, t = s.step(max_steps=steps)
        assert n == steps and abs(t - to) <= RTOL_FP64 * to
        assert_close_soa(s.download(), Qo, RTOL_FP64, f"{flux}/{bc}/N={nx}")


def test_graph_and_single_launches_agree_bitwise(hyp, orc):
    Q0, _ = c1_state(hyp, orc, 600)
    with hyp.Solver(hyp.Barton2009(), 600) as a, hyp.Solver(hyp.Barton2009(), 600) as b:
        a.upload(Q0)
        b.upload(Q0)
        a.step(max_steps=37)  # graph replays plus single launches
        for _ in range(37):
            b.step(max_steps=1)
        assert np.array_equal(a.download(), b.download())
        assert a.time() == b.time()


def test_t_end_split_across_calls(hyp, orc):
    Q0, pb = c1_state(hyp, orc, 200)
    t_end = 0.01
    Qo, so, to, _ = orc.run(pb, Q0, t_end=t_end)
    with hyp.Solver(hyp.Barton2009(), 200) as s:
        s.upload(Q0)
        n1, t1 = s.step(max_steps=7)
        n2, t2 = s.step(t_end=t_end)
        n3, t3 = s.step(t_end=t_end)  # already there: no step
        assert n1 + n2 == so and n3 == 0 and t3 == t2
        assert_close_soa(s.download(), Qo, RTOL_FP64, "split run")


def test_uniform_state_preserved_at_size(hyp, orc):
    nx = 1 << 22
    P = np.array([8.93 / 1.02, 0.3, -0.2, 0.1, 1e-4, 1.02, 0.01, 0, 0, 1, 0.02, 0, 0, 1.0])
    q = orc.prim2cons(orc.problem(), P)
    Q0 = np.ascontiguousarray(np.repeat(q[:, None], nx, axis=1))
    with hyp.Solver(hyp.Barton2009(), nx, bc="transmissive") as s:
        s.upload(Q0)
        s.step(max_steps=4)
        assert np.array_equal(s.download(), Q0)


def test_window_of_full_size_run(hyp, orc):
    """At the benchmark size (2^24 cells, 64 seeded segments) a cell after k steps
    depends only on cells within k of it and on the global dt sequence; the GPU's
    dt sequence is reproduced on the host from hyp_max_wavespeed, and a window
    around a segment boundary is re-run on the oracle with those dt."""
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    eos = hyp.Barton2009()
    nx, k, cfl = 1 << 24, 6, 0.5
    seg = orc.prim2cons(orc.problem(), segment_states(eos))
    Q0 = segment_fill(seg, nx)
    dx = 1.0 / nx
    dts = []
    with hyp.Solver(eos, nx, cfl=cfl) as s:
        s.upload(Q0)
        lm0 = s.max_wavespeed()
        assert abs(lm0 - np.max(np.abs(orc.speeds(orc.problem(), seg)))) <= 1e-14 * lm0
        for _ in range(k):
            lm = s.max_wavespeed()
            dts.append((cfl * dx) / lm)
            s.step(max_steps=1)
        Qg = s.download()
    b = (nx * 37) // 64  # a segment boundary
    lo, hi = b - 50, b + 50
    W = np.ascontiguousarray(Q0[:, lo - k: hi + k])
    pb = orc.problem(nx=W.shape[1], cfl=cfl, X=W.shape[1] * dx)  # the window keeps the full run's dx
    Wo = orc.run_dts(pb, W, dts)
    assert_close_soa(Qg[:, lo:hi], Wo[:, k:-k], RTOL_FP64, "window of the 2^24-cell run")


def test_negative_determinant_is_reported(hyp, orc):
    Q0, _ = c1_state(hyp, orc, 64)
    Q0[5:, 17] = -Q0[5:, 17]
    with hyp.Solver(hyp.Barton2009(), 64) as s:
        s.upload(Q0)
        with pytest.raises(hyp._lib.NegativeDeterminantError) as ei:
            s.step(max_steps=3)
        assert ei.value.cell == 17


def test_nonfinite_state_is_reported(hyp, orc):
    Q0, _ = c1_state(hyp, orc, 64)
    Q0[4, 40] = np.nan
    with hyp.Solver(hyp.Barton2009(), 64) as s:
        s.upload(Q0)
        with pytest.raises(hyp._lib.HypError):
            s.step(max_steps=2)


def test_profiling_counts_launches(hyp, orc):
    Q0, _ = c1_state(hyp, orc, 1000)
    with hyp.Solver(hyp.Barton2009(), 1000) as s:
        s.upload(Q0)
        s.set_profiling(True)
        s.step(max_steps=20)
        tm = s.timing()
        assert tm["n_cell"] == 20 and tm["n_update"] == 20
        assert 0 < tm["ms_cell"] <= tm["ms_total"] and math.isfinite(tm["ms_update"])


def test_contexts_on_concurrent_host_threads(hyp, orc):
    """One context per host thread: two threads stepping their own contexts at the
    same time (the ctypes calls release the GIL) get the bits each context gets alone."""
    import threading
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    eos = hyp.Barton2009()
    seg = orc.prim2cons(orc.problem(cfl=0.5), segment_states(eos, 8))
    jobs = [("fp64", segment_fill(seg, 3001)), ("mixed", segment_fill(seg[::-1].copy(), 5003))]

    def run(prec, Q0, out, k):
        with hyp.Solver(eos, Q0.shape[1], precision=prec) as s:
            s.upload(Q0)
            for _ in range(5):
                s.step(max_steps=8)
            out[k] = (s.download(), s.time())

    alone = {}
    for k, (prec, Q0) in enumerate(jobs):
        run(prec, Q0, alone, k)
    together = {}
    threads = [threading.Thread(target=run, args=(prec, Q0, together, k)) for k, (prec, Q0) in enumerate(jobs)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for k in range(len(jobs)):
        assert np.array_equal(alone[k][0], together[k][0]) and alone[k][1] == together[k][1]


@pytest.mark.parametrize("model,precision", [("single", "fp64"), ("single", "mixed"), ("multi", "mixed")])
def test_step_times_log(hyp, orc, model, precision):
    """hyp_step_times returns the time after every step (the Step / t / dt line of
    main.jl:229-237), read back once; its steps are hyp_step's, so the log equals the
    times of single steps and the state is the same, bitwise. With t_end inside the
    run the log stops with the steps."""
    if model == "single":
        Q0, _ = c1_state(hyp, orc)
        eos, kw = hyp.Barton2009(), {}
    else:
        from hyperelasticsolver_gb300._cases import mph_case, initial_condition
        eos = (hyp.Barton2009(), hyp.Barton2009(_b0=2.1 * np.sqrt(0.1)))
        pb = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, nx=1000, cfl=0.6,
                         eos=(orc.barton2009(), orc.barton2009(b0=2.1 * np.sqrt(0.1))))
        Pl, Pr = mph_case(6)
        Q0 = initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), 1000)
        kw = dict(model="multi", flux="hll")
    with hyp.Solver(eos, 1000, cfl=0.5, precision=precision, **kw) as s:
        s.upload(Q0)
        th, dt = s.step_times(60)
        Qa = s.download()
        s.upload(Q0)
        ts = [s.step(max_steps=1)[1] for _ in range(60)]
        assert len(th) == 60 and np.array_equal(th, ts)
        assert np.array_equal(s.download(), Qa)
        assert np.all(dt > 0) and abs(np.sum(dt) - th[-1]) <= 1e-14 * th[-1]
        s.upload(Q0)
        th2, _ = s.step_times(60, t_end=0.5 * (th[29] + th[30]))
        assert np.array_equal(th2, th[:31])
        with pytest.raises(hyp._lib.HypError):
            s.step_times(0)


@pytest.mark.parametrize("model,precision", [("single", "fp64"), ("single", "mixed"), ("multi", "fp64"),
                                             ("multi", "mixed")])
def test_set_eos_between_steps(hyp, orc, model, precision):
    """hyp_set_eos between steps: 20 steps with one EOS, then the EOS of a phase
    changed and 20 more steps, equal a fresh context with the new EOS continued from
    the 20-step state (FP64 bitwise; mixed to the rounding of re-splitting the state
    into hi/lo pairs; stale cached speeds or islands would differ by far more).
    Setting the same EOS again leaves the run unchanged: bitwise, except that the
    single-phase mixed step's cached speeds and islands are then recomputed by the
    upload's kernel, which agrees with the step's own to rounding."""
    Q0 = c1_state(hyp, orc, nx=600)[0]
    new = hyp.Barton2009(_rho0=9.0, _b0=2.3, _beta=3.577)  # changes the cached islands and speeds too
    if model == "single":
        eos_a, eos_b, phase, kw = hyp.Barton2009(), new, 0, {}
    else:
        from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
        from hyperelasticsolver_gb300._cases import mph_interface_prims
        soft = hyp.Barton2009(_b0=2.1 * np.sqrt(0.1))
        eos_a, eos_b, phase = (hyp.Barton2009(), soft), (hyp.Barton2009(), new), 1
        Q0 = np.ascontiguousarray(HM.prim2cons_mph(eos_a, mph_interface_prims(eos_a[0], 600)).T)
        kw = dict(model="multi", flux="hll")
    with hyp.Solver(eos_a, 600, precision=precision, **kw) as s:
        s.upload(Q0)
        s.step(max_steps=20)
        Q20, t20 = s.download(), s.time()[0]
        s.set_eos(new, phase=phase)
        _, t_switch = s.step(max_steps=20)
        Q_switch = s.download()
        orig = eos_a[phase] if model == "multi" else eos_a
        s.upload(Q0)  # the EOS set last stays in force across uploads: restore the original
        s.set_eos(orig, phase=phase)
        s.step(max_steps=20)
        s.set_eos(orig, phase=phase)  # the same parameters again
        s.step(max_steps=20)
        Q_same = s.download()
        with pytest.raises(hyp._lib.HypError):
            s.set_eos(new, phase=1 if model == "single" else 2)
    with hyp.Solver(eos_a, 600, precision=precision, **kw) as s:
        s.upload(Q0)
        s.step(max_steps=40)
        if precision == "fp64" or model == "multi":
            assert np.array_equal(s.download(), Q_same)
        else:  # the single-phase mixed caches are recomputed by the upload's kernel, to rounding
            assert_close_soa(s.download(), Q_same, 1e-6, "same EOS set again")
    with hyp.Solver(eos_b, 600, precision=precision, **kw) as s:
        s.upload(Q20, t0=t20)
        _, t_fresh = s.step(max_steps=20)
        Q_fresh = s.download()
    if precision == "fp64":
        assert t_fresh == t_switch and np.array_equal(Q_fresh, Q_switch)
    else:  # dt from an FP32 max speed: a re-split state may move it by an ulp
        assert abs(t_fresh - t_switch) <= 1e-6 * t_fresh
        assert_close_soa(Q_switch, Q_fresh, 1e-6, "set_eos vs fresh context")

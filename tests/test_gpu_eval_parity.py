"""Function-level evaluators against the oracle (GPU), element by element.

- get_eigvals: every speed (6 per phase), in the reference's order: u.n + c_k then
  u.n - c_k with c_k = sqrt|mu_k|, mu_k the acoustic tensor's eigenvalues as Julia's
  `eigvals` returns them (ascending real part, HyperelasticityMPh.jl:263), checked
  against the oracle and against LAPACK (numpy) on the oracle's acoustic tensor,
  including the rest state's repeated shear pair.
- acoustic(eos, ent, F, n) and get_eigvals(eos, Q, n) for general directions n
  (EquationsOfState.jl:223-246, HyperelasticityMPh.jl:252-266).
- stress(eos, den, e_int, F) (EquationsOfState.jl:162-176) and acoustic(eos, P, n)
  (EquationsOfState.jl:192-221).
- NumFluxes.hll with the caller's eigvals (NumFluxes.jl:90-91).
Tolerance: RTOL_FP64 = 1e-12 of each quantity's scale, or 4x the oracle's own
spread under a one-ulp perturbation of its inputs where that spread is larger
(measured per element, `ulp_sensitivity`)."""
import numpy as np
import pytest

from helpers import RTOL_FP64, assert_close, assert_within_sensitivity, ulp_sensitivity

pytestmark = pytest.mark.gpu

B0_SOFT = 2.1 * np.sqrt(0.1)


def random_F(rng, n, strain=0.08, min_det=0.3):
    out = []
    while len(out) < n:
        F = np.eye(3) + strain * rng.standard_normal((3, 3))
        if np.linalg.det(F) > min_det:
            out.append(F.reshape(-1, order="F"))
    return np.array(out)


def random_prims1(rng, n):
    F = random_F(rng, n)
    P = np.empty((n, 14))
    P[:, 0] = 8.93 / np.linalg.det(F.reshape(-1, 3, 3))
    P[:, 1:4] = rng.uniform(-1.0, 1.0, (n, 3))
    P[:, 4] = rng.uniform(0.0, 1e-3, n)
    P[:, 5:] = F
    return P


def rest_and_case_states(orc):
    """The rest state (speeds {c0, b0, b0}: a repeated root) and test case 6's left state."""
    I = np.eye(3).reshape(-1, order="F")
    A6 = np.diag([1.0 / 0.98, 1.0, 1.0]).reshape(-1, order="F")
    P = np.array([[8.93, 0.0, 0.0, 0.0, 0.0, *I], [8.93 * 0.98, 0.0, 1.05, 2.1, 0.0, *A6],
                  [8.93, 0.3, -0.2, 0.1, 1e-3, *I]])
    return P


def speeds_allowance_check(got, ref, what):
    """All speeds of each cell within RTOL_FP64 of the cell's largest |speed|."""
    got, ref = np.atleast_2d(got), np.atleast_2d(ref)
    scale = np.max(np.abs(ref), axis=1, keepdims=True)
    err = np.abs(got - ref) / scale
    assert np.all(np.isfinite(got)), f"{what}: non-finite"
    assert np.all(err <= RTOL_FP64), f"{what}: worst {err.max():.3e} at {np.unravel_index(err.argmax(), err.shape)}"
    return float(err.max())


def lapack_order_speeds(ac_cm, u_n):
    """u.n +- sqrt|eig| from numpy (LAPACK geev), eigenvalues sorted as Julia sorts them."""
    out = []
    for a, un in zip(np.atleast_2d(ac_cm), np.atleast_1d(u_n)):
        ev = np.linalg.eigvals(a.reshape(3, 3, order="F"))
        ev = sorted(ev, key=lambda z: (z.real, z.imag))
        c = np.sqrt(np.abs(np.array(ev)))
        out.append(np.concatenate([un + c, un - c]))
    return np.array(out)


def test_eigvals_all_speeds_single_phase(hyp, orc):
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    rng = np.random.default_rng(11)
    P = np.vstack([rest_and_case_states(orc), random_prims1(rng, 300)])
    pb = orc.problem()
    Q = orc.prim2cons(pb, P)
    eg, eo = H.get_eigvals(hyp.Barton2009(), Q), orc.speeds(pb, Q)
    worst = speeds_allowance_check(eg, eo, "get_eigvals (6 speeds, reference order)")
    # the order: c_k ascending for a positive-definite acoustic tensor
    c = eg[:, :3] - eg[:, 3:]
    assert np.all(np.diff(c, axis=1) >= -1e-12 * c[:, 2:3])
    # rest state: {b0, b0, c0} exactly as the physics says
    assert np.allclose(eg[0, :3], [2.1, 2.1, 4.6], rtol=1e-13, atol=0)
    # LAPACK on the oracle's acoustic tensor
    Po = orc.cons2prim(pb, Q)
    ac = orc.acoustic(orc.barton2009(), Po[:, 4], Po[:, 5:])
    lp = lapack_order_speeds(ac, Po[:, 1])
    worst_l = speeds_allowance_check(eg, lp, "get_eigvals vs LAPACK")
    print(f"6 speeds per cell vs oracle {worst:.2e}, vs LAPACK {worst_l:.2e} (of max |speed|)")


def test_eigvals_all_speeds_two_phase(hyp, orc):
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    from test_gpu_mph import random_mph, oracle_pb
    rng = np.random.default_rng(12)
    Q = random_mph(orc, 128, rng)
    eos = (hyp.Barton2009(), hyp.Barton2009(_b0=B0_SOFT))
    eg, eo = HM.get_eigvals(eos, Q), orc.speeds(oracle_pb(orc), Q)
    speeds_allowance_check(eg[:, :6], eo[:, :6], "phase 1 speeds")
    speeds_allowance_check(eg[:, 6:], eo[:, 6:], "phase 2 speeds")


def test_eigvals_general_direction(hyp, orc):
    from hyperelasticsolver_gb300 import Hyperelasticity as H, HyperelasticityMPh as HM
    from test_gpu_mph import random_mph, oracle_pb
    rng = np.random.default_rng(13)
    P = random_prims1(rng, 200)
    pb = orc.problem()
    Q = orc.prim2cons(pb, P)
    d = rng.standard_normal((200, 3))
    d[:100] /= np.linalg.norm(d[:100], axis=1, keepdims=True)  # unit and non-unit directions
    eg, eo = H.get_eigvals(hyp.Barton2009(), Q, d), orc.speeds(pb, Q, d)
    speeds_allowance_check(eg, eo, "get_eigvals along n")
    # one direction for all, and n = e1 through the general path equals the e1 path
    e1 = orc.speeds(pb, Q, [1.0, 0.0, 0.0])
    speeds_allowance_check(H.get_eigvals(hyp.Barton2009(), Q, np.tile([1.0, 0.0, 0.0], (200, 1)) * 1.0), e1, "e1")
    ey = H.get_eigvals(hyp.Barton2009(), Q, [0.0, 1.0, 0.0])
    speeds_allowance_check(ey, orc.speeds(pb, Q, [0.0, 1.0, 0.0]), "along e2")
    Q2 = random_mph(orc, 64, rng)
    d2 = rng.standard_normal((64, 3))
    eos = (hyp.Barton2009(), hyp.Barton2009(_b0=B0_SOFT))
    speeds_allowance_check(HM.get_eigvals(eos, Q2, d2), orc.speeds(oracle_pb(orc), Q2, d2), "two-phase along n")


def test_acoustic_general_direction(hyp, orc):
    from hyperelasticsolver_gb300 import EquationsOfState as E
    rng = np.random.default_rng(14)
    F = random_F(rng, 300, strain=0.1)
    S = rng.uniform(0.0, 2e-3, len(F))
    d = rng.standard_normal((len(F), 3))
    oe = orc.barton2009()
    got = E.acoustic(hyp.Barton2009(), S, F, d)
    ref = orc.acoustic(oe, S, F, d).reshape(-1, 3, 3).transpose(0, 2, 1)
    assert_close(got, ref, RTOL_FP64, "acoustic(eos, ent, F, n)")
    # a rotated frame: n = R e1 on F R^T gives R Omega(e1) R^T... checked through the oracle instead
    kw = dict(_rho0=8.93, _c0=6.22, _cv=9.0e-4, _t0=300, _b0=3.16, _alpha=1, _beta=3.577, _gamma=2.088)
    oe2 = orc.barton2009(8.93, 6.22, 9.0e-4, 300, 3.16, 1, 3.577, 2.088)
    got2 = E.acoustic(hyp.Barton2009(**kw), S, F, d)
    ref2 = orc.acoustic(oe2, S, F, d).reshape(-1, 3, 3).transpose(0, 2, 1)
    assert_close(got2, ref2, RTOL_FP64, "acoustic along n, general exponents")


def test_stress_den_eint(hyp, orc):
    """stress(eos, den, e_int, F) (EquationsOfState.jl:162-176), including states whose
    entropy argument sits at the 1e-6 clamp."""
    from hyperelasticsolver_gb300 import EquationsOfState as E, Strains as St
    rng = np.random.default_rng(15)
    F = random_F(rng, 300)
    oe = orc.barton2009()
    S = rng.uniform(0.0, 2e-3, len(F))
    e_int = orc.energy(oe, S, orc.finger(F))
    e_int[:20] -= 1.0  # far below the cold + shear energy: the clamp
    den = rng.uniform(8.0, 9.5, len(F))
    got = E.stress(hyp.Barton2009(), den, e_int, F)
    ref = orc.stress_den(oe, den, e_int, F)
    sens = ulp_sensitivity(lambda d, e, f: orc.stress_den(oe, d, e, f), (den, e_int, F))
    worst = assert_within_sensitivity(got, ref, sens, RTOL_FP64, "stress(eos, den, e_int, F)")
    # with den = rho0/det F and e_int = energy(S, G) it is stress(eos, S, F)
    den0 = 8.93 / np.linalg.det(F.reshape(-1, 3, 3).transpose(0, 2, 1))
    assert_close(E.stress(hyp.Barton2009(), den0[20:], e_int[20:], F[20:]), orc.stress(oe, S[20:], F[20:]), 1e-9,
                 "stress(den, e(S), F) = stress(S, F)")
    print(f"stress(eos, den, e_int, F): worst error / allowance {worst:.2f}")


def test_acoustic_prim(hyp, orc):
    """acoustic(eos, P, n) (EquationsOfState.jl:192-221): internal energy and den held."""
    from hyperelasticsolver_gb300 import EquationsOfState as E
    rng = np.random.default_rng(16)
    F = random_F(rng, 200)
    n = len(F)
    P = np.empty((n, 15))
    P[:, 0] = rng.uniform(0.2, 1.0, n)
    P[:, 1] = 8.93 / np.linalg.det(F.reshape(-1, 3, 3).transpose(0, 2, 1))
    P[:, 2:5] = rng.uniform(-0.5, 0.5, (n, 3))
    P[:, 5] = rng.uniform(0.0, 1e-3, n)
    P[:, 6:] = F
    d = rng.standard_normal((n, 3))
    d[:50] = [1.0, 0.0, 0.0]
    oe = orc.barton2009()
    got = E.acoustic(hyp.Barton2009(), P, d)
    ref = orc.acoustic_prim(oe, P, d)
    sens = ulp_sensitivity(lambda p, dd: orc.acoustic_prim(oe, p, dd), (P, d))
    worst = assert_within_sensitivity(got.transpose(0, 2, 1).reshape(n, 9), ref, sens, RTOL_FP64,
                                      "acoustic(eos, P, n)")
    print(f"acoustic(eos, P, n): worst error / allowance {worst:.2f}")


def test_hll_with_given_eigvals(hyp, orc):
    """NumFluxes.hll uses the speeds it is given (NumFluxes.jl:90-91): speeds wider than
    the cells' own change D-, D+ exactly as the oracle says; None = the cells' own."""
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM, NumFluxes as NF
    from test_gpu_mph import random_mph, oracle_pb
    rng = np.random.default_rng(17)
    Q = random_mph(orc, 65, rng)
    eos = (hyp.Barton2009(), hyp.Barton2009(_b0=B0_SOFT))
    pb = oracle_pb(orc)
    Ql, Qr = Q[:-1], Q[1:]
    eo = orc.speeds(pb, Q)
    wide_l = eo[:-1] - rng.uniform(0.5, 3.0, (64, 1))
    wide_r = eo[1:] + rng.uniform(0.5, 3.0, (64, 1))
    _, dm, dp = NF.hll(eos, Ql, Qr, [wide_l, wide_r])
    dmo, dpo = orc.hll(pb, Ql, Qr, wide_l, wide_r)
    for got, ref, nm, k in ((dm, dmo, "D-", 0), (dp, dpo, "D+", 1)):
        sens = ulp_sensitivity(lambda a, b, c, d: orc.hll(pb, a, b, c, d)[k], (Ql, Qr, wide_l, wide_r))
        assert_within_sensitivity(got, ref, sens, RTOL_FP64, f"hll {nm} with given speeds", axis=0)
    _, dm0, _ = NF.hll(eos, Ql, Qr)
    assert np.max(np.abs(dm - dm0)) > 1e-6 * np.max(np.abs(dm0))  # the given speeds are used
    # the cells' own speeds passed in give the face main.jl:225 computes (the speed bounds
    # agree to rounding: the evaluator's and the step's eigen-solves differ in the last bits)
    _, dm1, dp1 = NF.hll(eos, Ql, Qr, [HM.get_eigvals(eos, Ql), HM.get_eigvals(eos, Qr)])
    _, dm2, dp2 = NF.hll(eos, Ql, Qr)
    assert_close(dm1, dm2, RTOL_FP64, "hll, own speeds given")
    assert_close(dp1, dp2, RTOL_FP64, "hll, own speeds given")


def test_golden_function_forms_on_gpu(hyp, orc):
    """The 40-digit transliteration's values for the function forms above."""
    import json
    import os
    from hyperelasticsolver_gb300 import EquationsOfState as E, Hyperelasticity as H
    with open(os.path.join(os.path.dirname(__file__), "golden", "golden_literal.json")) as fh:
        x = json.load(fh)["extras"]
    eos, oe = hyp.Barton2009(), orc.barton2009()
    for t in x["acoustic_dir"]:
        got = E.acoustic(eos, t["S"], np.array(t["F"]), t["n"]).reshape(-1, order="F")
        assert_close(got, t["acoustic"], RTOL_FP64, "golden acoustic along n")
    for t in x["stress_den"]:
        F = np.array(t["F"])
        got = E.stress(eos, t["den"], t["e_int"], F)
        sens = ulp_sensitivity(lambda d, e, f: orc.stress_den(oe, d, e, f),
                               (np.array([t["den"]]), np.array([t["e_int"]]), F[None]), trials=6)
        assert_within_sensitivity(got, t["stress"], sens[0], RTOL_FP64, "golden stress(den, e_int, F)")
    for t in x["acoustic_prim"]:
        P = np.array(t["P"])
        got = E.acoustic(eos, P, t["n"]).reshape(-1, order="F")
        sens = ulp_sensitivity(lambda p: orc.acoustic_prim(oe, p, t["n"]), (P[None],), trials=6)
        assert_within_sensitivity(got, t["acoustic"], sens[0], RTOL_FP64, "golden acoustic(P, n)")
    for c in x["speeds_dir"]:
        sp = np.array(c["speeds"])
        got = H.get_eigvals(eos, np.array(c["Q"])[1:], c["n"])
        assert np.max(np.abs(got - sp)) <= RTOL_FP64 * np.max(np.abs(sp)), "golden get_eigvals along n"


def test_thirteen_value_forms(hyp, orc):
    """Hyperelasticity.jl's 13-value cons2prim / prim2cons / flux (:25-114) with the eos
    passed in, against the oracle's per-phase functions at alpha = 1 (the 14-value model
    the reference's solver runs), reordered to the 13-value layout."""
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    rng = np.random.default_rng(18)
    eos, pb = hyp.Barton2009(), orc.problem()
    P14 = random_prims1(rng, 50)
    Q14 = orc.prim2cons(pb, P14)
    Q13 = H.q14_to_q13(Q14)
    F = P14[:, 5:].reshape(-1, 3, 3).transpose(0, 2, 1)  # [i][j] = F[i, j]
    assert_close(H.prim2cons13(eos, P14[:, 1:4], F, P14[:, 4]), Q13, RTOL_FP64, "prim2cons13")
    den, vel, F13, e_int = H.cons2prim13(eos, Q13)
    Po = orc.cons2prim(pb, Q14)
    assert_close(den, Po[:, 0], RTOL_FP64, "den")
    assert_close(vel, Po[:, 1:4], RTOL_FP64, "vel")
    assert_close(F13, F, RTOL_FP64, "F")
    f13 = H.flux13(eos, Q13)
    fo = H.q14_to_q13(orc.flux(pb, Q14))
    assert_close(f13, fo, RTOL_FP64, "flux13")
    assert np.all(f13[:, 3:6] == 0.0)  # the rho F row-1 flux is identically zero (Hyperelasticity.jl:106)

"""The oracle pinned: known-answer tests from the physics, the committed 40-digit
golden vectors of the independent transliteration, LAPACK eigenvalues, and
internal consistency of its modes. CPU only."""
import json
import os

import numpy as np
import pytest

from helpers import rel_err

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_literal.json")


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


I9 = np.eye(3).reshape(-1, order="F")


def test_stress_vanishes_at_rest(orc):
    # A = I, S = 0: e = 0 and sigma = 0 (EquationsOfState.jl:118-137, 179-190)
    e = orc.barton2009()
    assert np.max(np.abs(orc.stress(e, 0.0, I9))) < 1e-14
    assert abs(orc.energy(e, 0.0, I9)) < 1e-15


def test_speeds_at_rest_are_c0_b0_b0(orc):
    # k0 = c0^2 - 4/3 b0^2 makes the rest-state acoustic tensor diag(c0^2, b0^2, b0^2)
    e = orc.barton2009()
    ac = orc.acoustic(e, 0.0, I9).reshape(3, 3, order="F")
    np.testing.assert_allclose(np.diag(ac), [4.6 ** 2, 2.1 ** 2, 2.1 ** 2], rtol=1e-14)
    assert np.max(np.abs(ac - np.diag(np.diag(ac)))) < 1e-13
    mods = np.sort(np.sqrt(orc.eig3_moduli(ac.reshape(-1, order="F"))))[::-1]
    np.testing.assert_allclose(mods, [4.6, 2.1, 2.1], rtol=1e-14)  # the repeated pair included


def test_testcase6_left_speeds(orc):
    # HyperelasticityMPh.jl:355-360 left distortion with S = 1e-3
    e = orc.barton2009()
    F = np.array([[0.98, 0, 0], [0.02, 1, 0.1], [0, 0, 1.0]]).reshape(-1, order="F")
    mods = np.sort(np.sqrt(orc.eig3_moduli(orc.acoustic(e, 1e-3, F))))[::-1]
    np.testing.assert_allclose(mods, [5.78791431, 2.41681731, 1.9840291], rtol=2e-8)


def test_eigen_moduli_match_lapack(orc):
    rng = np.random.default_rng(7)
    e = orc.barton2009()
    for _ in range(50):
        F = np.eye(3) + 0.15 * rng.standard_normal((3, 3))
        if np.linalg.det(F) <= 0:
            continue
        ac = orc.acoustic(e, rng.uniform(0, 2e-3), F.reshape(-1, order="F"))
        ref = np.sort(np.abs(np.linalg.eigvals(ac.reshape(3, 3, order="F"))))[::-1]
        got = np.sort(orc.eig3_moduli(ac))[::-1]
        assert abs(got[0] - ref[0]) <= 1e-13 * ref[0]  # the spectral radius (what the solver uses)
        np.testing.assert_allclose(got, ref, rtol=1e-13)  # all moduli


def test_quadrature_nodes(orc):
    x, w = orc.quadrature(0)
    xr, wr = np.polynomial.legendre.leggauss(6)
    np.testing.assert_allclose(x, (xr + 1) / 2, rtol=0, atol=2e-16)
    np.testing.assert_allclose(w, wr / 2, rtol=0, atol=2e-16)
    xl, wl = orc.quadrature(1)
    assert xl[0] == 0.0 and xl[-1] == 1.0 and abs(np.sum(wl) - 1) < 1e-15
    # 6-point Lobatto integrates polynomials of degree <= 9 exactly
    assert abs(np.sum(wl * xl ** 9) - 0.1) < 1e-15


def test_golden_tensor_functions(orc, golden):
    e = orc.barton2009()
    for t in golden["tensors"]:
        F = np.array(t["F"])
        assert rel_err(orc.finger(F), t["finger"]) < 1e-14
        assert rel_err(orc.invariants(np.array(t["finger"])), t["invariants"]) < 1e-14
        if abs(t["energy"]) > 1e-12:
            assert rel_err(orc.energy(e, t["S"], np.array(t["finger"])), t["energy"]) < 1e-12
        st = np.array(t["stress"])
        if np.max(np.abs(st)) > 1e-12:
            assert rel_err(orc.stress(e, t["S"], F), st) < 1e-13
        assert rel_err(orc.acoustic(e, t["S"], F), t["acoustic"]) < 1e-13
        got = orc.eig3_sorted(np.array(t["acoustic"]))  # Julia's eigvals order, every modulus
        assert np.max(np.abs(got - t["moduli"])) <= 1e-14 * np.max(t["moduli"])


def test_golden_cells(orc, golden):
    pb = orc.problem()
    for c in golden["cells"]:
        P = np.array(c["P"])[1:]  # alpha == 1 dropped
        Q = orc.prim2cons(pb, P)
        assert rel_err(Q, c["Q"][1:]) < 1e-14
        Qg = np.array(c["Q"][1:])
        assert rel_err(orc.cons2prim(pb, Qg), c["prim"][1:]) < 1e-12
        assert rel_err(orc.flux(pb, Qg), c["flux"][1:]) < 1e-13
        s = orc.speeds(pb, Qg)  # all six speeds, in the reference's order
        assert np.max(np.abs(s - c["speeds"])) < 1e-14 * np.max(np.abs(c["speeds"]))


def test_golden_nondefault_exponents(orc, golden):
    """main.jl:133's alternative Barton2009 parameters (beta = 3.577, gamma = 2.088: the
    general powers through exp/log) against the 40-digit transliteration."""
    nd = golden["nondefault"]
    e = orc.barton2009(*nd["eos"])
    for t in nd["tensors"]:
        F = np.array(t["F"])
        G = orc.finger(F)
        assert rel_err(orc.energy(e, t["S"], G), t["energy"]) < 1e-12
        assert rel_err(orc.stress(e, t["S"], F), t["stress"]) < 1e-13
        assert rel_err(orc.acoustic(e, t["S"], F), t["acoustic"]) < 1e-13
        got = orc.eig3_sorted(np.array(t["acoustic"]))
        assert np.max(np.abs(got - t["moduli"])) <= 1e-14 * np.max(t["moduli"])
    pb = orc.problem(eos=(e, e))
    for c in nd["cells"]:
        Q = orc.prim2cons(pb, np.array(c["P"])[1:])
        assert rel_err(Q, c["Q"][1:]) < 1e-14
        Qg = np.array(c["Q"][1:])
        assert rel_err(orc.flux(pb, Qg), c["flux"][1:]) < 1e-13
        s = orc.speeds(pb, Qg)
        assert np.max(np.abs(s - c["speeds"])) < 1e-14 * np.max(np.abs(c["speeds"]))


def test_golden_twophase_noncons_and_hll(orc, golden):
    eos = (orc.barton2009(), orc.barton2009(b0=golden["eos2_b0"]))
    pb = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, eos=eos)
    for c in golden["noncons"]:
        assert rel_err(orc.noncons(pb, np.array(c["Q"])), c["bcol"]) < 1e-13
    for h in golden["hll"]:
        dm, dp = orc.hll(pb, np.array(h["Ql"]), np.array(h["Qr"]), np.array(h["spdL"]), np.array(h["spdR"]))
        assert rel_err(dm, h["dm"]) < 1e-12
        assert rel_err(dp, h["dp"]) < 1e-12


def test_golden_twophase_hll_nondefault_exponents(orc, golden):
    """The two-phase HLL face with phase 1 on main.jl:133's alternative parameters."""
    nd = golden["nondefault"]
    h = nd["hll"]
    eos = (orc.barton2009(*nd["eos"]), orc.barton2009(b0=golden["eos2_b0"]))
    pb = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, eos=eos)
    assert rel_err(np.sort(orc.speeds(pb, np.array(h["Ql"]))), np.sort(h["spdL"])) < 1e-13  # HLL takes min / max
    dm, dp = orc.hll(pb, np.array(h["Ql"]), np.array(h["Qr"]), np.array(h["spdL"]), np.array(h["spdR"]))
    assert rel_err(dm, h["dm"]) < 1e-12
    assert rel_err(dp, h["dp"]) < 1e-12


def test_golden_twophase_lxf(orc, golden):
    """The two-phase LxF face (NumFluxes.jl:25-60): flux and D+- = half the
    Gauss-Lobatto path integral, against the 40-digit transliteration."""
    eos = (orc.barton2009(), orc.barton2009(b0=golden["eos2_b0"]))
    pb = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_LXF, eos=eos)
    for c in golden["lxf2"]:
        cons, dm, dp = orc.lxf(pb, np.array(c["Ql"]), np.array(c["Qr"]), c["lam"])
        assert rel_err(cons, c["cons"]) < 1e-13
        assert rel_err(dm, c["dm"]) < 1e-12
        assert rel_err(dp, c["dp"]) < 1e-12


def test_golden_hank2016(orc, golden):
    """Hank2016 energy, pressure and stress (EquationsOfState.jl:305-366) against the
    40-digit transliteration (its own dual numbers for the stress)."""
    h = orc.hank2016()
    for c in golden["hank"]:
        G = np.array(c["G"])
        assert abs(orc.hank_energy(h, c["den"], c["pres"], G) - c["energy"]) <= 1e-13 * abs(c["energy"])
        p = orc.hank_pressure(h, c["den"], c["energy"], np.array(c["invariants"]))
        assert abs(p - c["pressure"]) <= 1e-13 * max(abs(c["pressure"]), 1e9)  # cancellation against gamma p_inf
        assert rel_err(orc.hank_stress(h, c["den"], c["pres"], np.array(c["F"])), c["stress"]) < 1e-12


def test_golden_rusanov_steps(orc, golden):
    g = golden["rusanov"]
    Q0 = np.array(g["Q0"]).T.copy()
    pb = orc.problem(nx=Q0.shape[1], cfl=0.5)
    Q, steps, t, dt = orc.run(pb, Q0, max_steps=2, nthreads=1)
    assert steps == 2
    assert abs(t - sum(g["dt"])) < 1e-15
    err = rel_err(Q, np.array(g["Q2"]).T, axis=1)
    assert np.all(err < 1e-13), err


def test_uniform_state_is_preserved_exactly(orc):
    pb = orc.problem(nx=16)
    e = orc.barton2009()
    F = np.array([[1.01, 0.02, 0], [0, 0.99, 0.01], [0.005, 0, 1.0]]).reshape(-1, order="F")
    P = np.array([8.93 / np.linalg.det(F.reshape(3, 3, order="F")), 0.3, -0.2, 0.1, 1e-4, *F])
    Q0 = np.repeat(orc.prim2cons(pb, P)[:, None], 16, axis=1)
    for bc in (orc.BC_FROZEN, orc.BC_TRANSMISSIVE):
        pb.bc = bc
        Q, _, _, _ = orc.run(pb, Q0, max_steps=5, nthreads=2)
        assert np.array_equal(Q, Q0)


def test_constant_alpha_gives_zero_noncons(orc):
    # alpha constant across a face: B(Q) dQ only involves d alpha, so D+- = 0 (NumFluxes.jl:35-60)
    from hyperelasticsolver_gb300._cases import mph_case
    eos = (orc.barton2009(), orc.barton2009())
    pb = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_LXF, eos=eos)
    Pl, Pr = mph_case(5)
    Ql, Qr = orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr)
    cons, dm, dp = orc.lxf(pb, Ql, Qr, 5.0)
    assert np.max(np.abs(dm)) == 0 and np.max(np.abs(dp)) == 0


def test_prim_cons_round_trip(orc):
    pb = orc.problem()
    rng = np.random.default_rng(3)
    for _ in range(20):
        F = np.eye(3) + 0.05 * rng.standard_normal((3, 3))
        P = np.array([8.93 / np.linalg.det(F), *rng.uniform(-1, 1, 3), rng.uniform(0, 1e-3), *F.reshape(-1, order="F")])
        P2 = orc.cons2prim(pb, orc.prim2cons(pb, P))
        assert rel_err(np.delete(P2, 4), np.delete(P, 4)) < 1e-13
        assert abs(P2[4] - P[4]) < 1e-11 * max(P[4], 1e-3)


@pytest.mark.parametrize("model,flux", [(1, 0), (1, 1), (2, 2), (2, 1)])
def test_literal_and_face_modes_agree_bitwise(orc, model, flux):
    """The literal mode (each face evaluated twice, as update_cell) and the
    once-per-face mode give identical results: the functions are pure."""
    from hyperelasticsolver_gb300._cases import mph_case, riemann_1ph, initial_condition
    import hyperelasticsolver_gb300 as h
    nx = 12
    if model == 1:
        pb = orc.problem(nx=nx, flux=flux)
        Pl, Pr = riemann_1ph(h.Barton2009())
    else:
        pb = orc.problem(model=2, flux=flux, nx=nx, eos=(orc.barton2009(), orc.barton2009(b0=0.66)))
        Pl, Pr = mph_case(6)
    Q0 = initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx)
    a = orc.run(pb, Q0, max_steps=3, literal=True, nthreads=2)[0]
    b = orc.run(pb, Q0, max_steps=3, literal=False, nthreads=2)[0]
    assert np.array_equal(a, b)


def test_dual_run_gradient_matches_central_differences(orc):
    """The oracle's forward-mode run (every scalar a dual with 15 partials: the left
    state and the moduli b0sq, k0) against central differences of plain oracle runs."""
    from hyperelasticsolver_gb300._cases import adjoint_states, initial_condition
    from hyperelasticsolver_gb300.EquationsOfState import Barton2009
    eos = Barton2009()
    pl, pr = adjoint_states(eos)
    nx, steps = 24, 8
    idx = [0, 1, 2, 3, 5, 6, 7, 8, 9, 10, 11, 12, 13]
    theta0 = np.concatenate([pl[idx], [eos.b0sq, eos.k0]])
    target = np.full(nx, eos.rho0)

    def loss(th):
        b0sq, k0 = th[13], th[14]
        e = orc.barton2009(b0=np.sqrt(b0sq), c0=np.sqrt(k0 + 4 / 3 * b0sq))
        pb = orc.problem(nx=nx, cfl=0.5, eos=(e, e))
        p = pl.copy()
        p[idx] = th[:13]
        Q, _, _, _ = orc.run(pb, initial_condition(orc.prim2cons(pb, p), orc.prim2cons(pb, pr), nx),
                             max_steps=steps, nthreads=2)
        rho = orc.cons2prim(pb, Q.T)[:, 0]
        return 0.5 * np.sum((rho - target) ** 2)

    L, g = orc.misfit_grad_dual(orc.problem(nx=nx, cfl=0.5), pl, pr, steps, target, nthreads=2)
    assert abs(L - loss(theta0)) <= 1e-13 * L
    fd = np.zeros(15)
    for k in range(15):
        h = 1e-6 * max(abs(theta0[k]), 1.0)  # an absolute floor keeps rounding out of the small entries
        tp, tm = theta0.copy(), theta0.copy()
        tp[k] += h
        tm[k] -= h
        fd[k] = (loss(tp) - loss(tm)) / (tp[k] - tm[k])
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    assert rel.max() <= 1e-6, rel


def test_eigvals_order_is_julias(orc):
    """get_eigvals returns u.n + c_k then u.n - c_k with c_k = sqrt|mu_k| and mu_k in the
    order Julia's eigvals gives (ascending real part, HyperelasticityMPh.jl:263); checked
    against LAPACK (numpy) eigenvalues sorted the same way, for all three moduli."""
    rng = np.random.default_rng(8)
    e = orc.barton2009()
    for _ in range(50):
        F = np.eye(3) + 0.15 * rng.standard_normal((3, 3))
        if np.linalg.det(F) <= 0:
            continue
        ac = orc.acoustic(e, rng.uniform(0, 2e-3), F.reshape(-1, order="F"), rng.standard_normal(3))
        ev = np.abs(sorted(np.linalg.eigvals(ac.reshape(3, 3, order="F")), key=lambda z: (z.real, z.imag)))
        # eigenvalues are accurate relative to the matrix norm (LAPACK's bound), not each to itself
        assert np.max(np.abs(orc.eig3_sorted(ac) - ev)) <= 1e-13 * np.max(ev)
    # a non-symmetric matrix with a complex pair: the pair's real part orders it
    M = np.array([[3.0, -2.0, 0.0], [2.0, 3.0, 0.0], [0.0, 0.0, 1.0]])
    ev = sorted(np.linalg.eigvals(M), key=lambda z: (z.real, z.imag))
    np.testing.assert_allclose(orc.eig3_sorted(M.reshape(-1, order="F")), np.abs(ev), rtol=1e-14)
    M = np.array([[-5.0, 1.0, 0.0], [0.0, 2.0, 0.5], [0.3, 0.0, 0.5]])
    ev = sorted(np.linalg.eigvals(M), key=lambda z: (z.real, z.imag))
    np.testing.assert_allclose(orc.eig3_sorted(M.reshape(-1, order="F")), np.abs(ev), rtol=1e-13)


def test_golden_function_forms(orc, golden):
    """acoustic(eos, ent, F, n) for general n, stress(eos, den, e_int, F), acoustic(eos, P, n),
    get_eigvals along n and an HLL face given wider speeds, against the 40-digit
    transliteration (its acoustic(eos, P, n) by 40-digit central differences)."""
    x = golden["extras"]
    e = orc.barton2009()
    for t in x["acoustic_dir"]:
        assert rel_err(orc.acoustic(e, t["S"], np.array(t["F"]), t["n"]), t["acoustic"]) < 1e-13
    for t in x["stress_den"]:
        assert rel_err(orc.stress_den(e, t["den"], t["e_int"], np.array(t["F"])), t["stress"]) < 1e-12
    for t in x["acoustic_prim"]:
        assert rel_err(orc.acoustic_prim(e, np.array(t["P"]), t["n"]), t["acoustic"]) < 1e-12
    pb = orc.problem()
    for c in x["speeds_dir"]:
        s = orc.speeds(pb, np.array(c["Q"])[1:], c["n"])
        assert np.max(np.abs(s - c["speeds"])) < 1e-13 * np.max(np.abs(c["speeds"]))
    h = x["hll_given"]
    eos = (orc.barton2009(), orc.barton2009(b0=golden["eos2_b0"]))
    pb2 = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, eos=eos)
    dm, dp = orc.hll(pb2, np.array(h["Ql"]), np.array(h["Qr"]), np.array(h["spdL"]), np.array(h["spdR"]))
    assert rel_err(dm, h["dm"]) < 1e-12 and rel_err(dp, h["dp"]) < 1e-12


def test_acoustic_prim_holds_energy_not_entropy(orc):
    """acoustic(eos, P, n) differs from acoustic(eos, S, A, n) only through the entropy
    following F at fixed e_int: at S with exp(S/cv) = 1 (cold state) and no shear
    deformation the two agree; in general they do not."""
    e = orc.barton2009()
    I9 = np.eye(3).reshape(-1, order="F")
    P = np.concatenate([[1.0, 8.93, 0, 0, 0, 0.0], I9])
    np.testing.assert_allclose(orc.acoustic_prim(e, P, [1.0, 0, 0]), orc.acoustic(e, 0.0, I9), rtol=1e-12, atol=1e-12)
    rng = np.random.default_rng(3)
    F = (np.eye(3) + 0.05 * rng.standard_normal((3, 3))).reshape(-1, order="F")
    P = np.concatenate([[1.0, 8.93 / np.linalg.det(F.reshape(3, 3)), 0, 0, 0, 1e-3], F])
    assert rel_err(orc.acoustic_prim(e, P, [1.0, 0, 0]), orc.acoustic(e, 1e-3, F)) > 1e-6

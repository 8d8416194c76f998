"""Two-phase instantaneous pressure relaxation (an extension with no reference to
match: parity unpinned). CPU only: the oracle's restatement and the product's
closed-form code (hyp_relax.cuh compiled for the host) on the invariants the
procedure must keep -- alpha_1 + alpha_2 = 1, each phase's mass and momentum, the
mixture's total energy, one pressure in both phases afterwards, relaxing a relaxed
state changes nothing -- and against each other."""
import ctypes

import numpy as np
import pytest

from test_physics_host import shim, P  # noqa: F401  (the host build of the product's physics)

B0_SOFT = 2.1 * np.sqrt(0.1)
EP1 = (8.93, 4.6, 3.9e-4, 300, 2.1, 1, 3, 2)
EP2 = (8.93, 4.6, 3.9e-4, 300, B0_SOFT, 1, 3, 2)


def _pb(orc, relax=1):
    return orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, relax=relax,
                       eos=(orc.barton2009(), orc.barton2009(b0=B0_SOFT)))


def _states(orc, n, seed=3):
    """Two-phase cells whose phases sit at different pressures: mixtures of the
    reference's test-case states and random strains, alpha_1 in (0.05, 0.95)."""
    from hyperelasticsolver_gb300._cases import mph_case
    rng = np.random.default_rng(seed)
    pb = _pb(orc)
    out = []
    for tc in (4, 6, 7):
        Pl, Pr = mph_case(tc)
        Q = orc.prim2cons(pb, np.array([Pl, Pr]))
        for w in (0.25, 0.5, 0.75):
            out.append(w * Q[0] + (1 - w) * Q[1])
    while len(out) < n:
        row = []
        a1 = rng.uniform(0.05, 0.95)
        for a, strain in ((a1, 0.04), (1 - a1, 0.02)):
            F = np.eye(3) + strain * rng.standard_normal((3, 3))
            row += [a, 8.93 / np.linalg.det(F), *rng.uniform(-0.3, 0.3, 3), rng.uniform(0, 5e-4),
                    *F.reshape(-1, order="F")]
        out.append(orc.prim2cons(pb, np.array(row)))
    return np.array(out[:n])


def _pressures(orc, Q):
    """Each phase's mean-stress pressure -tr(sigma)/3 from the oracle's stress."""
    pb = _pb(orc)
    Pm = orc.cons2prim(pb, Q)
    eos = (orc.barton2009(), orc.barton2009(b0=B0_SOFT))
    out = []
    for k in range(2):
        sig = orc.stress(eos[k], Pm[:, 15 * k + 5], Pm[:, 15 * k + 6:15 * k + 15])
        out.append(-(sig[:, 0] + sig[:, 4] + sig[:, 8]) / 3.0)
    return np.array(out).T


def _invariants(Q):
    mass = [Q[:, 15 * k + 2:15 * k + 5] for k in range(2)]
    return Q[:, 0] + Q[:, 15], Q[:, 5] + Q[:, 20], mass


def test_oracle_relaxation_invariants(orc):
    Q = _states(orc, 40)
    R, st = orc.relax(_pb(orc), Q)
    assert np.all(st == 0)
    a0, E0, mom0 = _invariants(Q)
    a1, E1, mom1 = _invariants(R)
    assert np.max(np.abs(a1 - a0)) <= 4e-16
    assert np.max(np.abs(E1 - E0) / np.abs(E0)) <= 1e-13  # mixture total energy
    for k in range(2):
        assert np.array_equal(mom1[k], mom0[k])  # each phase's momentum is untouched
    # each phase's mass alpha_k rho_k (rho from det(alpha rho A / alpha)) is kept
    pb = _pb(orc)
    P0, P1 = orc.cons2prim(pb, Q), orc.cons2prim(pb, R)
    for k in range(2):
        m0, m1 = P0[:, 15 * k] * P0[:, 15 * k + 1], P1[:, 15 * k] * P1[:, 15 * k + 1]
        assert np.max(np.abs(m1 - m0) / m0) <= 1e-13
    p0, p1 = _pressures(orc, Q), _pressures(orc, R)
    assert np.min(np.abs(p0[:, 0] - p0[:, 1])) > 1e-3  # the inputs are out of equilibrium
    scale = np.maximum(np.abs(p1).max(axis=1), 8.93 * 4.6 ** 2 * 1e-3)
    assert np.max(np.abs(p1[:, 0] - p1[:, 1]) / scale) <= 1e-10  # one pressure afterwards
    # relaxing the relaxed state is a no-op (to rounding)
    R2, st2 = orc.relax(pb, R)
    assert np.all(st2 == 0)
    assert np.max(np.abs(R2 - R) / np.maximum(np.abs(R).max(axis=0), 1e-300)) <= 1e-12


def test_vanishing_phase_is_left_alone(orc):
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    import hyperelasticsolver_gb300 as h
    pb = _pb(orc)
    Pm = mph_interface_prims(h.Barton2009(), 64)
    Q = orc.prim2cons(pb, Pm)
    R, st = orc.relax(pb, Q)
    pure = np.minimum(Q[:, 0], Q[:, 15]) < 1e-5
    assert pure.sum() >= 32 and np.all(st == 0)
    assert np.array_equal(R[pure], Q[pure])


def test_product_code_matches_oracle(shim, orc):  # noqa: F811
    """hyp_relax.cuh (closed-form dp/de) compiled for the host against the oracle
    (dual-number stress, differenced dp/de): the same root to rounding."""
    shim.hs_relax2.restype = ctypes.c_int
    Q = _states(orc, 40, seed=5)
    R, st = orc.relax(_pb(orc), Q)
    got = np.array(Q, copy=True)
    for i in range(len(Q)):
        row = np.ascontiguousarray(got[i])
        assert shim.hs_relax2(P(EP1), P(EP2), row.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
        got[i] = row
    scale = np.maximum(np.abs(R).max(axis=0), 1e-300)
    assert np.max(np.abs(got - R) / scale) <= 1e-11


def test_closed_form_pressure_derivative(shim, orc):  # noqa: F811
    """dp/de at fixed distortion (closed form) against a central difference of the
    product's own pressure, and the pressure against the oracle's mean stress."""
    rng = np.random.default_rng(9)
    eos = orc.barton2009()
    for _ in range(20):
        A = (np.eye(3) + 0.05 * rng.standard_normal((3, 3))).reshape(-1, order="F")
        lam = rng.uniform(0.97, 1.03)
        S = rng.uniform(0, 1e-3)
        G = orc.finger(lam * A)
        e = orc.energy(eos, S, G)
        buf = np.zeros(2)
        shim.hs_relax_pressure(P(EP1), P(A), ctypes.c_double(lam), ctypes.c_double(e),
                               buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        sig = orc.stress(eos, S, lam * A)
        p_ref = -(sig[0] + sig[4] + sig[8]) / 3.0
        assert abs(buf[0] - p_ref) <= 1e-11 * max(abs(p_ref), 1.0)
        h = 1e-6 * max(abs(e), 1e-3)
        up, dn = np.zeros(2), np.zeros(2)
        for v, d in ((up, h), (dn, -h)):
            shim.hs_relax_pressure(P(EP1), P(A), ctypes.c_double(lam), ctypes.c_double(e + d),
                                   v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert abs(buf[1] - (up[0] - dn[0]) / (2 * h)) <= 1e-6 * max(abs(buf[1]), 1.0)


def test_mechanical_relaxation_invariants(orc):
    """Velocity then pressure relaxation: one velocity and one pressure afterwards; the
    mixture's momentum and total energy and each phase's mass kept; the velocity step
    only adds internal energy (|u_k - u*|^2 / 2 per phase)."""
    Q = _states(orc, 40, seed=7)
    pb = _pb(orc, relax=2)
    R, st = orc.relax(pb, Q)
    assert np.all(st == 0)
    mom0 = Q[:, 2:5] + Q[:, 17:20]
    mom1 = R[:, 2:5] + R[:, 17:20]
    assert np.max(np.abs(mom1 - mom0) / np.abs(mom0).max()) <= 1e-14
    E0, E1 = Q[:, 5] + Q[:, 20], R[:, 5] + R[:, 20]
    assert np.max(np.abs(E1 - E0) / np.abs(E0)) <= 1e-13
    P1 = orc.cons2prim(pb, R)
    assert np.max(np.abs(P1[:, 2:5] - P1[:, 17:20])) <= 1e-14 * np.abs(P1[:, 2:5]).max()
    p1 = _pressures(orc, R)
    scale = np.maximum(np.abs(p1).max(axis=1), 8.93 * 4.6 ** 2 * 1e-3)
    assert np.max(np.abs(p1[:, 0] - p1[:, 1]) / scale) <= 1e-10


def test_mechanical_relaxation_keeps_the_interface_run_bounded(orc):
    """The smoothed-interface workload (alpha_1 from 1 - 1e-6 to 1e-6 over 8 cells) on 256
    cells for 300 HLL steps: with velocity and pressure relaxed every cell keeps a positive
    determinant and finite values, where pressure relaxation alone lets the phases'
    velocities drift apart and the minority phase's density collapse."""
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    import hyperelasticsolver_gb300 as h
    nx = 256
    pb = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, nx=nx, cfl=0.5, relax=2,
                     eos=(orc.barton2009(), orc.barton2009(b0=B0_SOFT)))
    Q = np.ascontiguousarray(orc.prim2cons(pb, mph_interface_prims(h.Barton2009(), nx)).T)
    Q, steps, _, _ = orc.run(pb, Q, max_steps=300, nthreads=4)
    assert steps == 300 and np.all(np.isfinite(Q))
    assert np.max(np.abs(Q[0] + Q[15] - 1.0)) <= 1e-12

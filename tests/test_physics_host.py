"""The product's closed-form physics (hyp_physics.cuh, compiled for the host by
g++) against the oracle's dual-number restatement. CPU only: checks the
derivation of the acoustic tensor, stress and eigen-solve without a GPU."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from helpers import rel_err

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def shim():
    d = tempfile.mkdtemp(prefix="hyp_shim_")
    so = os.path.join(d, "shim.so")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-o", so,
                        os.path.join(HERE, "host_physics_shim.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(so)
    for n in ("hs_energy", "hs_entropy", "hs_spectral_radius"):
        getattr(L, n).restype = ctypes.c_double
    L.hs_cell1_vjp.restype = ctypes.c_int
    L.hs_hank_energy.restype = ctypes.c_double
    return L


def P(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))


EOS = [(8.93, 4.6, 3.9e-4, 300, 2.1, 1, 3, 2), (8.93, 6.22, 9.0e-4, 300, 3.16, 1, 3.577, 2.088)]


@pytest.mark.parametrize("ep", EOS)
def test_closed_forms_match_dual_numbers(shim, orc, ep):
    e = orc.barton2009(*ep)
    ea = np.array(ep, dtype=np.float64)
    rng = np.random.default_rng(11)
    worst = {}
    for _ in range(150):
        F = np.eye(3) + 0.1 * rng.standard_normal((3, 3))
        if np.linalg.det(F) <= 0:
            continue
        F = F.reshape(-1, order="F")
        S = rng.uniform(0, 2e-3)
        out = np.zeros(9)
        shim.hs_stress(P(ea), ctypes.c_double(S), P(F), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        worst["stress"] = max(worst.get("stress", 0), rel_err(out, orc.stress(e, S, F)))
        ac_ref = orc.acoustic(e, S, F)
        shim.hs_acoustic(P(ea), ctypes.c_double(S), P(F), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        worst["acoustic"] = max(worst.get("acoustic", 0), rel_err(out, ac_ref))
        sr = shim.hs_spectral_radius(P(ac_ref))
        ref = np.max(np.abs(np.linalg.eigvals(ac_ref.reshape(3, 3, order="F"))))
        worst["radius"] = max(worst.get("radius", 0), abs(sr - ref) / ref)
        G = orc.finger(F)
        worst["energy"] = max(worst.get("energy", 0),
                              abs(shim.hs_energy(P(ea), ctypes.c_double(S), P(G)) - orc.energy(e, S, G))
                              / max(abs(orc.energy(e, S, G)), 1e-3))
    assert worst["stress"] < 1e-12, worst
    assert worst["acoustic"] < 1e-12, worst
    assert worst["radius"] < 1e-13, worst
    assert worst["energy"] < 1e-12, worst


def test_cell_flux_and_speed(shim, orc):
    e = orc.barton2009()
    ea = np.array(EOS[0], dtype=np.float64)
    pb = orc.problem()
    rng = np.random.default_rng(5)
    for _ in range(100):
        F = np.eye(3) + 0.08 * rng.standard_normal((3, 3))
        if np.linalg.det(F) <= 0:
            continue
        Pr = np.array([8.93 / np.linalg.det(F), *rng.uniform(-1, 1, 3), rng.uniform(0, 1e-3), *F.reshape(-1, order="F")])
        Q = orc.prim2cons(pb, Pr)
        out = np.zeros(18)
        shim.hs_cell(P(ea), P(np.concatenate([[1.0], Q])), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert out[17] == 0
        assert rel_err(out[:14], orc.flux(pb, Q)) < 1e-12
        lam = np.max(np.abs(orc.speeds(pb, Q)))
        assert abs(abs(out[14]) + out[15] - lam) < 1e-13 * lam
    # an inverted distortion raises the negative-determinant status
    Qbad = orc.prim2cons(pb, np.array([8.93, 0, 0, 0, 0, *np.eye(3).reshape(-1)]))
    Qbad[5:] = -Qbad[5:]
    out = np.zeros(18)
    shim.hs_cell(P(ea), P(np.concatenate([[1.0], Qbad])), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert int(out[17]) & 1


def _ep_moduli(ep, db0sq=0.0, dk0=0.0):
    ep = np.array(ep, dtype=np.float64)
    b0sq = ep[4] ** 2 + db0sq
    k0 = ep[1] ** 2 - 4 / 3 * ep[4] ** 2 + dk0
    ep[4], ep[1] = np.sqrt(b0sq), np.sqrt(k0 + 4 / 3 * b0sq)
    return ep


@pytest.mark.parametrize("ep", EOS)
def test_cell_vjp_matches_central_differences(shim, ep):
    """The hand-written reverse pass of the cell flux and wave speed (hyp_adjoint.cuh)
    against central differences of the forward cell functions, for the 14 state
    components and the moduli b0sq, k0 (each with the other held fixed)."""
    ea = np.array(ep, dtype=np.float64)

    def cell(e, q):
        o = np.zeros(15)
        shim.hs_cell1(P(e), P(q), P(o))
        return o

    rng = np.random.default_rng(7)
    for trial in range(12):
        A = np.eye(3) + 0.08 * rng.standard_normal((3, 3))
        p = np.concatenate([[ep[0] * np.exp(0.05 * rng.standard_normal())], rng.standard_normal(3),
                            [1e-4 * abs(rng.standard_normal()) * (trial % 2)], A.reshape(-1, order="F")])
        q = np.zeros(14)
        shim.hs_prim2cons1(P(ea), P(p), P(q))
        w = rng.standard_normal(15)
        qb, eb = np.zeros(14), np.zeros(2)
        shim.hs_cell1_vjp(P(ea), P(q), P(w[:14]), ctypes.c_double(w[14]), P(qb), P(eb))
        phi = lambda qq, e=ea: w @ cell(e, qq)
        fd = np.zeros(14)
        for t in range(14):
            hq = 1e-6 * max(1.0, abs(q[t]))
            d = np.zeros(14)
            d[t] = hq
            fd[t] = (phi(q + d) - phi(q - d)) / (2 * hq)
        fe = np.array([(phi(q, _ep_moduli(ep, db0sq=1e-5)) - phi(q, _ep_moduli(ep, db0sq=-1e-5))) / 2e-5,
                       (phi(q, _ep_moduli(ep, dk0=1e-5)) - phi(q, _ep_moduli(ep, dk0=-1e-5))) / 2e-5])
        assert np.max(np.abs(qb - fd)) <= 1e-7 * np.max(np.abs(fd)), (trial, qb, fd)
        assert np.max(np.abs(eb - fe)) <= 1e-7 * np.max(np.abs(fe)), (trial, eb, fe)


def test_prim2cons_vjp_matches_central_differences(shim):
    ea = np.array(EOS[0], dtype=np.float64)

    def p2c(e, p):
        o = np.zeros(14)
        shim.hs_prim2cons1(P(e), P(p), P(o))
        return o

    rng = np.random.default_rng(8)
    for trial in range(8):
        A = np.eye(3) + 0.08 * rng.standard_normal((3, 3))
        p = np.concatenate([[8.9], rng.standard_normal(3), [0.0], A.reshape(-1, order="F")])
        qb = rng.standard_normal(14)
        pb, eb = np.zeros(14), np.zeros(2)
        shim.hs_prim2cons1_vjp(P(ea), P(p), P(qb), P(pb), P(eb))
        phi = lambda pp, e=ea: qb @ p2c(e, pp)
        fd = np.zeros(14)
        for t in range(14):
            hp = 1e-6 * max(1.0, abs(p[t])) if t != 4 else 1e-9  # S is on the scale of cv = 3.9e-4
            d = np.zeros(14)
            d[t] = hp
            fd[t] = (phi(p + d) - phi(p - d)) / (2 * hp)
        fe = np.array([(phi(p, _ep_moduli(EOS[0], db0sq=1e-5)) - phi(p, _ep_moduli(EOS[0], db0sq=-1e-5))) / 2e-5,
                       (phi(p, _ep_moduli(EOS[0], dk0=1e-5)) - phi(p, _ep_moduli(EOS[0], dk0=-1e-5))) / 2e-5])
        assert np.max(np.abs(pb - fd)) <= 1e-7 * np.max(np.abs(fd)), (trial, pb, fd)
        assert np.max(np.abs(eb - fe)) <= 1e-7 * np.max(np.abs(fe)), (trial, eb, fe)


def test_hank2016_closed_form_matches_dual_numbers(shim, orc):
    """Hank2016 stress in closed form (hyp_hank.cuh) against the oracle's dual-number
    gradient (EquationsOfState.jl:354-361), and the energy."""
    h = np.array([2.7, 26e9, 3.4, 21.5e9, 0.5])
    ho = orc.hank2016()
    rng = np.random.default_rng(12)
    for _ in range(20):
        F = (np.eye(3) + 0.05 * rng.standard_normal((3, 3))).reshape(-1, order="F")
        den, pres = 2.7 * rng.uniform(0.9, 1.1), rng.uniform(-1e9, 5e9)
        sig = np.zeros(9)
        shim.hs_hank_stress(P(h), ctypes.c_double(den), ctypes.c_double(pres), P(F), P(sig))
        ref = orc.hank_stress(ho, den, pres, F)
        assert np.max(np.abs(sig - ref)) <= 1e-12 * np.max(np.abs(ref))
        G = orc.finger(F)
        e = shim.hs_hank_energy(P(h), ctypes.c_double(den), ctypes.c_double(pres), P(G))
        assert abs(e - orc.hank_energy(ho, den, pres, G)) <= 1e-13 * abs(e)


def test_spectral_radius_on_hard_spectra(shim):
    """The spectral radius (FP32 seeds and three Newton steps when the top root
    separates by 10 %, Jacobi rotations for a symmetric matrix otherwise, deflation
    for a general one) against numpy: symmetric matrices with well separated,
    nearly equal (relative gaps 1e-3 ... 1e-12) and repeated top eigenvalues,
    negative dominant eigenvalues, and general matrices whose complex pair is the
    larger or the smaller in modulus."""
    rng = np.random.default_rng(40)
    worst = 0.0

    def check(m, tol):
        nonlocal worst
        a = np.ascontiguousarray(m.reshape(-1, order="F"))
        ref = np.max(np.abs(np.linalg.eigvals(m)))
        err = abs(shim.hs_spectral_radius(P(a)) - ref) / ref
        worst = max(worst, err)
        assert err < tol, (m, err)

    for gap in [0.5, 1e-1, 1e-3, 1e-6, 1e-9, 1e-12, 0.0]:
        for sign in (1.0, -1.0):
            for _ in range(20):
                Qm, _r = np.linalg.qr(rng.standard_normal((3, 3)))
                top = rng.uniform(1, 50)
                lam = sign * np.array([top, top * (1 - gap), rng.uniform(-0.5, 0.5) * top])
                check(Qm @ np.diag(lam) @ Qm.T, 1e-13)
    for _ in range(200):  # general real matrices: a real root and a complex pair
        th = rng.uniform(0.1, 3.0)
        rad, r = rng.uniform(0.5, 5.0), rng.uniform(-5.0, 5.0)
        B = np.array([[rad * np.cos(th), -rad * np.sin(th), 0], [rad * np.sin(th), rad * np.cos(th), 0], [0, 0, r]])
        S = rng.standard_normal((3, 3)) + 3 * np.eye(3)
        check(S @ B @ np.linalg.inv(S), 1e-11)
    print(f"spectral radius worst relative error {worst:.1e}")


def test_eigen_moduli_with_repeated_roots(shim):
    """All three moduli (the function-level get_eigvals): symmetric matrices with a
    repeated pair -- the acoustic tensor at rest has c0^2 once and b0^2 twice --
    agree with numpy to a few ulps of the largest."""
    rng = np.random.default_rng(41)
    worst = 0.0
    out = np.zeros(3)
    for lam in ([4.6 ** 2, 2.1 ** 2, 2.1 ** 2], [3.0, 3.0, 3.0], [5.0, 5.0, -1.0], [1.0, 1.0 + 1e-9, 0.2]):
        for _ in range(30):
            Qm, _r = np.linalg.qr(rng.standard_normal((3, 3)))
            m = Qm @ np.diag(lam) @ Qm.T
            a = np.ascontiguousarray(m.reshape(-1, order="F"))
            shim.hs_eig_moduli3(P(a), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
            ref = np.sort(np.abs(np.linalg.eigvalsh(m)))[::-1]
            worst = max(worst, np.max(np.abs(out - ref)) / ref[0])
    assert worst < 1e-14, worst

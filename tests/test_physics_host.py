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

"""Writes tests/golden/golden_literal.json: 40-digit values of the reference's
functions from the independent transliteration oracle/literal.py, for seeded
inputs. Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np
import mpmath as mp

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
from oracle import literal as L  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_literal.json")


def f(x):
    return float(L.val(x))


def main():
    rng = np.random.default_rng(20261203)
    e = L.Barton()
    e2 = L.Barton(b0=2.1 * np.sqrt(0.1))
    g = {"eos": [8.93, 4.6, 3.9e-4, 300, 2.1, 1, 3, 2], "eos2_b0": 2.1 * float(np.sqrt(0.1)), "tensors": [],
         "cells": [], "noncons": [], "hll": [], "rusanov": {}, "lxf2": [], "hank": []}
    # tensor-level functions
    for k in range(6):
        F = np.eye(3) + 0.08 * rng.standard_normal((3, 3))
        if np.linalg.det(F) <= 0:
            F = np.eye(3)
        Fv = [float(x) for x in F.reshape(-1, order="F")]
        S = float(rng.uniform(0, 1.5e-3)) if k else 0.0
        Fm = [mp.mpf(x) for x in Fv]
        G = L.finger(Fm)
        ac = L.acoustic(e, mp.mpf(S), Fm)
        g["tensors"].append({
            "F": Fv, "S": S,
            "finger": [f(x) for x in G],
            "invariants": [f(x) for x in L.invariants(G)],
            "energy": f(L.energy(e, mp.mpf(S), G)),
            "stress": [f(x) for x in L.stress(e, mp.mpf(S), Fm)],
            "acoustic": [f(x) for x in ac],
            "moduli": [float(x) for x in L.eig_moduli(ac)],
        })
    # single-phase cells (alpha = 1)
    for k in range(4):
        F = np.eye(3) + 0.05 * rng.standard_normal((3, 3))
        u = rng.uniform(-1, 1, 3)
        S = float(rng.uniform(0, 1e-3))
        rho = 8.93 / np.linalg.det(F)
        P = [1.0, rho, *u, S, *F.reshape(-1, order="F")]
        Pm = [mp.mpf(float(x)) for x in P]
        Q = L.prim2cons(e, Pm)
        g["cells"].append({
            "P": [float(x) for x in P],
            "Q": [f(x) for x in Q],
            "prim": [f(x) for x in L.cons2prim(e, Q)],
            "flux": [f(x) for x in L.flux(e, Q)],
            "speeds": [float(x) for x in L.speeds(e, Q)],
        })
    # two-phase non-conservative columns and an HLL face (test case 6 states, mixed)
    from hyperelasticsolver_gb300._cases import mph_case
    Pl, Pr = mph_case(6)
    eos = (e, e2)
    Ql = L.prim2cons(eos[0], [mp.mpf(float(x)) for x in Pl[:15]]) + L.prim2cons(eos[1], [mp.mpf(float(x)) for x in Pl[15:]])
    Qr = L.prim2cons(eos[0], [mp.mpf(float(x)) for x in Pr[:15]]) + L.prim2cons(eos[1], [mp.mpf(float(x)) for x in Pr[15:]])
    Ql = [mp.mpf(float(x)) for x in Ql]
    Qr = [mp.mpf(float(x)) for x in Qr]
    Qmix = [(a * 3 + b) / 4 for a, b in zip(Ql, Qr)]
    Qmix = [mp.mpf(float(x)) for x in Qmix]
    g["noncons"].append({"Q": [float(x) for x in Qmix], "bcol": [f(x) for x in L.noncons_cols(eos, Qmix)]})
    spdL = L.speeds(eos[0], Ql[:15]) + L.speeds(eos[1], Ql[15:])
    spdR = L.speeds(eos[0], Qr[:15]) + L.speeds(eos[1], Qr[15:])
    dm, dp = L.hll(eos, Ql, Qr, spdL, spdR)
    g["hll"].append({"Ql": [float(x) for x in Ql], "Qr": [float(x) for x in Qr],
                     "spdL": [float(x) for x in spdL], "spdR": [float(x) for x in spdR],
                     "dm": [f(x) for x in dm], "dp": [f(x) for x in dp]})
    # two Rusanov steps on 6 cells (single phase, frozen ends)
    cells = []
    for k in range(6):
        F = np.eye(3) + 0.03 * rng.standard_normal((3, 3))
        u = rng.uniform(-0.5, 0.5, 3)
        P = [1.0, 8.93 / np.linalg.det(F), *u, 0.0, *F.reshape(-1, order="F")]
        Q = L.prim2cons(e, [mp.mpf(float(x)) for x in P])
        cells.append([mp.mpf(float(x)) for x in Q[1:]])
    g["rusanov"]["Q0"] = [[float(x) for x in c] for c in cells]
    Q = cells
    dts = []
    for _ in range(2):
        Q, dt = L.rusanov_step(e, Q, mp.mpf("0.5"))
        dts.append(float(dt))
    g["rusanov"]["Q2"] = [[float(x) for x in c] for c in Q]
    g["rusanov"]["dt"] = dts
    # the two-phase LxF face (Gauss-Lobatto path integral) on the test case 6 states
    lam = mp.mpf(12)
    cons, dm, dp = L.lxf2(eos, Ql, Qr, lam)
    g["lxf2"] = [{"Ql": [float(x) for x in Ql], "Qr": [float(x) for x in Qr], "lam": float(lam),
                  "cons": [f(x) for x in cons], "dm": [f(x) for x in dm], "dp": [f(x) for x in dp]}]
    # Hank2016 energy / pressure / stress at seeded states
    h = L.Hank()
    g["hank"] = []
    for k in range(3):
        F = np.eye(3) + 0.05 * rng.standard_normal((3, 3))
        Fv = [float(x) for x in F.reshape(-1, order="F")]
        den = float(2.7 * rng.uniform(0.95, 1.05))
        pres = float(rng.uniform(0.0, 2e9))
        Fm = [mp.mpf(x) for x in Fv]
        G = L.finger(Fm)
        inv = L.invariants(G)
        e_int = L.hank_energy(h, mp.mpf(den), mp.mpf(pres), G)
        g["hank"].append({"F": Fv, "den": den, "pres": pres, "G": [f(x) for x in G],
                          "energy": f(e_int), "invariants": [f(x) for x in inv],
                          "pressure": f(L.hank_pressure(h, mp.mpf(den), e_int, inv)),
                          "stress": [f(x) for x in L.hank_stress(h, mp.mpf(den), mp.mpf(pres), Fm)]})
    # the alternative Barton2009 parameters of main.jl:133 (non-integer beta, gamma: the
    # general powers), from their own generator so the entries above keep their inputs
    alt = [8.93, 6.22, 9.0e-4, 300, 3.16, 1, 3.577, 2.088]
    ea = L.Barton(*alt)
    ra = np.random.default_rng(20261204)
    g["nondefault"] = {"eos": alt, "tensors": [], "cells": []}
    for k in range(4):
        F = np.eye(3) + 0.06 * ra.standard_normal((3, 3))
        if np.linalg.det(F) <= 0:
            F = np.eye(3)
        Fv = [float(x) for x in F.reshape(-1, order="F")]
        S = float(ra.uniform(0, 1.5e-3))
        Fm = [mp.mpf(x) for x in Fv]
        G = L.finger(Fm)
        ac = L.acoustic(ea, mp.mpf(S), Fm)
        g["nondefault"]["tensors"].append({
            "F": Fv, "S": S, "energy": f(L.energy(ea, mp.mpf(S), G)),
            "stress": [f(x) for x in L.stress(ea, mp.mpf(S), Fm)],
            "acoustic": [f(x) for x in ac], "moduli": [float(x) for x in L.eig_moduli(ac)]})
    for k in range(3):
        F = np.eye(3) + 0.05 * ra.standard_normal((3, 3))
        u = ra.uniform(-1, 1, 3)
        S = float(ra.uniform(0, 1e-3))
        P = [1.0, 8.93 / np.linalg.det(F), *u, S, *F.reshape(-1, order="F")]
        Q = L.prim2cons(ea, [mp.mpf(float(x)) for x in P])
        g["nondefault"]["cells"].append({
            "P": [float(x) for x in P], "Q": [f(x) for x in Q],
            "flux": [f(x) for x in L.flux(ea, Q)], "speeds": [float(x) for x in L.speeds(ea, Q)]})
    # a two-phase HLL face (test case 6 states) with phase 1 on the alternative parameters
    eosa = (ea, e2)
    Qla = [mp.mpf(float(x)) for x in L.prim2cons(ea, [mp.mpf(float(x)) for x in Pl[:15]])
           + L.prim2cons(e2, [mp.mpf(float(x)) for x in Pl[15:]])]
    Qra = [mp.mpf(float(x)) for x in L.prim2cons(ea, [mp.mpf(float(x)) for x in Pr[:15]])
           + L.prim2cons(e2, [mp.mpf(float(x)) for x in Pr[15:]])]
    sL = L.speeds(ea, Qla[:15]) + L.speeds(e2, Qla[15:])
    sR = L.speeds(ea, Qra[:15]) + L.speeds(e2, Qra[15:])
    dm, dp = L.hll(eosa, Qla, Qra, sL, sR)
    g["nondefault"]["hll"] = {"Ql": [float(x) for x in Qla], "Qr": [float(x) for x in Qra],
                              "spdL": [float(x) for x in sL], "spdR": [float(x) for x in sR],
                              "dm": [f(x) for x in dm], "dp": [f(x) for x in dp]}
    # function-level forms beside the step's path, from their own generator so the entries
    # above keep their inputs: acoustic(eos, ent, F, n) for general n, stress(eos, den,
    # e_int, F) (one state at the entropy clamp), acoustic(eos, P, n), get_eigvals along n,
    # and an HLL face given speeds wider than its cells' own (NumFluxes.jl:90-91)
    rx = np.random.default_rng(20261205)
    x = {"acoustic_dir": [], "stress_den": [], "acoustic_prim": [], "speeds_dir": []}
    for k in range(3):
        F = np.eye(3) + 0.06 * rx.standard_normal((3, 3))
        Fv = [float(v) for v in F.reshape(-1, order="F")]
        S = float(rx.uniform(0, 1.5e-3))
        nv = [float(v) for v in rx.standard_normal(3)]
        ac = L.acoustic(e, mp.mpf(S), [mp.mpf(v) for v in Fv], [mp.mpf(v) for v in nv])
        x["acoustic_dir"].append({"F": Fv, "S": S, "n": nv, "acoustic": [f(v) for v in ac]})
    for k in range(3):
        F = np.eye(3) + 0.06 * rx.standard_normal((3, 3))
        Fv = [float(v) for v in F.reshape(-1, order="F")]
        den = float(rx.uniform(8.5, 9.3))
        Fm = [mp.mpf(v) for v in Fv]
        eint = L.energy(e, mp.mpf(float(rx.uniform(0, 1e-3))), L.finger(Fm)) - (1 if k == 2 else 0)
        eint = float(eint)
        x["stress_den"].append({"F": Fv, "den": den, "e_int": eint,
                                "stress": [f(v) for v in L.stress_den(e, mp.mpf(den), mp.mpf(eint), Fm)]})
    for k in range(3):
        F = np.eye(3) + 0.05 * rx.standard_normal((3, 3))
        P = [float(rx.uniform(0.3, 1.0)), 8.93 / float(np.linalg.det(F)), *[float(v) for v in rx.uniform(-0.5, 0.5, 3)],
             float(rx.uniform(0, 1e-3)), *[float(v) for v in F.reshape(-1, order="F")]]
        nv = [1.0, 0.0, 0.0] if k == 0 else [float(v) for v in rx.standard_normal(3)]
        ac = L.acoustic_prim(e, [mp.mpf(v) for v in P], [mp.mpf(v) for v in nv])
        x["acoustic_prim"].append({"P": P, "n": nv, "acoustic": [f(v) for v in ac]})
    for k in range(3):
        F = np.eye(3) + 0.05 * rx.standard_normal((3, 3))
        u = rx.uniform(-1, 1, 3)
        S = float(rx.uniform(0, 1e-3))
        P = [1.0, 8.93 / np.linalg.det(F), *u, S, *F.reshape(-1, order="F")]
        Q = L.prim2cons(e, [mp.mpf(float(v)) for v in P])
        Q = [mp.mpf(f(v)) for v in Q]
        nv = [float(v) for v in rx.standard_normal(3)]
        x["speeds_dir"].append({"Q": [float(v) for v in Q], "n": nv,
                                "speeds": [f(v) for v in L.speeds(e, Q, [mp.mpf(v) for v in nv])]})
    wl = [float(v) - 1.5 for v in spdL]
    wr = [float(v) + 2.5 for v in spdR]
    dmw, dpw = L.hll(eos, Ql, Qr, [mp.mpf(v) for v in wl], [mp.mpf(v) for v in wr])
    x["hll_given"] = {"Ql": [float(v) for v in Ql], "Qr": [float(v) for v in Qr], "spdL": wl, "spdR": wr,
                      "dm": [f(v) for v in dmw], "dp": [f(v) for v in dpw]}
    g["extras"] = x
    with open(OUT, "w") as fh:
        json.dump(g, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()

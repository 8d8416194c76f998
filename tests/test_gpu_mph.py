"""Parity of the two-phase FP64 CUDA path (path-conservative HLL, volume-fraction
and interface terms) with the oracle (GPU), at RTOL_FP64 = 1e-12."""
import numpy as np
import pytest

from helpers import RTOL_FP64, assert_close, assert_close_soa, assert_within_sensitivity, ulp_sensitivity

pytestmark = pytest.mark.gpu

B0_SOFT = 2.1 * np.sqrt(0.1)  # phase 2: shear modulus b0^2 scaled by 0.1, c0 held


def eos_pair(hyp):
    return (hyp.Barton2009(), hyp.Barton2009(_b0=B0_SOFT))


def oracle_pb(orc, nx=3, cfl=0.5, bc=0, flux=None):
    return orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL if flux is None else flux, nx=nx, cfl=cfl, bc=bc,
                       eos=(orc.barton2009(), orc.barton2009(b0=B0_SOFT)))


def random_mph(orc, n, rng):
    """Random two-phase primitive states: alpha1 in (0.05, 0.95), per-phase strain and velocity."""
    out = []
    while len(out) < n:
        row = []
        a1 = rng.uniform(0.05, 0.95)
        for a in (a1, 1 - a1):
            F = np.eye(3) + 0.04 * rng.standard_normal((3, 3))
            if np.linalg.det(F) <= 0.5:
                break
            row += [a, 8.93 / np.linalg.det(F), *rng.uniform(-0.4, 0.4, 3), rng.uniform(0, 5e-4),
                    *F.reshape(-1, order="F")]
        if len(row) == 30:
            out.append(row)
    return orc.prim2cons(oracle_pb(orc), np.array(out))


def test_twophase_evaluators(hyp, orc):
    from hyperelasticsolver_gb300 import HyperelasticityMPh as H, NumFluxes as NF
    rng = np.random.default_rng(5)
    Q = random_mph(orc, 64, rng)
    eos, pb = eos_pair(hyp), oracle_pb(orc)
    assert_close(H.flux_mph(eos, Q), orc.flux(pb, Q), RTOL_FP64, "flux_mph")
    eg, eo = H.get_eigvals(eos, Q), orc.speeds(pb, Q)
    for ph in (slice(0, 6), slice(6, 12)):  # all twelve speeds, each phase to its largest |speed|
        scale = np.max(np.abs(eo[:, ph]), axis=1, keepdims=True)
        assert np.max(np.abs(eg[:, ph] - eo[:, ph]) / scale) <= RTOL_FP64, "get_eigvals"
    B = H.noncons_flux(eos, Q)
    bo = orc.noncons(pb, Q)
    assert_close(B[:, :15, 0], bo[:, :15], RTOL_FP64, "B column 1")
    assert_close(B[:, 15:, 15], bo[:, 15:], RTOL_FP64, "B column 16")
    Ql, Qr = Q[:-1], Q[1:]
    # D-, D+ sum flux differences and path integrals that cancel: each component is held to
    # 1e-12 of its largest value over the faces or to the oracle's one-ulp spread (measured)
    _, dm, dp = NF.hll(eos, Ql, Qr)
    dmo, dpo = orc.hll(pb, Ql, Qr, eo[:-1], eo[1:])
    for k, (got, ref) in enumerate(((dm, dmo), (dp, dpo))):
        sens = ulp_sensitivity(lambda a, b: orc.hll(pb, a, b, orc.speeds(pb, a), orc.speeds(pb, b))[k], (Ql, Qr))
        assert_within_sensitivity(got, ref, sens, RTOL_FP64, f"hll D{'-+'[k]}", axis=0)
    lam = rng.uniform(5.0, 8.0, len(Ql))
    cons, dm, dp = NF.lxf(eos, Ql, Qr, lam)
    pbl = oracle_pb(orc, flux=orc.FLUX_LXF)
    co, dmo, dpo = orc.lxf(pbl, Ql, Qr, lam)
    assert_close(cons, co, RTOL_FP64, "two-phase lxf cons")
    for k, (got, ref) in enumerate(((dm, dmo), (dp, dpo))):
        sens = ulp_sensitivity(lambda a, b: orc.lxf(pbl, a, b, lam)[1 + k], (Ql, Qr))
        assert_within_sensitivity(got, ref, sens, RTOL_FP64, f"two-phase lxf D{'-+'[k]}", axis=0)


def test_golden_hll_face_on_gpu(hyp, orc):
    import json
    import os
    from hyperelasticsolver_gb300 import HyperelasticityMPh as H, NumFluxes as NF
    with open(os.path.join(os.path.dirname(__file__), "golden", "golden_literal.json")) as fh:
        g = json.load(fh)
    eos = (hyp.Barton2009(), hyp.Barton2009(_b0=g["eos2_b0"]))
    for c in g["noncons"]:
        B = H.noncons_flux(eos, np.array(c["Q"]))
        got = np.concatenate([B[:15, 0], B[15:, 15]])
        assert_close(got, c["bcol"], RTOL_FP64, "golden noncons")
    pb = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_HLL, eos=(orc.barton2009(), orc.barton2009(b0=g["eos2_b0"])))
    pbl = orc.problem(model=orc.MODEL_MULTI, flux=orc.FLUX_LXF, eos=(orc.barton2009(), orc.barton2009(b0=g["eos2_b0"])))
    faces = list(g["hll"]) + [dict(g["extras"]["hll_given"], given=True)]
    for h in faces:
        Ql, Qr = np.array(h["Ql"]), np.array(h["Qr"])
        sl, sr = np.array(h["spdL"]), np.array(h["spdR"])
        _, dm, dp = NF.hll(eos, Ql, Qr, [sl, sr]) if h.get("given") else NF.hll(eos, Ql, Qr)
        for k, (got, ref) in enumerate(((dm, h["dm"]), (dp, h["dp"]))):
            # the golden face's own conditioning, measured on the oracle (a one-ulp spread of the inputs)
            sens = ulp_sensitivity(lambda a, b, c, d: orc.hll(pb, a, b, c, d)[k], (Ql, Qr, sl, sr), trials=6)
            assert_within_sensitivity(got, ref, sens, RTOL_FP64, f"golden hll D{'-+'[k]}")
    for c in g["lxf2"]:
        Ql, Qr = np.array(c["Ql"]), np.array(c["Qr"])
        cons, dm, dp = NF.lxf(eos, Ql, Qr, c["lam"])
        assert_close(cons, c["cons"], RTOL_FP64, "golden lxf flux")
        for k, (got, ref) in enumerate(((dm, c["dm"]), (dp, c["dp"]))):
            sens = ulp_sensitivity(lambda a, b: orc.lxf(pbl, a, b, c["lam"])[1 + k], (Ql, Qr), trials=6)
            assert_within_sensitivity(got, ref, sens, RTOL_FP64, f"golden lxf D{'-+'[k]}")


@pytest.mark.parametrize("flux", ["hll", "lxf"])
@pytest.mark.parametrize("testcase", [4, 6, 7])
def test_reference_testcases_step(hyp, orc, testcase, flux):
    """The reference's two-phase Riemann test cases (HyperelasticityMPh.jl:275-426) on
    100 cells with the HLL flux (main.jl:225) or the path-conservative LxF flux
    (main.jl:223) and frozen ends (main.jl:178-227), 30 steps."""
    from hyperelasticsolver_gb300._cases import mph_case, initial_condition
    nx, steps = 100, 30
    pb = oracle_pb(orc, nx=nx, cfl=0.6, flux=orc.FLUX_HLL if flux == "hll" else orc.FLUX_LXF)
    Pl, Pr = mph_case(testcase)
    Q0 = initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx)
    Qo, so, to, _ = orc.run(pb, Q0, max_steps=steps)
    with hyp.Solver(eos_pair(hyp), nx, model="multi", flux=flux, cfl=0.6) as s:
        s.upload(Q0)
        n, t = s.step(max_steps=steps)
        assert n == steps and abs(t - to) <= RTOL_FP64 * to
        err = assert_close_soa(s.download(), Qo, RTOL_FP64, f"test case {testcase} ({flux})")
    print(f"two-phase test case {testcase} ({flux}), {steps} steps: max per-variable relative error {err:.2e}")


@pytest.mark.parametrize("flux", ["hll", "lxf"])
def test_smoothed_interface_transmissive(hyp, orc, flux):
    """Volume fraction going from 1 - 1e-6 to 1e-6 across 8 cells (tanh profile as
    main.jl:110-123), transmissive ends."""
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    nx, steps = 64, 12
    P = mph_interface_prims(hyp.Barton2009(), nx)
    pb = oracle_pb(orc, nx=nx, cfl=0.5, bc=orc.BC_TRANSMISSIVE,
                   flux=orc.FLUX_HLL if flux == "hll" else orc.FLUX_LXF)
    Q0 = np.ascontiguousarray(orc.prim2cons(pb, P).T)
    Qo, so, to, _ = orc.run(pb, Q0, max_steps=steps)
    with hyp.Solver(eos_pair(hyp), nx, model="multi", flux=flux, bc="transmissive", cfl=0.5) as s:
        s.upload(Q0)
        n, t = s.step(max_steps=steps)
        assert n == steps
        err = assert_close_soa(s.download(), Qo, RTOL_FP64, "smoothed interface")
    print(f"two-phase smoothed interface, {steps} steps: max per-variable relative error {err:.2e}")


def test_twophase_uniform_state_preserved(hyp, orc):
    rng = np.random.default_rng(8)
    q = random_mph(orc, 1, rng)[0]
    Q0 = np.ascontiguousarray(np.repeat(q[:, None], 4096, axis=1))
    with hyp.Solver(eos_pair(hyp), 4096, model="multi", flux="hll", bc="transmissive") as s:
        s.upload(Q0)
        s.step(max_steps=3)
        assert np.array_equal(s.download(), Q0)


def phase_densities(Q, rho0=8.93):
    """rho_true of both phases, sqrt(det(alpha rho A / alpha) / rho0) (HyperelasticityMPh.jl:113-114)."""
    out = []
    for p in range(2):
        a = Q[15 * p]
        m = Q[15 * p + 6:15 * p + 15] / a
        det = (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[3] * (m[1] * m[8] - m[7] * m[2])
               + m[6] * (m[1] * m[5] - m[4] * m[2]))
        out.append(np.sqrt(det / rho0))
    return out


def l1_linf(a, b):
    return np.sum(np.abs(a - b)) / np.sum(np.abs(b)), np.max(np.abs(a - b)) / np.max(np.abs(b))


KERNELS = ["tile", "pair"]  # face kernels with the phases in scalar FP32 / as packed FP32 pairs


def _mixed_kernel(s, prec, kernel):
    if prec == "mixed":
        s.set_mixed_kernel(kernel)


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("flux", ["hll", "lxf"])
@pytest.mark.parametrize("testcase", [4, 6, 7])
def test_mixed_twophase_vs_fp64(hyp, orc, testcase, flux, kernel):
    """Mixed-precision two-phase step (FP32 physics, compensated state, float-float
    cons2prim islands) against the FP64 two-phase step: relative L1 error of each
    phase's density <= 1e-6 after 100 steps of the reference's test cases."""
    from hyperelasticsolver_gb300._cases import mph_case, initial_condition
    nx, steps = 400, 100
    pb = oracle_pb(orc, nx=nx, cfl=0.6)
    Pl, Pr = mph_case(testcase)
    Q0 = initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx)
    out = {}
    for prec in ("fp64", "mixed"):
        with hyp.Solver(eos_pair(hyp), nx, model="multi", flux=flux, precision=prec, cfl=0.6) as s:
            _mixed_kernel(s, prec, kernel)
            s.upload(Q0)
            n, t = s.step(max_steps=steps)
            assert n == steps
            out[prec] = (s.download(), t)
    assert abs(out["mixed"][1] - out["fp64"][1]) <= 1e-6 * out["fp64"][1]
    errs = [l1_linf(a, b) for a, b in zip(phase_densities(out["mixed"][0]), phase_densities(out["fp64"][0]))]
    print(f"mixed ({kernel}) two-phase test case {testcase} ({flux}), {steps} steps: density L1/Linf per phase "
          + ", ".join(f"{l1:.1e}/{li:.1e}" for l1, li in errs))
    assert max(e[0] for e in errs) <= 1e-6


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("flux", ["hll", "lxf"])
def test_mixed_twophase_smoothed_interface(hyp, orc, flux, kernel):
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    nx, steps = 2048, 100
    P = mph_interface_prims(hyp.Barton2009(), nx)
    Q0 = np.ascontiguousarray(orc.prim2cons(oracle_pb(orc), P).T)
    out = {}
    for prec in ("fp64", "mixed"):
        with hyp.Solver(eos_pair(hyp), nx, model="multi", flux=flux, precision=prec, cfl=0.5) as s:
            _mixed_kernel(s, prec, kernel)
            s.upload(Q0)
            s.step(max_steps=steps)
            out[prec] = s.download()
    errs = [l1_linf(a, b) for a, b in zip(phase_densities(out["mixed"]), phase_densities(out["fp64"]))]
    print(f"mixed ({kernel}) two-phase smoothed interface ({flux}), {steps} steps: density L1/Linf per phase "
          + ", ".join(f"{l1:.1e}/{li:.1e}" for l1, li in errs))
    assert max(e[0] for e in errs) <= 1e-6


@pytest.mark.parametrize("kernel", KERNELS)
def test_mixed_twophase_uniform_state_preserved(hyp, orc, kernel):
    rng = np.random.default_rng(8)
    q = random_mph(orc, 1, rng)[0]
    Q0 = np.ascontiguousarray(np.repeat(q[:, None], 1000, axis=1))
    with hyp.Solver(eos_pair(hyp), 1000, model="multi", flux="hll", precision="mixed", bc="transmissive") as s:
        s.set_mixed_kernel(kernel)
        s.upload(Q0)
        Qa = s.download()  # the compensated pair holds the FP64 input to ~48 bits
        s.step(max_steps=3)
        Qb = s.download()
    assert np.max(np.abs(Qa - Q0) / np.maximum(np.abs(Q0), 1e-300)) < 1e-13
    # With Q_l = Q_r the FP32 Q_hll differs from Q by rounding, so the two path integrals
    # through it cancel only to rounding: the state stays uniform to that level.
    scale = np.max(np.abs(Qa), axis=1, keepdims=True)
    assert np.max(np.abs(Qb - Qa) / np.maximum(scale, 1e-30)) < 1e-9


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("flux", ["hll", "lxf"])
def test_nondefault_exponents_twophase(hyp, orc, flux, kernel):
    """Phase 1 with non-integer beta, gamma (the alternative Barton2009 parameters of
    main.jl:133): the step runs the kernels' general-exponent instances (powers through
    exp/log), which the default parameters never reach. FP64 against the oracle at
    RTOL_FP64 after 30 steps of test case 6; mixed against FP64 after 100 steps."""
    from hyperelasticsolver_gb300._cases import mph_case, initial_condition
    eos = (hyp.Barton2009(_beta=3.577, _gamma=2.088), hyp.Barton2009(_b0=B0_SOFT))
    oflux = orc.FLUX_HLL if flux == "hll" else orc.FLUX_LXF
    nx = 200
    pb = orc.problem(model=orc.MODEL_MULTI, flux=oflux, nx=nx, cfl=0.6,
                     eos=(orc.barton2009(beta=3.577, gamma=2.088), orc.barton2009(b0=B0_SOFT)))
    Pl, Pr = mph_case(6)
    Q0 = initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx)
    Qo, _, to, _ = orc.run(pb, Q0, max_steps=30)
    with hyp.Solver(eos, nx, model="multi", flux=flux, cfl=0.6) as s:
        s.upload(Q0)
        n, t = s.step(max_steps=30)
        assert n == 30 and abs(t - to) <= RTOL_FP64 * to
        err = assert_close_soa(s.download(), Qo, RTOL_FP64, f"non-default exponents ({flux})")
    out = {}
    for prec in ("fp64", "mixed"):
        with hyp.Solver(eos, nx, model="multi", flux=flux, precision=prec, cfl=0.6) as s:
            _mixed_kernel(s, prec, kernel)
            s.upload(Q0)
            assert s.step(max_steps=100)[0] == 100
            out[prec] = s.download()
    errs = [l1_linf(a, b) for a, b in zip(phase_densities(out["mixed"]), phase_densities(out["fp64"]))]
    print(f"two-phase non-default exponents ({flux}, {kernel}): FP64 vs oracle {err:.1e}; mixed density L1/Linf "
          + ", ".join(f"{l1:.1e}/{li:.1e}" for l1, li in errs))
    assert max(e[0] for e in errs) <= 1e-6


@pytest.mark.parametrize("flux", ["hll", "lxf"])
@pytest.mark.parametrize("bc", ["frozen", "transmissive"])
@pytest.mark.parametrize("nx", [5, 63, 64, 126, 127, 400])
def test_fused_face_update_blocks(hyp, orc, nx, bc, flux):
    """The mixed step with paired faces runs its faces and update in one kernel (63
    cells per block, each block computing its right neighbour's first face again); the
    scalar faces run them as two kernels. Across block edges (nx around multiples
    of 63) and with both end rules the two agree to FP32 rounding after 40 steps (the
    paired and scalar faces round alike, not identically): each variable within 1e-4 of
    its scale (HLL: measured up to 1.7e-6 on 5 cells, where every cell moves), each
    phase's density within 1e-6 in L1 (HLL: measured 1.2e-8). A fluctuation taken
    from the wrong face, or a cell updated twice or not at all, is an O(1) error."""
    from hyperelasticsolver_gb300._cases import mph_case, initial_condition
    pb = oracle_pb(orc, nx=nx, cfl=0.6)
    Pl, Pr = mph_case(6)
    Q0 = initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx)
    out = {}
    for kernel in KERNELS:
        with hyp.Solver(eos_pair(hyp), nx, model="multi", flux=flux, precision="mixed", bc=bc, cfl=0.6) as s:
            s.set_mixed_kernel(kernel)
            s.upload(Q0)
            n, t = s.step(max_steps=40)
            assert n == 40
            out[kernel] = (s.download(), t)
    (Qt, tt), (Qp, tp) = out["tile"], out["pair"]
    assert abs(tp - tt) <= 1e-6 * tt
    scale = np.maximum(np.max(np.abs(Qt), axis=1, keepdims=True), 1e-6)  # variables that stay ~0: absolute
    assert np.max(np.abs(Qp - Qt) / scale) <= 1e-4
    for a, b in zip(phase_densities(Qp), phase_densities(Qt)):
        assert np.sum(np.abs(a - b)) / np.sum(np.abs(b)) <= 1e-6
    if bc == "frozen":  # the end cells keep their uploaded values (the compensated pair holds ~48 bits)
        ends = Q0[:, [0, -1]]
        assert np.max(np.abs(Qp[:, [0, -1]] - ends) / np.maximum(np.abs(ends), 1e-300)) < 1e-13

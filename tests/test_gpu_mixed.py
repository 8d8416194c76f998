"""The mixed-precision single-phase step (FP32 fluxes, compensated FP32 state,
float-float cons2prim islands) against FP64 (GPU).

Accuracy target: relative L1 error of the density rho_true (cons2prim's
density, HyperelasticityMPh.jl:114) <= 1e-6 against the FP64 oracle / FP64
path; L-infinity is reported alongside."""
import numpy as np
import pytest

from helpers import RTOL_FP64

pytestmark = pytest.mark.gpu

L1_TARGET = 1e-6


def density(Q, rho0=8.93):
    """rho_true = sqrt(det(rho A) / rho0) of SoA single-phase states (14, n)."""
    m = Q[5:14]
    det = (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[3] * (m[1] * m[8] - m[7] * m[2])
           + m[6] * (m[1] * m[5] - m[4] * m[2]))
    return np.sqrt(det / rho0)


def errors(Qm, Qref):
    a, b = density(Qm), density(Qref)
    l1 = np.sum(np.abs(a - b)) / np.sum(np.abs(b))
    linf = np.max(np.abs(a - b)) / np.max(np.abs(b))
    return l1, linf


def riemann(orc, nx):
    from hyperelasticsolver_gb300._cases import riemann_1ph, initial_condition
    import hyperelasticsolver_gb300 as h
    Pl, Pr = riemann_1ph(h.Barton2009())
    pb = orc.problem(nx=nx, cfl=0.5)
    return initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx), pb


KERNELS = ["tile", "pair"]  # one block per tile; two tiles per block in packed FP32 pairs


@pytest.mark.parametrize("kernel", KERNELS)
def test_riemann_problem_mixed_vs_oracle(hyp, orc, kernel):
    Q0, pb = riemann(orc, 1000)
    t_end = 0.3 / orc.max_speed(pb, Q0)
    Qo, so, to, _ = orc.run(pb, Q0, t_end=t_end)
    with hyp.Solver(hyp.Barton2009(), 1000, precision="mixed", cfl=0.5) as s:
        s.set_mixed_kernel(kernel)
        s.upload(Q0)
        n, t = s.step(max_steps=so)
        assert n == so
        assert abs(t - to) <= 1e-5 * to  # dt from an FP32 max wave speed
        l1, linf = errors(s.download(), Qo)
    print(f"mixed ({kernel}) Riemann N=1000, {n} steps: density L1 {l1:.2e}, Linf {linf:.2e}")
    assert l1 <= L1_TARGET


@pytest.mark.parametrize("kernel", KERNELS)
def test_random_states_mixed_vs_oracle(hyp, orc, kernel):
    from test_gpu_1ph import random_prims
    rng = np.random.default_rng(99)
    nx, steps = 2048, 200
    pb = orc.problem(nx=nx, cfl=0.5, bc=orc.BC_TRANSMISSIVE)
    P = random_prims(nx, rng, strain=0.03, umax=0.3, smax=2e-4)
    Q0 = np.ascontiguousarray(orc.prim2cons(pb, P).T)
    Qo, _, to, _ = orc.run(pb, Q0, max_steps=steps)
    with hyp.Solver(hyp.Barton2009(), nx, precision="mixed", bc="transmissive", cfl=0.5) as s:
        s.set_mixed_kernel(kernel)
        s.upload(Q0)
        n, t = s.step(max_steps=steps)
        l1, linf = errors(s.download(), Qo)
    print(f"mixed ({kernel}) random states N={nx}, {steps} steps: density L1 {l1:.2e}, Linf {linf:.2e}")
    assert l1 <= L1_TARGET


@pytest.mark.parametrize("kernel", KERNELS)
def test_segments_mixed_vs_fp64_gpu(hyp, orc, kernel):
    """The benchmark's initial data (64 seeded segments) at 2^20 cells, 200 steps:
    mixed against the FP64 GPU path (itself held to 1e-12 of the oracle)."""
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    eos = hyp.Barton2009()
    nx = 1 << 20
    Q0 = segment_fill(orc.prim2cons(orc.problem(), segment_states(eos)), nx)
    out = {}
    for prec in ("fp64", "mixed"):
        with hyp.Solver(eos, nx, precision=prec, cfl=0.5) as s:
            if prec == "mixed":
                s.set_mixed_kernel(kernel)
            s.upload(Q0)
            s.step(max_steps=200)
            out[prec] = (s.download(), s.time()[0])
    l1, linf = errors(out["mixed"][0], out["fp64"][0])
    print(f"mixed ({kernel}) vs fp64, 2^20 cells, 200 steps: density L1 {l1:.2e}, Linf {linf:.2e}")
    assert l1 <= L1_TARGET
    assert abs(out["mixed"][1] - out["fp64"][1]) <= 1e-5 * out["fp64"][1]


@pytest.mark.parametrize("kernel", KERNELS)
def test_uniform_state_exact_in_mixed(hyp, orc, kernel):
    nx = 1 << 16
    P = np.array([8.93 / 1.02, 0.3, -0.2, 0.1, 1e-4, 1.02, 0.01, 0, 0, 1, 0.02, 0, 0, 1.0])
    q = orc.prim2cons(orc.problem(), P)
    Q0 = np.ascontiguousarray(np.repeat(q[:, None], nx, axis=1))
    with hyp.Solver(hyp.Barton2009(), nx, precision="mixed", bc="transmissive") as s:
        s.set_mixed_kernel(kernel)
        s.upload(Q0)
        s.step(max_steps=5)
        Q = s.download()
    # the compensated pair reproduces the FP64 input to ~48 bits and does not move
    assert np.max(np.abs(Q - Q0) / np.maximum(np.abs(Q0), 1e-300)) < 1e-13


def test_mixed_graph_and_single_launches_agree(hyp, orc):
    Q0, _ = riemann(orc, 700)
    with hyp.Solver(hyp.Barton2009(), 700, precision="mixed") as a, \
            hyp.Solver(hyp.Barton2009(), 700, precision="mixed") as b:
        a.upload(Q0)
        b.upload(Q0)
        a.step(max_steps=41)  # graph replays (12 steps) plus single launches
        for _ in range(41):
            b.step(max_steps=1)
        assert np.array_equal(a.download(), b.download())
        assert a.time() == b.time()
        assert a.max_wavespeed() == b.max_wavespeed()


def test_mixed_t_end_split_and_wavespeed(hyp, orc):
    Q0, pb = riemann(orc, 300)
    with hyp.Solver(hyp.Barton2009(), 300, precision="mixed") as s, \
            hyp.Solver(hyp.Barton2009(), 300) as d:
        s.upload(Q0)
        d.upload(Q0)
        assert abs(s.max_wavespeed() - d.max_wavespeed()) <= 1e-6 * d.max_wavespeed()
        n1, _ = s.step(max_steps=9)
        n2, t2 = s.step(t_end=0.004)
        lam = s.max_wavespeed()
        n3, t3 = s.step(t_end=0.004)  # nothing to do; the state's max lambda must survive
        assert n3 == 0 and t3 == t2 and s.max_wavespeed() == lam
        m, _ = d.step(t_end=0.004)
        assert abs((n1 + n2) - m) <= 1


@pytest.mark.parametrize("nx,bc", [(3, "frozen"), (254, "transmissive"), (255, "frozen"), (4097, "frozen"),
                                   (70001, "transmissive")])
def test_tma_pair_and_tile_kernels_agree(hyp, orc, nx, bc):
    """The persistent TMA-prefetched kernel, the two-tiles-per-block pair kernel and the
    one-block-per-tile kernel run the same tile arithmetic on the same inputs, for sizes
    that leave partial tiles (and, for the pair kernel, a block whose second tile is
    partial or empty) and unaligned row ends. The kernels are compiled separately and
    the pair kernel writes its multiply-adds out as fused pairs, so they agree to the
    mixed-precision rounding level (1e-6 relative per variable), not bitwise."""
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    eos = hyp.Barton2009()
    seg = orc.prim2cons(orc.problem(cfl=0.5), segment_states(eos, 8))
    Q0 = segment_fill(seg, nx)
    out = {}
    for kernel in ("tma", "pair", "tile"):
        with hyp.Solver(eos, nx, bc=bc, precision="mixed") as s:
            s.set_mixed_kernel(kernel)
            s.upload(Q0)
            s.step(max_steps=30)
            out[kernel] = (s.download(), s.time(), s.max_wavespeed())
    b, (tb, sb), lb = out["tile"]
    scale = np.maximum(np.max(np.abs(b), axis=1, keepdims=True), 1e-30)
    for kernel in ("tma", "pair"):
        a, (ta, sa), la = out[kernel]
        err = np.max(np.abs(a - b) / scale)
        print(f"{kernel} vs tile, {nx} cells {bc}: max rel {err:.1e}")
        assert err <= 1e-6
        assert sa == sb and abs(ta - tb) <= 1e-6 * tb
        assert abs(la - lb) <= 1e-6 * lb


def test_tma_wait_timeout_is_reported_and_recoverable(hyp, orc):
    """The TMA kernel's barrier waits are bounded. With a poll budget of 0 every wait
    runs out at once: each block records the timeout, lets its in-flight box copy land
    and ends, and the step reports HYP_ERR_TIMEOUT (no fault, no hang). With the
    budget restored the same context steps a fresh upload as the tile kernel does."""
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    eos = hyp.Barton2009()
    seg = orc.prim2cons(orc.problem(cfl=0.5), segment_states(eos, 8))
    nx = 4097
    Q0 = segment_fill(seg, nx)
    with hyp.Solver(eos, nx, precision="mixed") as s:
        s.set_mixed_kernel("tma")
        s.upload(Q0)
        s.set_wait_limit(0)
        with pytest.raises(hyp._lib.HypError) as err:
            s.step(max_steps=3)
        assert err.value.code == hyp._lib.HYP_ERR_TIMEOUT
        s.set_wait_limit(1 << 20)
        s.upload(Q0)
        n, _ = s.step(max_steps=20)
        assert n == 20
        Qa = s.download()
    with hyp.Solver(eos, nx, precision="mixed") as t:
        t.upload(Q0)
        t.step(max_steps=20)
        Qb = t.download()
    scale = np.maximum(np.max(np.abs(Qb), axis=1, keepdims=True), 1e-30)
    assert np.max(np.abs(Qa - Qb) / scale) <= 1e-6


@pytest.mark.parametrize("model", ["single", "multi"])
@pytest.mark.parametrize("n", [1000, 1 << 22])
def test_pinned_upload_and_pipelined_download_are_bitwise(hyp, orc, model, n):
    """hyp_upload from page-locked memory (the install kernel reads the host array in place)
    and from pageable memory (copied to the staging block first) install bitwise the same
    state, wave speed and following steps; the row-pipelined download (large states) returns
    bitwise what the one-pass download does."""
    from hyperelasticsolver_gb300._lib import PinnedArray
    from hyperelasticsolver_gb300 import Hyperelasticity as H, HyperelasticityMPh as HM
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill, mph_interface_prims
    if model == "single":
        eos = hyp.Barton2009()
        Q0 = segment_fill(H.prim2cons(eos, segment_states(eos, 64)), n)
    else:
        eos = (hyp.Barton2009(), hyp.Barton2009(_b0=2.1 * np.sqrt(0.1)))
        Q0 = np.ascontiguousarray(HM.prim2cons_mph(eos, mph_interface_prims(eos[0], n)).T)
    pin = PinnedArray(Q0.shape)
    pin.array[...] = Q0
    out = {}
    try:
        for src in ("pageable", "pinned"):
            with hyp.Solver(eos, n, model=model, flux="rusanov" if model == "single" else "hll",
                            precision="mixed") as s:
                s.upload(Q0 if src == "pageable" else pin.array)
                lam = s.max_wavespeed()
                first = s.download()
                s.step(max_steps=5)
                after = s.download()
                again = s.download(pin.array if src == "pinned" else None)  # into page-locked memory too
                out[src] = (lam, first, after, np.array(again))
    finally:
        pin.close()
    a, b = out["pageable"], out["pinned"]
    assert a[0] == b[0]
    for x, y in zip(a[1:], b[1:]):
        assert np.array_equal(x, y)
    assert np.array_equal(a[2], a[3])
    # the installed state is the uploaded one to the hi/lo pair's precision
    assert np.max(np.abs(a[1] - Q0) / np.maximum(np.max(np.abs(Q0), axis=1, keepdims=True), 1e-300)) < 1e-13

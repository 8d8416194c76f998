"""The batched, two-phase and adjoint workloads at their full stated sizes (GPU).

- Batch: 4096 independent single-phase Riemann problems, cell counts log-uniform in
  [256, 65536] (48.9 M cells), 500 steps each with its own CFL time step, mixed
  precision against the FP64 batch: relative L1 density error <= 1e-6 per problem.
- Two phases: 2^22 cells, volume fraction a smoothed step from 1 - 1e-6 to 1e-6 over 8
  cells, phase 2 with a tenth of the shear modulus, 300 path-conservative HLL steps
  (main.jl:225), mixed against FP64: relative L1 error of each phase's density <= 1e-6.
- Adjoint: gradient of a density misfit after 1000 FP64 Rusanov steps on 65,536 cells
  with checkpoints every 50 steps, against central differences of the forward run in
  all 15 parameters (step 1e-6 relative): agreement within 1e-5 relative.
The oracle is too slow for these sizes; the FP64 device paths they are checked against
are themselves held to the oracle at 1e-12 by the other tests, and the checks here are
the size-independent properties of each workload."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L1_TARGET = 1e-6


def _density(Q, rho0=8.93):
    m = Q[5:14]
    det = (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[3] * (m[1] * m[8] - m[7] * m[2])
           + m[6] * (m[1] * m[5] - m[4] * m[2]))
    return np.sqrt(det / rho0)


def _phase_density(Q, p, rho0=8.93):
    """rho_true of phase p: sqrt(det(alpha rho A / alpha) / rho0) (HyperelasticityMPh.jl:113-114)."""
    m = Q[15 * p + 6:15 * p + 15] / Q[15 * p]
    det = (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[3] * (m[1] * m[8] - m[7] * m[2])
           + m[6] * (m[1] * m[5] - m[4] * m[2]))
    return np.sqrt(det / rho0)


def test_batch_4096_problems_500_steps(hyp):
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    from hyperelasticsolver_gb300._cases import batch_sizes, batch_prims, batch_fill
    eos = hyp.Barton2009()
    sizes = batch_sizes(4096)
    assert len(sizes) == 4096 and sizes.min() >= 256 and sizes.max() <= 65536
    Pl, Pr = batch_prims(eos, len(sizes))
    Q0 = batch_fill(H.prim2cons(eos, Pl), H.prim2cons(eos, Pr), sizes)
    steps = 500
    out = {}
    for prec in ("mixed", "fp64"):
        with hyp.Batch(eos, sizes, precision=prec) as b:
            b.upload(Q0)
            b.step(steps)
            t, s = b.status()
            assert np.all(s == steps)
            out[prec] = (b.download(), t)
    (Qm, tm), (Q64, t64) = out["mixed"], out["fp64"]
    assert np.max(np.abs(tm - t64) / t64) <= 1e-6
    a, r = _density(Qm), _density(Q64)
    offs = np.concatenate([[0], np.cumsum(sizes)])
    l1 = np.array([np.sum(np.abs(a[o:e] - r[o:e])) / np.sum(np.abs(r[o:e])) for o, e in zip(offs[:-1], offs[1:])])
    print(f"batch of 4096 problems ({offs[-1]} cells), {steps} steps: per-problem density L1 max {l1.max():.2e}, "
          f"median {np.median(l1):.2e}")
    assert np.all(np.isfinite(l1)) and l1.max() <= L1_TARGET


def test_twophase_2p22_cells_300_steps(hyp):
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    eos = (hyp.Barton2009(), hyp.Barton2009(_b0=2.1 * np.sqrt(0.1)))
    n, steps = 1 << 22, 300
    Q0 = np.ascontiguousarray(HM.prim2cons_mph(eos, mph_interface_prims(eos[0], n)).T)
    out = {}
    for prec in ("mixed", "fp64"):
        with hyp.Solver(eos, n, model="multi", flux="hll", precision=prec, cfl=0.5) as s:
            s.upload(Q0)
            k, t = s.step(max_steps=steps)
            assert k == steps
            out[prec] = (s.download(), t)
    (Qm, tm), (Q64, t64) = out["mixed"], out["fp64"]
    assert abs(tm - t64) <= 1e-6 * t64
    errs = []
    for p in range(2):
        a, r = _phase_density(Qm, p), _phase_density(Q64, p)
        errs.append(np.sum(np.abs(a - r)) / np.sum(np.abs(r)))
    print(f"two-phase 2^22 cells, {steps} HLL steps: per-phase density L1 {errs[0]:.2e} / {errs[1]:.2e}")
    assert max(errs) <= L1_TARGET


def test_adjoint_65536_cells_1000_steps():
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300.adjoint import RiemannMisfit, PARAM_NAMES
    from hyperelasticsolver_gb300._cases import adjoint_states, adjoint_target_theta
    eos = h.Barton2009()
    pl, pr = adjoint_states(eos)
    pb = RiemannMisfit(eos, pl, pr, 65536, 1000, ckpt_every=50)
    th0 = pb.theta0()
    target = pb.final_density(adjoint_target_theta(th0))
    L, g, tm = pb.loss_and_grad(th0, target)
    assert L > 0 and np.all(np.isfinite(g))
    fd = pb.fd_grad(th0, target)
    scale = np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    rel = np.abs(g - fd) / scale
    print(f"adjoint, 65536 cells x 1000 steps, checkpoints every 50: max rel vs central differences {rel.max():.2e}; "
          f"reverse pass {tm['ms_recompute'] + tm['ms_adjoint']:.1f} ms")
    assert rel.max() <= 1e-5, [(PARAM_NAMES[k], g[k], fd[k], rel[k]) for k in np.argsort(-rel)[:4]]


def test_twophase_2p22_cells_300_steps_with_relaxation(hyp):
    """The same two-phase workload with velocity and pressure relaxation after every step
    (an extension; mixed relaxes in FP64): mixed against FP64, per-phase density L1 <= 1e-6."""
    from hyperelasticsolver_gb300 import HyperelasticityMPh as HM
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    eos = (hyp.Barton2009(), hyp.Barton2009(_b0=2.1 * np.sqrt(0.1)))
    n, steps = 1 << 22, 300
    Q0 = np.ascontiguousarray(HM.prim2cons_mph(eos, mph_interface_prims(eos[0], n)).T)
    out = {}
    for prec in ("mixed", "fp64"):
        with hyp.Solver(eos, n, model="multi", flux="hll", precision=prec, cfl=0.5, relax="mechanical") as s:
            s.upload(Q0)
            k, t = s.step(max_steps=steps)
            assert k == steps
            out[prec] = s.download()
    errs = []
    for p in range(2):
        a, r = _phase_density(out["mixed"], p), _phase_density(out["fp64"], p)
        errs.append(np.sum(np.abs(a - r)) / np.sum(np.abs(r)))
    a1 = out["fp64"][0]
    assert np.max(np.abs(out["fp64"][0] + out["fp64"][15] - 1.0)) <= 1e-12  # alpha1 + alpha2 = 1
    print(f"two-phase 2^22 cells, {steps} HLL steps with relaxation: per-phase density L1 {errs[0]:.2e} / "
          f"{errs[1]:.2e}; alpha1 range {a1.min():.3e} .. {a1.max():.3e}")
    assert max(errs) <= L1_TARGET

"""Adjoint of the single-phase FP64 Rusanov run (hyp_adjoint): gradients of a
density misfit with respect to the 13 left-state parameters and the two EOS
moduli, against central finite differences of the forward run (step 1e-6
relative, agreement within 1e-5 relative), and independence of the checkpoint
interval."""
import numpy as np
import pytest

import hyperelasticsolver_gb300 as h
from hyperelasticsolver_gb300.adjoint import RiemannMisfit, PARAM_NAMES
from hyperelasticsolver_gb300._cases import adjoint_states, adjoint_target_theta

pytestmark = pytest.mark.gpu

FD_REL = 1e-5  # |g - g_fd| <= FD_REL * max(|g_fd|, 1e-3 max|g_fd|)


def _problem(nx=256, n_steps=120, K=16, bc="frozen"):
    eos = h.Barton2009()
    pl, pr = adjoint_states(eos)
    pb = RiemannMisfit(eos, pl, pr, nx, n_steps, bc=bc, ckpt_every=K)
    th0 = pb.theta0()
    target = pb.final_density(adjoint_target_theta(th0))
    return pb, th0, target


def _check_fd(g, fd):
    scale = np.maximum(np.abs(fd), 1e-3 * np.max(np.abs(fd)))
    rel = np.abs(g - fd) / scale
    bad = [(PARAM_NAMES[k], g[k], fd[k], rel[k]) for k in range(15) if rel[k] > FD_REL]
    assert not bad, bad
    return rel.max()


@pytest.mark.parametrize("bc", ["frozen", "transmissive"])
def test_gradient_matches_central_differences(bc):
    pb, th0, target = _problem(bc=bc)
    L, g, _ = pb.loss_and_grad(th0, target)
    assert L > 0 and np.all(np.isfinite(g))
    assert abs(pb.loss(th0, target) - L) <= 1e-12 * L  # the recorded run is the plain run
    fd = pb.fd_grad(th0, target)
    worst = _check_fd(g, fd)
    print(f"adjoint vs central differences ({bc}): max rel {worst:.2e}")


def test_gradient_matches_forward_mode_dual_oracle(orc):
    """Against a forward-mode dual-number run of the oracle (the reference
    restatement with every scalar carrying the 15 partials), same target."""
    import os
    pb, th0, target = _problem(nx=128, n_steps=60, K=16)
    L, g, _ = pb.loss_and_grad(th0, target)
    Lo, go = orc.misfit_grad_dual(orc.problem(nx=128, cfl=0.5), pb.prim_left, pb.prim_right, 60, target,
                                  nthreads=min(8, os.cpu_count() or 1))
    assert abs(L - Lo) <= 1e-10 * Lo
    rel = np.abs(g - go) / np.maximum(np.abs(go), 1e-3 * np.max(np.abs(go)))
    print(f"adjoint vs dual-number oracle: max rel {rel.max():.2e}")
    assert rel.max() <= 1e-8, [(PARAM_NAMES[k], g[k], go[k]) for k in np.argsort(-rel)[:4]]


def test_checkpoint_interval_does_not_change_the_gradient():
    pb, th0, target = _problem(n_steps=50)
    gs = []
    for K in (1, 7, 50):
        pb.K = K
        gs.append(pb.loss_and_grad(th0, target)[1])
    assert np.array_equal(gs[0], gs[1]) and np.array_equal(gs[0], gs[2])


def test_adjoint_requires_a_recorded_run():
    eos = h.Barton2009()
    pl, pr = adjoint_states(eos)
    Q0 = h._cases.initial_condition(h.Hyperelasticity.prim2cons(eos, pl), h.Hyperelasticity.prim2cons(eos, pr), 64)
    with h.Solver(eos, 64) as s:
        s.upload(Q0)
        with pytest.raises(h._lib.HypError):
            s.adjoint(np.zeros((14, 64)))
        s.record(10, 4)
        s.step(max_steps=1)  # the state no longer ends the recorded run
        with pytest.raises(h._lib.HypError):
            s.adjoint(np.zeros((14, 64)))
    with h.Solver(eos, 64, precision="mixed") as s:
        s.upload(Q0)
        with pytest.raises(h._lib.UnsupportedError):
            s.record(10, 4)

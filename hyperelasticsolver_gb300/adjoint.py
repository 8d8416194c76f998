"""Gradient of a density misfit of a single-phase Riemann run with respect to the
left state and the EOS moduli, through the device adjoint (hyp_adjoint).

theta (15) = the left primitive state without its entropy, (rho, u(3), A(9)
column-major), then the Barton2009 shear modulus b0sq = b0^2 and bulk modulus
k0 = c0^2 - 4/3 b0^2 (EquationsOfState.jl:111-112). The run: Q0 = the two-state
fill of main.jl:99-106 from prim2cons of both states (HyperelasticityMPh.jl:63-90
at alpha = 1), n_steps FP64 Rusanov steps (main.jl:202-227), loss
L = 1/2 sum_i (rho_i(T) - target_i)^2 with rho = sqrt(det(rho A)/rho0).

loss_and_grad is the pullback a ChainRulesCore.rrule composes: the step adjoint
gives dL/dQ0 and the modulus terms of the steps; prim2cons_vjp carries dL/dQ0
(summed over each state's cells) back to the primitive states and adds the
modulus terms of the initial energies.
"""
import numpy as np

from . import Hyperelasticity as H
from .EquationsOfState import Barton2009
from .solver import Solver
from ._cases import initial_condition

PARAM_NAMES = ("rho", "u1", "u2", "u3", "A11", "A21", "A31", "A12", "A22", "A32", "A13", "A23", "A33", "b0sq", "k0")
PRIM_INDEX = np.array([0, 1, 2, 3, 5, 6, 7, 8, 9, 10, 11, 12, 13])  # theta[:13] in the 14-vector (rho, u, S, A)


def eos_with_moduli(eos, b0sq, k0):
    """The Barton2009 of eos with the given shear and bulk moduli (b0 = sqrt(b0sq), c0^2 = k0 + 4/3 b0sq)."""
    return Barton2009(eos.rho0, np.sqrt(k0 + 4.0 / 3.0 * b0sq), eos.cv, eos.t0, np.sqrt(b0sq), eos.alpha, eos.beta,
                      eos.gamma)


class RiemannMisfit:
    """A Riemann run whose left state and moduli are parameters."""

    def __init__(self, eos, prim_left, prim_right, nx, n_steps, X=1.0, cfl=0.5, bc="frozen", ckpt_every=50):
        self.eos = eos
        self.prim_left = np.asarray(prim_left, dtype=np.float64).copy()
        self.prim_right = np.asarray(prim_right, dtype=np.float64).copy()
        self.nx, self.n_steps, self.X, self.cfl, self.bc, self.K = int(nx), int(n_steps), X, cfl, bc, int(ckpt_every)
        self.left = np.arange(self.nx) < self.nx / 2

    def theta0(self):
        return np.concatenate([self.prim_left[PRIM_INDEX], [self.eos.b0sq, self.eos.k0]])

    def setup(self, theta):
        """(EOS, left prim, right prim, Q0) at theta."""
        theta = np.asarray(theta, dtype=np.float64)
        e = eos_with_moduli(self.eos, theta[13], theta[14])
        pl = self.prim_left.copy()
        pl[PRIM_INDEX] = theta[:13]
        ql = H.prim2cons(e, pl)
        qr = H.prim2cons(e, self.prim_right)
        return e, pl, self.prim_right, initial_condition(ql, qr, self.nx)

    def _solver(self, e):
        return Solver(e, self.nx, flux="rusanov", bc=self.bc, precision="fp64", X=self.X, cfl=self.cfl)

    def final_density(self, theta):
        e, _, _, Q0 = self.setup(theta)
        with self._solver(e) as s:
            s.upload(Q0)
            s.step(max_steps=self.n_steps)
            Q = s.download()
        return H.cons2prim(e, Q.T)[:, 0]

    def loss(self, theta, target):
        e, _, _, Q0 = self.setup(theta)
        with self._solver(e) as s:
            s.upload(Q0)
            s.step(max_steps=self.n_steps)
            return s.density_misfit(target, grad=False)

    def loss_and_grad(self, theta, target):
        """(L, dL/dtheta (15), device timings of the forward record and the reverse pass)."""
        e, pl, pr, Q0 = self.setup(theta)
        with self._solver(e) as s:
            s.upload(Q0)
            s.record(self.n_steps, self.K)
            L, dQ = s.density_misfit(target)
            dQ0, deos = s.adjoint(dQ)
            tm = s.adjoint_timing()
        qb = np.stack([dQ0[:, self.left].sum(axis=1), dQ0[:, ~self.left].sum(axis=1)])
        pb, eb = H.prim2cons_vjp(e, np.stack([pl, pr]), qb)
        g = np.concatenate([pb[0][PRIM_INDEX], deos + eb])
        return L, g, tm

    def fd_grad(self, theta, target, rel=1e-6, which=None):
        """Central differences with step rel * |theta_k|."""
        theta = np.asarray(theta, dtype=np.float64)
        which = range(15) if which is None else which
        g = np.full(15, np.nan)
        for k in which:
            h = rel * abs(theta[k]) if theta[k] != 0.0 else rel
            tp, tm = theta.copy(), theta.copy()
            tp[k] += h
            tm[k] -= h
            g[k] = (self.loss(tp, target) - self.loss(tm, target)) / (tp[k] - tm[k])
        return g

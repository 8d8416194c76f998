"""Initial data: the reference's Riemann test cases and the seeded synthetic workloads.

`mph_case` restates the primitive left/right states of
HyperelasticityMPh.initial_states (HyperelasticityMPh.jl:275-426); the values are
the reference's test-case table. The other builders generate the synthetic
single-phase workloads (primitive layout rho, u(3), S, A(9), column-major A).
"""
import numpy as np


def _col(F):
    return list(np.asarray(F, dtype=np.float64).reshape(-1, order="F"))


def mph_case(testcase):
    """Primitive 30-vectors (Pl, Pr) of HyperelasticityMPh.jl:275-426."""
    I = np.eye(3)
    F3 = np.array([[1.0, 0.0, 0.0], [-0.01, 0.95, 0.02], [-0.015, 0.0, 0.9]])
    F5r = np.array([[1.0, 0.0, 0.0], [0.015, 0.95, 0.0], [-0.01, 0.0, 0.9]])
    F4l = np.array([[0.98, 0.0, 0.0], [0.02, 1.0, 0.1], [0.0, 0.0, 1.0]])
    F4r = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.1], [0.0, 0.0, 1.0]])
    if testcase == 1:
        a, den, ul, ur, Sl, Sr, Fl, Fr = (0.5, 0.5, 0.5, 0.5), 5.0, [0, 0, 0], [0, 0, 0], 0.0, 0.0, I, I
    elif testcase == 2:
        a, den, ul, ur, Sl, Sr, Fl, Fr = (0.5, 0.5, 0.5, 0.5), 5.0, [1.0, 0, 0], [1.0, 0, 0], 0.0, 0.0, I, I
    elif testcase == 3:
        a, den, ul, ur, Sl, Sr, Fl, Fr = (0.5, 0.5, 0.5, 0.5), 8.9, [2.0, 0.0, 0.1], [2.0, 0.0, 0.1], 0.0, 0.0, F3, F3
    elif testcase == 4:
        a, den, ul, ur, Sl, Sr, Fl, Fr = (0.5, 0.5, 0.5, 0.5), 8.9, [0.0, 0.5, 1.0], [0, 0, 0], 1e-3, 0.0, F4l, F4r
    elif testcase == 5:
        a, den, ul, ur, Sl, Sr, Fl, Fr = (0.5, 0.5, 0.5, 0.5), 8.9, [2.0, 0.0, 0.1], [0.0, -0.03, -0.01], 0.0, 0.0, F3, F5r
    elif testcase == 6:
        a, den, ul, ur, Sl, Sr, Fl, Fr = (0.1, 0.9, 0.9, 0.1), 8.9, [0.0, 0.5, 1.0], [0, 0, 0], 1e-3, 0.0, F4l, F4r
    elif testcase == 7:
        a, den, ul, ur, Sl, Sr, Fl, Fr = (0.1, 0.9, 0.9, 0.1), 8.9, [2.0, 0.0, 0.1], [0.0, -0.03, -0.01], 0.0, 0.0, F3, F5r
    elif testcase == 10:
        a, den, ul, ur, Sl, Sr, Fl, Fr = (0.4, 0.6, 0.6, 0.4), 8.9, [2.0, 0.0, 0.1], [2.0, 0.0, 0.1], 0.0, 0.0, F3, F3
    else:
        raise ValueError(f"unknown test case {testcase}")
    al1, al2, ar1, ar2 = a
    dl, dr = den / np.linalg.det(Fl), den / np.linalg.det(Fr)
    Pl = [al1, dl, *ul, Sl, *_col(Fl), al2, dl, *ul, Sl, *_col(Fl)]
    Pr = [ar1, dr, *ur, Sr, *_col(Fr), ar2, dr, *ur, Sr, *_col(Fr)]
    return np.array(Pl, dtype=np.float64), np.array(Pr, dtype=np.float64)


def riemann_1ph(eos, u_l=(0.0, 0.5, 1.0), u_r=(0.0, -0.5, -1.0), A_l=(1 / 0.98, 1.0, 1.0), A_r=(1.0, 1.0, 1.0), S=0.0):
    """Single-phase Riemann primitive states (rho, u, S, A): velocities in units of b0,
    diagonal distortions, density rho0/det(A) (consistent with cons2prim's density)."""
    def prim(u, Ad):
        A = np.diag(Ad)
        return np.array([eos.rho0 / np.linalg.det(A), *(np.asarray(u) * eos.b0), S, *_col(A)])
    return prim(u_l, A_l), prim(u_r, A_r)


ADJOINT_SEED = 20261205


def adjoint_states(eos):
    """Primitive states of the adjoint workload: the two-state problem of riemann_1ph with a
    normal velocity of +-0.1 b0 (|u1| in the wave-speed bound has a kink at u1 = 0, where the
    loss would have no derivative) and small off-diagonal entries in the left distortion, so
    that every one of the 13 left-state parameters is non-zero."""
    A_l = np.array([[1 / 0.98, 0.01, 0.015], [0.012, 1.0, 0.02], [-0.01, 0.008, 1.0]])
    def prim(u, A):
        return np.array([eos.rho0 / np.linalg.det(A), *(np.asarray(u) * eos.b0), 0.0, *_col(A)])
    return prim((0.1, 0.5, 1.0), A_l), prim((-0.1, -0.5, -1.0), np.eye(3))


def adjoint_target_theta(theta0, seed=ADJOINT_SEED, scale=0.02):
    """Parameters of the target run: theta0 * (1 + scale * N(0, 1)), seeded."""
    rng = np.random.default_rng(seed)
    return np.asarray(theta0) * (1.0 + scale * rng.standard_normal(len(theta0)))


def initial_condition(Ql, Qr, nx):
    """Two-state Riemann fill, (i-1) < nx/2 on the left (main.jl:99-106). Returns SoA (nvar, nx)."""
    Ql, Qr = np.asarray(Ql, dtype=np.float64), np.asarray(Qr, dtype=np.float64)
    left = (np.arange(nx) < nx / 2)[None, :]
    return np.ascontiguousarray(np.where(left, Ql[:, None], Qr[:, None]))


def random_rotation(rng):
    """Haar-random rotation (QR of a Gaussian matrix with sign fix, det +1)."""
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


SEGMENT_SEED = 20261204  # first seed from 20261203 whose 63 boundaries all survive 320 steps


def segment_states(eos, n_seg=64, seed=SEGMENT_SEED, shared_rotation=True):
    """Primitive states of the seeded piecewise-constant workload: per segment
    rho/rho0 log-uniform in [0.9, 1.1], |u| uniform in [0, 0.5 b0] along a uniform
    direction, A = R (I + 0.05 G) (G standard Gaussian, resampled until det > 0)
    rescaled so that rho0/det(A) equals the drawn rho, S = 0. R is one random
    rotation shared by all segments (shared_rotation=True) or drawn per segment.
    Returns an (n_seg, 14) array.

    With a rotation per segment the Rusanov dissipation averages distortions of
    different orientation across a segment boundary and det(rho A) reaches 0
    within a few hundred steps at about a third of the boundaries (the reference
    raises DomainError there), so the workload shares one rotation."""
    rng = np.random.default_rng(seed)
    R_shared = random_rotation(np.random.default_rng(seed + 1))
    out = np.empty((n_seg, 14))
    for s in range(n_seg):
        rho = eos.rho0 * np.exp(rng.uniform(np.log(0.9), np.log(1.1)))
        v = rng.standard_normal(3)
        v /= np.linalg.norm(v)
        u = v * rng.uniform(0.0, 0.5 * eos.b0)
        while True:
            A = np.eye(3) + 0.05 * rng.standard_normal((3, 3))
            if np.linalg.det(A) > 0:
                break
        R = random_rotation(rng)
        A = (R_shared if shared_rotation else R) @ A
        A *= (eos.rho0 / (rho * np.linalg.det(A))) ** (1.0 / 3.0)
        out[s] = [rho, *u, 0.0, *_col(A)]
    return out


def segment_fill(states, nx):
    """Broadcast per-segment conservative (or primitive) states to nx cells: SoA (k, nx)."""
    states = np.asarray(states)
    n_seg = states.shape[0]
    seg = (np.arange(nx, dtype=np.int64) * n_seg) // nx
    return np.ascontiguousarray(states[seg].T)


def mph_interface_prims(eos, nx, a_hi=1.0 - 1e-6, a_lo=1e-6, width_cells=8):
    """Two-phase primitive states (nx, 30) of the volume-fraction interface workload:
    both phases carry the single-phase Riemann states (riemann_1ph) left and right of
    x = 0.5, and alpha1 is a smoothed step from a_hi to a_lo over about width_cells
    cells at x = 0.5 (the tanh profile of main.jl:110-123 with eps = width_cells * dx);
    alpha2 = 1 - alpha1."""
    Pl, Pr = riemann_1ph(eos)
    x = (np.arange(nx) + 0.5) / nx
    eps = width_cells / nx
    a1 = a_lo + (a_hi - a_lo) * 0.5 * (1.0 - np.tanh(4.0 * (x - 0.5) / eps))
    out = np.empty((nx, 30))
    for i in range(nx):
        P = Pl if x[i] < 0.5 else Pr
        out[i, 0] = a1[i]
        out[i, 1:15] = P
        out[i, 15] = 1.0 - a1[i]
        out[i, 16:30] = P
    return out


def batch_sizes(n_problems=4096, lo=256, hi=65536, seed=SEGMENT_SEED):
    """Cell counts floor(exp(U[ln lo, ln hi])) of the batched workload (seeded)."""
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), n_problems))).astype(np.int64)


def batch_prims(eos, n_problems, seed=SEGMENT_SEED):
    """Per-problem primitive Riemann states (left, right), each (n_problems, 14): the
    single-phase Riemann states of riemann_1ph with a seeded jitter per problem
    (velocity scale in [0.8, 1.2], left compression 1/A11 in [0.97, 0.99])."""
    rng = np.random.default_rng(seed + 7)
    L, R = [], []
    for _ in range(n_problems):
        su = rng.uniform(0.8, 1.2)
        a11 = 1.0 / rng.uniform(0.97, 0.99)
        pl, pr = riemann_1ph(eos, u_l=(0.0, 0.5 * su, 1.0 * su), u_r=(0.0, -0.5 * su, -1.0 * su),
                             A_l=(a11, 1.0, 1.0))
        L.append(pl)
        R.append(pr)
    return np.array(L), np.array(R)


def batch_fill(Ql, Qr, sizes):
    """Batch state SoA (14, sum(sizes)): problem p gets Ql[p] on (i-1) < N_p/2, Qr[p] after."""
    total = int(np.sum(sizes))
    out = np.empty((Ql.shape[1], total))
    o = 0
    for p, n in enumerate(sizes):
        left = np.arange(n) < n / 2
        out[:, o:o + n] = np.where(left[None, :], Ql[p][:, None], Qr[p][:, None])
        o += n
    return out

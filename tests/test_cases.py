"""The seeded synthetic workloads (CPU): the 64-segment single-phase state, the
two-phase volume-fraction interface, and the ragged batch, checked against the
properties their definitions state."""
import numpy as np


def test_segment_states():
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    eos = h.Barton2009()
    P = segment_states(eos, 64)
    assert P.shape == (64, 14) and np.array_equal(P, segment_states(eos, 64))
    rho, u, S = P[:, 0], P[:, 1:4], P[:, 4]
    A = P[:, 5:].reshape(64, 3, 3).transpose(0, 2, 1)  # column-major 9-vectors
    assert np.all(rho >= 0.9 * eos.rho0 - 1e-12) and np.all(rho <= 1.1 * eos.rho0 + 1e-12)
    assert np.all(np.linalg.norm(u, axis=1) <= 0.5 * eos.b0 + 1e-12) and np.all(S == 0.0)
    np.testing.assert_allclose(eos.rho0 / np.linalg.det(A), rho, rtol=1e-12)  # rho = rho0 / det A
    Q = segment_fill(P, 6400)
    assert Q.shape == (14, 6400) and np.array_equal(Q[:, 100 * 17], P[17])


def test_interface_profile():
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300._cases import mph_interface_prims
    n = 4096
    P = mph_interface_prims(h.Barton2009(), n)
    a1, a2 = P[:, 0], P[:, 15]
    assert np.all(a1 + a2 == 1.0) and np.all(np.diff(a1) <= 0.0)
    assert abs(a1[0] - (1 - 1e-6)) < 1e-9 and abs(a1[-1] - 1e-6) < 1e-9
    mid = np.count_nonzero((a1 > 0.01) & (a1 < 0.99))
    assert 4 <= mid <= 16  # a smoothed step about 8 cells wide at x = 0.5
    assert abs(np.argmin(np.abs(a1 - 0.5)) - n // 2) <= 1


def test_batch_sizes_and_fill():
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300._cases import batch_sizes, batch_prims, batch_fill
    sizes = batch_sizes()
    assert sizes.shape == (4096,) and np.array_equal(sizes, batch_sizes())
    assert sizes.min() >= 256 and sizes.max() < 65536
    assert 0.85 * 4096 < np.median(sizes) < 1.15 * 4096  # log-uniform on [256, 65536]: median 4096
    Pl, Pr = batch_prims(h.Barton2009(), 3)
    small = np.array([5, 6, 7])
    Q = batch_fill(Pl, Pr, small)
    assert Q.shape == (14, 18)
    for p, (o, n) in enumerate(zip([0, 5, 11], small)):
        left = np.arange(n) < n / 2  # (i - 1) < N/2 with 1-based i (main.jl:103)
        assert np.array_equal(Q[:, o:o + n][:, left], np.repeat(Pl[p][:, None], left.sum(), axis=1))
        assert np.array_equal(Q[:, o:o + n][:, ~left], np.repeat(Pr[p][:, None], (~left).sum(), axis=1))


def test_thirteen_value_layout_round_trip():
    """Hyperelasticity.jl's 13-value cell (rho u, rho F row-major, rho E) and the 14-value
    layout: the round trip is exact and the density comes from det(rho F)."""
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    rng = np.random.default_rng(1)
    eos = h.Barton2009()
    F = np.eye(3) + 0.05 * rng.standard_normal((3, 3))
    rho = eos.rho0 / np.linalg.det(F)
    q13 = np.concatenate([rho * rng.uniform(-1, 1, 3), (rho * F).reshape(-1), [rho * 0.7]])  # row-major rho F
    q14 = H.q13_to_q14(eos, q13)
    assert abs(q14[0] - rho) <= 1e-14 * rho
    assert np.array_equal(q14[5:14].reshape(3, 3, order="F"), (rho * F))  # column-major 9-vector
    assert np.array_equal(H.q14_to_q13(q14), q13)

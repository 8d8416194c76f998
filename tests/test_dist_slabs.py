"""Domain decomposition of one single-phase domain into slabs (CPU, gloo).

The orchestration of hyperelasticsolver_gb300.domain (local max -> max-allreduce ->
step with the global max -> halo exchange of boundary-cell records) drives the oracle
here, as a slab stepper, on 2 and 3 gloo ranks over 127.0.0.1; the gathered result
must equal the single-domain oracle run bit for bit. The CUDA slabs go through the
same functions (tests/test_gpu_slabs.py checks them on one GPU)."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

N_GLOBAL = 1024  # a power of two: the slabs' dx = (cells / N) / cells is the global 1/N exactly
STEPS = 40


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class OracleSlab:
    """The oracle as one slab (test infrastructure): held ends (frozen), the step with a
    prescribed dt = cfl dx / global max, as the CUDA slab computes it."""

    def __init__(self, orc, Q_global, world, rank, cfl=0.5):
        from hyperelasticsolver_gb300.domain import slab_layout
        self.orc = orc
        self.first, self.n, self.left, self.right = slab_layout(N_GLOBAL, world, rank)
        self.Q = np.ascontiguousarray(Q_global[:, self.first:self.first + self.n])
        self.pb = orc.problem(nx=self.n, X=self.n / N_GLOBAL, cfl=cfl)
        self.cfl, self.dx, self.t = cfl, 1.0 / N_GLOBAL, 0.0
        self.record_rows, self.record_dtype = 14, np.float64

    def local_max(self):
        return self.orc.max_speed(self.pb, self.Q, nthreads=1)

    def step(self, lam):
        dt = (self.cfl * self.dx) / lam
        self.Q = self.orc.run_dts(self.pb, self.Q, [dt], nthreads=1)
        self.t += dt
        return self.t

    def get_cells(self, first, count=1):
        return self.Q[:, first:first + count].copy()

    def set_cells(self, first, rec):
        self.Q[:, first:first + rec.shape[1]] = rec

    def owned(self):
        return self.Q[:, int(self.left):self.n - int(self.right)]


def _initial(orc):
    from hyperelasticsolver_gb300._cases import riemann_1ph, initial_condition
    import hyperelasticsolver_gb300 as h
    Pl, Pr = riemann_1ph(h.Barton2009())
    pb = orc.problem(nx=N_GLOBAL, cfl=0.5)
    return initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), N_GLOBAL)


def _rank(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    import oracle as orc
    from hyperelasticsolver_gb300.domain import TorchComm, step_decomposed
    from test_dist_slabs import OracleSlab, _initial
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s = OracleSlab(orc, _initial(orc), world, rank)
        comm = TorchComm(dist)
        t = 0.0
        for _ in range(STEPS):
            t = step_decomposed(s, comm)
        q.put((rank, s.first + int(s.left), s.owned().copy(), t))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_slabs_equal_single_domain_bitwise(orc, world):
    Q0 = _initial(orc)
    Qref, steps, tref, _ = orc.run(orc.problem(nx=N_GLOBAL, cfl=0.5), Q0, max_steps=STEPS, nthreads=1)
    assert steps == STEPS
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in procs), key=lambda o: o[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    Q = np.empty_like(Qref)
    for rank, lo, owned, t in out:
        Q[:, lo:lo + owned.shape[1]] = owned
        assert t == tref  # the same dt sequence: the allreduced max is the single-domain max
    assert np.array_equal(Q, Qref)


def test_slab_layout_covers_the_domain_once():
    from hyperelasticsolver_gb300.domain import owned_range, slab_layout
    for n, world in ((1000, 1), (1000, 3), (17, 5), (1 << 24, 8)):
        ranges = [owned_range(n, world, r) for r in range(world)]
        assert ranges[0][0] == 0 and ranges[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
        sizes = [hi - lo for lo, hi in ranges]
        assert max(sizes) - min(sizes) <= 1
        for r in range(world):
            first, m, left, right = slab_layout(n, world, r)
            lo, hi = ranges[r]
            assert (left, right) == (r > 0, r < world - 1)
            assert first == lo - left and first + m == hi + right
    with pytest.raises(ValueError):
        owned_range(5, 2, 0)


def test_step_all_in_one_process_equals_single_domain(orc):
    """The in-process driver (all slabs of one decomposition in one process, as the
    one-GPU emulation uses) gives the same bits as the gloo ranks."""
    from hyperelasticsolver_gb300.domain import step_all
    Q0 = _initial(orc)
    Qref, _, tref, _ = orc.run(orc.problem(nx=N_GLOBAL, cfl=0.5), Q0, max_steps=STEPS, nthreads=1)
    slabs = [OracleSlab(orc, Q0, 4, r) for r in range(4)]
    for _ in range(STEPS):
        ts = step_all(slabs)
    assert all(t == tref for t in ts)
    Q = np.concatenate([s.owned() for s in slabs], axis=1)
    assert np.array_equal(Q, Qref)

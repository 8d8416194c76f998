"""A batch's problems dealt over ranks (CPU, gloo).

The problems of a batch are independent, so hyperelasticsolver_gb300.domain deals
them to ranks by cell count (shard_problems) and each rank steps its share as its own
batch with no exchange between steps. Here the oracle steps each rank's problems on 2
and 3 gloo ranks over 127.0.0.1, rank 0 gathers the shard states, and the result must
equal the oracle's run of every problem in one process bit for bit.
(tests/test_gpu_batch.py steps the shards as separate CUDA batches on one GPU.)"""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STEPS = 30


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _sizes():
    rng = np.random.default_rng(9)
    return np.floor(np.exp(rng.uniform(np.log(16), np.log(300), 11))).astype(np.int64)


def _initial(orc, sizes):
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300._cases import batch_prims, batch_fill
    Pl, Pr = batch_prims(h.Barton2009(), len(sizes), seed=21)
    pb = orc.problem()
    return batch_fill(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), sizes)


def _run_problems(orc, sizes, Q):
    """The oracle over consecutive problems of SoA state Q (one process, problem by problem)."""
    out, times, o = np.empty_like(Q), [], 0
    for n in sizes:
        Qp, k, t, _ = orc.run(orc.problem(nx=int(n), cfl=0.5), Q[:, o:o + n], max_steps=STEPS, nthreads=1)
        assert k == STEPS
        out[:, o:o + n] = Qp
        times.append(t)
        o += n
    return out, np.array(times)


def _rank(rank, world, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    import oracle as orc
    from hyperelasticsolver_gb300.domain import shard_columns, shard_problems
    from test_dist_batch_shards import _initial, _run_problems, _sizes
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sizes = _sizes()
        mine = shard_problems(sizes, world)[rank]
        Q0 = _initial(orc, sizes)[:, shard_columns(sizes, mine)]  # this rank's shard only
        Qr, tr = _run_problems(orc, sizes[mine], Q0)
        got = [None] * world if rank == 0 else None
        dist.gather_object((mine, Qr, tr), got, dst=0)
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_batch_shards_equal_one_process(orc, world):
    from hyperelasticsolver_gb300.domain import gather_shards
    sizes = _sizes()
    Qref, tref = _run_problems(orc, sizes, _initial(orc, sizes))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    parts = out[0]
    assert all(out[r] is None for r in range(1, world))
    shards = [m for m, _, _ in parts]
    Q = gather_shards(sizes, shards, [Qr for _, Qr, _ in parts])
    assert np.array_equal(Q, Qref)
    for m, _, tr in parts:
        assert np.array_equal(tr, tref[m])  # each problem's own CFL time


def test_shard_problems_cover_each_problem_once_and_balance():
    from hyperelasticsolver_gb300._cases import batch_sizes
    from hyperelasticsolver_gb300.domain import gather_shards, shard_columns, shard_problems
    for sizes, world in ((batch_sizes(), 8), (batch_sizes(), 3), (np.array([5, 1, 9, 2]), 4), (_sizes(), 1)):
        shards = shard_problems(sizes, world)
        assert len(shards) == world
        allp = np.sort(np.concatenate(shards))
        assert np.array_equal(allp, np.arange(len(sizes)))
        loads = np.array([sizes[s].sum() for s in shards])
        assert loads.max() <= sizes.sum() / world + sizes.max()
        assert all(np.all(np.diff(s) > 0) for s in shards)  # batch order within a shard
        assert shard_problems(sizes, world)[0].tolist() == shards[0].tolist()  # deterministic
        # the shards' columns partition the batch state and gather back to it
        Q = np.arange(2 * sizes.sum(), dtype=np.float64).reshape(2, -1)
        assert np.array_equal(gather_shards(sizes, shards, [Q[:, shard_columns(sizes, s)] for s in shards]), Q)
    loads = [int(batch_sizes()[s].sum()) for s in shard_problems(batch_sizes(), 8)]
    assert max(loads) - min(loads) <= 2  # 4096 problems over 8 ranks: near-even cells
    for bad in ((np.array([3, 4]), 3), (np.array([3, 0]), 1), (np.array([3]), 0)):
        with pytest.raises(ValueError):
            shard_problems(*bad)

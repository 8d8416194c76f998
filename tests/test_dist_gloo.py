"""bench.py's multi-process path on CPU: two ranks over gloo (127.0.0.1), as
torchrun launches them, agree on the max-over-ranks timing and report the whole-job
value from it. The problems are independent replicas, so nothing but these timing
scalars crosses ranks."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    dist = bench.dist_setup()
    ms = 10.0 + 5.0 * rank  # this rank's timed region
    m = bench.dist_max(dist, ms)
    dist.barrier()
    q.put((rank, bench.WORLD, m))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 and o[2] == 15.0 for o in out)

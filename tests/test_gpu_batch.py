"""Batches of independent single-phase problems (GPU): each problem of a batch
must evolve as it does alone (same per-cell arithmetic; the kernels are compiled
separately, so multiply-add contraction may differ in the last bit), the mixed
batch must stay within the density-error target of the FP64 batch, and the
autotuner's variants must agree."""
import numpy as np
import pytest

from helpers import RTOL_FP64, assert_close_soa

pytestmark = pytest.mark.gpu

# two mixed-precision runs of the same problem by separately compiled kernels
MIXED_AGREE = 1e-6


def make_batch_state(orc, sizes, seed=11):
    import hyperelasticsolver_gb300 as h
    from hyperelasticsolver_gb300._cases import batch_prims, batch_fill
    Pl, Pr = batch_prims(h.Barton2009(), len(sizes), seed=seed)
    pb = orc.problem()
    return batch_fill(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), sizes)


def density(Q, rho0=8.93):
    m = Q[5:14]
    det = (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[3] * (m[1] * m[8] - m[7] * m[2])
           + m[6] * (m[1] * m[5] - m[4] * m[2]))
    return np.sqrt(det / rho0)


# problems whose ends fall on, just before and just after the 254-cell tiles of the
# mixed batch's tile-major state (a tile's halo cells are its neighbours' edge cells)
TILE_EDGE_SIZES = [3, 253, 254, 255, 508, 509, 762, 763, 1017]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("sizes_kind", ["random", "tile_edges"])
def test_batch_matches_individual_runs(hyp, orc, precision, sizes_kind):
    rng = np.random.default_rng(3)
    if sizes_kind == "random":
        sizes = np.floor(np.exp(rng.uniform(np.log(16), np.log(700), 20))).astype(np.int64)
    else:
        sizes = np.array(TILE_EDGE_SIZES, dtype=np.int64)
    Q0 = make_batch_state(orc, sizes)
    steps = 37
    with hyp.Batch(hyp.Barton2009(), sizes, precision=precision) as b:
        b.upload(Q0)
        b.step(steps)
        Qb = b.download()
        tb, sb = b.status()
    assert np.all(sb == steps)
    tol = RTOL_FP64 if precision == "fp64" else MIXED_AGREE
    for p, n in enumerate(sizes):
        o = int(np.sum(sizes[:p]))
        with hyp.Solver(hyp.Barton2009(), int(n), precision=precision) as s:
            s.upload(np.ascontiguousarray(Q0[:, o:o + n]))
            k, t = s.step(max_steps=steps)
            assert k == steps and abs(t - tb[p]) <= tol * t
            assert_close_soa(Qb[:, o:o + n], s.download(), tol, f"problem {p} ({n} cells)")


def test_fp64_batch_matches_oracle(hyp, orc):
    sizes = np.array([40, 17, 64], dtype=np.int64)
    Q0 = make_batch_state(orc, sizes, seed=5)
    with hyp.Batch(hyp.Barton2009(), sizes, precision="fp64") as b:
        b.upload(Q0)
        b.step(25)
        Qb = b.download()
    o = 0
    for n in sizes:
        Qo, _, _, _ = orc.run(orc.problem(nx=int(n), cfl=0.5), Q0[:, o:o + n], max_steps=25)
        assert_close_soa(Qb[:, o:o + n], Qo, RTOL_FP64, f"problem of {n} cells")
        o += n


def test_batch_nondefault_exponents(hyp, orc):
    """Non-integer beta, gamma (main.jl:133's alternative Barton2009 parameters): the
    FP64 batch against the oracle, and the mixed batch against single mixed runs."""
    sizes = np.array([40, 17, 64], dtype=np.int64)
    Q0 = make_batch_state(orc, sizes, seed=6)
    eos = hyp.Barton2009(_beta=3.577, _gamma=2.088)
    oeos = (orc.barton2009(beta=3.577, gamma=2.088),) * 2
    out = {}
    for prec in ("fp64", "mixed"):
        with hyp.Batch(eos, sizes, precision=prec) as b:
            b.upload(Q0)
            b.step(25)
            out[prec] = b.download()
    o = 0
    for n in sizes:
        Qo, _, _, _ = orc.run(orc.problem(nx=int(n), cfl=0.5, eos=oeos), Q0[:, o:o + n], max_steps=25)
        assert_close_soa(out["fp64"][:, o:o + n], Qo, RTOL_FP64, f"FP64 problem of {n} cells")
        with hyp.Solver(eos, int(n), precision="mixed") as s:
            s.upload(np.ascontiguousarray(Q0[:, o:o + n]))
            s.step(max_steps=25)
            assert_close_soa(out["mixed"][:, o:o + n], s.download(), MIXED_AGREE, f"mixed problem of {n} cells")
        o += n


def test_mixed_batch_accuracy_and_autotune(hyp, orc):
    """500 steps on 48 problems (256..4096 cells): per-problem relative L1 density
    error of the mixed batch against the FP64 batch <= 1e-6; every autotuner variant
    gives the same result bit for bit."""
    from hyperelasticsolver_gb300._cases import batch_sizes
    sizes = batch_sizes(48, 256, 4096, seed=2)
    Q0 = make_batch_state(orc, sizes, seed=2)
    with hyp.Batch(hyp.Barton2009(), sizes, precision="fp64") as b:
        b.upload(Q0)
        b.step(500)
        Q64 = b.download()
    results = []
    with hyp.Batch(hyp.Barton2009(), sizes, precision="mixed") as b:
        b.upload(Q0)
        chosen, ms = b.autotune(trial_steps=5)
        nv = hyp._lib.HYP_BATCH_NUM_VARIANTS
        assert 0 <= chosen < nv and len(ms) == nv and np.all(ms > 0)
        for v in range(nv):
            b.set_variant(v)
            b.upload(Q0)
            b.step(500)
            results.append(b.download())
    for r in results[1:]:
        assert_close_soa(r, results[0], MIXED_AGREE, "autotuner variants")
    l1 = []
    o = 0
    for n in sizes:
        a, ref = density(results[0][:, o:o + n]), density(Q64[:, o:o + n])
        l1.append(np.sum(np.abs(a - ref)) / np.sum(np.abs(ref)))
        o += n
    print(f"mixed batch, 48 problems x 500 steps: density L1 max {max(l1):.2e}, median {np.median(l1):.2e}; "
          f"autotune ms/step {np.array2string(ms, precision=3)} -> variant {chosen}")
    assert max(l1) <= 1e-6


def test_batch_t_end_stops_each_problem(hyp, orc):
    sizes = np.array([100, 300, 50], dtype=np.int64)
    Q0 = make_batch_state(orc, sizes, seed=9)
    t_end = 0.004
    with hyp.Batch(hyp.Barton2009(), sizes, precision="mixed") as b:
        b.upload(Q0)
        b.step(200, t_end=t_end)
        Qb = b.download()
        tb, sb = b.status()
    o = 0
    for p, n in enumerate(sizes):
        with hyp.Solver(hyp.Barton2009(), int(n), precision="mixed") as s:
            s.upload(np.ascontiguousarray(Q0[:, o:o + n]))
            k, t = s.step(t_end=t_end)
            assert k == sb[p] and abs(t - tb[p]) <= MIXED_AGREE * t and tb[p] >= t_end
            assert_close_soa(Qb[:, o:o + n], s.download(), MIXED_AGREE, f"problem {p}")
        o += n


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_shards_equal_the_whole_batch(hyp, orc, precision):
    """A batch dealt into three shards (domain.shard_problems), each stepped as its own
    batch (as three GPUs would), gathers back to the whole batch's result bit for bit:
    the same kernel on the same problem's cells, whatever else shares the batch."""
    from hyperelasticsolver_gb300.domain import gather_shards, shard_columns, shard_problems
    sizes = np.array(TILE_EDGE_SIZES + [40, 17, 600, 1300], dtype=np.int64)
    Q0 = make_batch_state(orc, sizes, seed=13)
    with hyp.Batch(hyp.Barton2009(), sizes, precision=precision) as b:
        b.upload(Q0)
        b.step(31)
        Qb = b.download()
        tb, _ = b.status()
    shards = shard_problems(sizes, 3)
    parts = []
    for problems in shards:
        with hyp.Batch(hyp.Barton2009(), sizes[problems], precision=precision) as b:
            b.upload(np.ascontiguousarray(Q0[:, shard_columns(sizes, problems)]))
            b.step(31)
            parts.append(b.download())
            assert np.array_equal(b.status()[0], tb[problems])
    assert np.array_equal(gather_shards(sizes, shards, parts), Qb)

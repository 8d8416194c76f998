"""CUDA slabs of a decomposed single-phase domain (hyp_set_slab, hyp_slab_local_max,
hyp_slab_step, hyp_get_cells / hyp_set_cells), several slabs driven in one process on
one GPU by hyperelasticsolver_gb300.domain.step_all -- the same phases the ranks of a
multi-GPU run take (local max, max-allreduce, step, halo exchange), with no kernel
waiting on another. The decomposed run must equal the single-domain hyp_step run bit
for bit: FP64 and mixed precision, Rusanov / frozen ends and LxF / transmissive ends."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 3000
STEPS = 30


def _state(hyp):
    from hyperelasticsolver_gb300 import Hyperelasticity as H
    from hyperelasticsolver_gb300._cases import segment_states, segment_fill
    eos = hyp.Barton2009()
    return eos, segment_fill(H.prim2cons(eos, segment_states(eos, 16)), N)


@pytest.mark.parametrize("precision,kernel", [("fp64", None), ("mixed", "tile"), ("mixed", "pair")])
@pytest.mark.parametrize("flux,bc", [("rusanov", "frozen"), ("lxf", "transmissive")])
@pytest.mark.parametrize("world", [2, 5])
def test_slabs_equal_single_domain_bitwise(hyp, precision, kernel, flux, bc, world):
    from hyperelasticsolver_gb300.domain import GpuSlab, step_all
    eos, Q0 = _state(hyp)
    with hyp.Solver(eos, N, flux=flux, bc=bc, precision=precision) as s:
        if kernel:
            s.set_mixed_kernel(kernel)
        s.upload(Q0)
        n, tref = s.step(max_steps=STEPS)
        assert n == STEPS
        Qref = s.download()
    slabs = [GpuSlab(eos, N, world, r, flux=flux, bc=bc, precision=precision) for r in range(world)]
    try:
        for sl in slabs:
            if kernel:
                sl.solver.set_mixed_kernel(kernel)
            sl.upload(Q0)
        for _ in range(STEPS):
            ts = step_all(slabs)
        assert all(t == tref for t in ts)
        Q = np.concatenate([sl.download_owned() for sl in slabs], axis=1)
    finally:
        for sl in slabs:
            sl.close()
    assert Q.shape == Qref.shape
    assert np.array_equal(Q, Qref)


def test_slab_records_round_trip_and_refusals(hyp):
    from hyperelasticsolver_gb300.domain import GpuSlab
    eos, Q0 = _state(hyp)
    for precision, rows, dtype in (("fp64", 14, np.float64), ("mixed", 32, np.float32)):
        with GpuSlab(eos, N, 3, 1, precision=precision) as sl:
            sl.upload(Q0)
            assert sl.record_rows == rows and sl.record_dtype == dtype
            rec = sl.get_cells(5, 3)
            assert rec.shape == (rows, 3)
            sl.set_cells(7, rec)
            assert np.array_equal(sl.get_cells(7, 3), rec)
            with pytest.raises(hyp._lib.HypError):
                sl.solver.step(max_steps=1)  # a slab steps with the global max only
            with pytest.raises(hyp._lib.HypError):
                sl.get_cells(sl.n - 1, 2)  # beyond the slab
    with hyp.Solver((hyp.Barton2009(), hyp.Barton2009()), 64, model="multi", flux="hll") as s:
        assert hyp._lib.load().hyp_set_slab(s._h, 1.0 / 64, 1, 1) == hyp._lib.HYP_ERR_UNSUPPORTED


@pytest.mark.parametrize("first,count", [(250, 10), (0, 300), (505, 260), (N - 7, 7)])
def test_mixed_records_across_tiles(hyp, first, count):
    """Mixed records of cells on both sides of the 254-cell tiles of the tile-major
    state: one 2D copy per tile the range touches. The records' hi + lo rows are the
    downloaded state's values; writing a range back at the same cells changes nothing,
    and written at other cells it reads back unchanged."""
    from hyperelasticsolver_gb300.domain import GpuSlab
    eos, Q0 = _state(hyp)
    with GpuSlab(eos, N, 1, 0, precision="mixed") as sl:
        sl.upload(Q0)
        rec = sl.get_cells(first, count)
        assert rec.shape == (32, count) and rec.dtype == np.float32
        Q = sl.solver.download()
        assert np.array_equal(rec[:14].astype(np.float64) + rec[14:28].astype(np.float64), Q[:, first:first + count])
        sl.set_cells(first, rec)
        assert np.array_equal(sl.solver.download(), Q)
        other = (first + 127) % (N - count)
        sl.set_cells(other, rec)
        assert np.array_equal(sl.get_cells(other, count), rec)

"""The allocation-free step entry point (hyp_step_noalloc_f64) against the context API.

hyp_step_noalloc_f64 is for callers that cannot allocate device memory where they
step the solver (their device memory belongs to another allocator, or the loop must
not call cudaMalloc). It keeps its scratch in one fixed static device array, so it
accepts at most 65,536 cells. This test calls it through the C ABI on device buffers
the test owns (allocated with torch), twice in a row, and checks each result against
the context API's hyp_step on the same state, within the FP64 tolerance of the other
tests. It lives in its own file that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

from helpers import RTOL_FP64, assert_close_soa

pytestmark = pytest.mark.gpu

MAX_CELLS = 65536


def _riemann_state(orc, nx):
    from hyperelasticsolver_gb300._cases import riemann_1ph, initial_condition
    import hyperelasticsolver_gb300 as h
    Pl, Pr = riemann_1ph(h.Barton2009())
    pb = orc.problem(nx=nx, cfl=0.5)
    return initial_condition(orc.prim2cons(pb, Pl), orc.prim2cons(pb, Pr), nx)


@pytest.mark.parametrize("flux,bc", [("rusanov", "frozen"), ("lxf", "transmissive")])
@pytest.mark.parametrize("k", [0, 24, 25])  # even: the input goes straight to the output; odd: via the scratch state
@pytest.mark.parametrize("in_place", [False, True])
def test_noalloc_step_matches_context_step_twice(hyp, orc, flux, bc, k, in_place):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    L = hyp._lib.load()
    nx = 4096
    Q0 = _riemann_state(orc, nx)
    fl = {"rusanov": hyp._lib.HYP_FLUX_RUSANOV, "lxf": hyp._lib.HYP_FLUX_LXF}[flux]
    bcc = {"frozen": hyp._lib.HYP_BC_FROZEN, "transmissive": hyp._lib.HYP_BC_TRANSMISSIVE}[bc]
    # reference: the context API, k steps then k more (no steps: the input itself)
    ref1, ref2, tr1, tr2 = Q0, Q0, 0.0, 0.0
    if k > 0:
        with hyp.Solver(hyp.Barton2009(), nx, cfl=0.5, flux=flux, bc=bc) as s:
            s.upload(Q0)
            s.step(max_steps=k)
            ref1, (tr1, _) = s.download(), s.time()
            s.step(max_steps=k)
            ref2, (tr2, _) = s.download(), s.time()
    cfg = hyp._model.config(hyp.Barton2009(), hyp._lib.HYP_MODEL_SINGLE, n_cells=nx, flux=fl, bc=bcc, cfl=0.5)
    d_in = torch.from_numpy(Q0).cuda()
    d_out = d_in if in_place else torch.empty_like(d_in)
    d_out2 = d_in if in_place else torch.empty_like(d_in)
    torch.cuda.synchronize()
    t = ctypes.c_double(0.0)
    cell = ctypes.c_int64(0)
    # call 1: Q0 -> k steps
    rc = L.hyp_step_noalloc_f64(cfg, d_in.data_ptr(), d_out.data_ptr(), nx, k, 0.0, None, ctypes.byref(t),
                                ctypes.byref(cell))
    assert rc == 0, rc
    assert cell.value == -1
    free_after_first = torch.cuda.mem_get_info()[0]
    assert abs(t.value - tr1) <= RTOL_FP64 * tr1
    assert_close_soa(d_out.cpu().numpy(), ref1, RTOL_FP64, "no-alloc call 1")
    # call 2: continue from call 1's output for k more steps
    t1 = t.value
    rc = L.hyp_step_noalloc_f64(cfg, d_out.data_ptr(), d_out2.data_ptr(), nx, k, t1, None, ctypes.byref(t),
                                ctypes.byref(cell))
    assert rc == 0, rc
    assert torch.cuda.mem_get_info()[0] == free_after_first  # nothing allocated by the second call
    assert abs(t.value - tr2) <= RTOL_FP64 * tr2
    assert_close_soa(d_out2.cpu().numpy(), ref2, RTOL_FP64, "no-alloc call 2")
    if k > 0:  # and both calls against the oracle directly, not only through the context API
        pb = orc.problem(nx=nx, cfl=0.5, flux={"rusanov": orc.FLUX_RUSANOV, "lxf": orc.FLUX_LXF}[flux],
                         bc={"frozen": orc.BC_FROZEN, "transmissive": orc.BC_TRANSMISSIVE}[bc])
        Qo, so, to, _ = orc.run(pb, Q0, max_steps=2 * k, nthreads=4)
        assert so == 2 * k and abs(t.value - to) <= RTOL_FP64 * to
        assert_close_soa(d_out2.cpu().numpy(), Qo, RTOL_FP64, "no-alloc call 2 vs oracle")


def test_noalloc_rejects_sizes_beyond_its_scratch(hyp):
    torch = pytest.importorskip("torch")
    L = hyp._lib.load()
    n = MAX_CELLS + 1
    cfg = hyp._model.config(hyp.Barton2009(), hyp._lib.HYP_MODEL_SINGLE, n_cells=n, cfl=0.5)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")  # never touched: the size check comes first
    t = ctypes.c_double(0.0)
    rc = L.hyp_step_noalloc_f64(cfg, buf.data_ptr(), buf.data_ptr(), n, 1, 0.0, None, ctypes.byref(t), None)
    assert rc == hyp._lib.HYP_ERR_INVALID

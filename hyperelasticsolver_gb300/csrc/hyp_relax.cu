// hyp_relax.cu -- the instantaneous pressure relaxation of hyp_relax.cuh applied to
// every cell of a two-phase context after each step (hyp_set_relaxation), and its
// function-level evaluator (hyp_eval_relax).
//
// FP64 contexts relax the state in place. Mixed contexts relax in FP64 from the
// compensated (hi, lo) pair and store the result as a new pair: the relaxation is an
// FP64 island of the mixed step, like its cons2prim islands. Cells where a phase is
// below kRelaxMinAlpha (all but the interface cells of a sharp interface) return at
// once, so the pass costs a read of the volume fractions there.
#include <string>
#include "hyp_internal.cuh"
#include "hyp_relax.cuh"

using namespace hyp;

namespace {

__device__ __forceinline__ void record_relax_err(DevState* S, int code, long long cell) {
  if (atomicCAS(&S->err_code, 0, code) == 0) S->err_cell = cell;
}

// After a step of parity p: the new state is Q (FP64) or (Qh, Ql) (mixed); an
// inactive step (t >= t_end before it) left it alone and so does the relaxation.
__global__ void __launch_bounds__(kBlock) relax2_f64_kernel(double* __restrict__ Q, int64_t n, Eos2 eos, int mode,
                                                            const double* t_in, double t_end, int bc, DevState* S) {
  if (!(*t_in < t_end)) return;
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (i >= n || (bc == HYP_BC_FROZEN && (i == 0 || i == n - 1))) return;
  if (!(Q[i] >= kRelaxMinAlpha && Q[15 * n + i] >= kRelaxMinAlpha)) return;
  double q[30];
  for (int v = 0; v < 30; ++v) q[v] = Q[v * n + i];
  const int st = relax_cell2(eos.e, mode, q);
  if (st) {
    record_relax_err(S, st, i);
    return;
  }
  for (int v = 0; v < 30; ++v) Q[v * n + i] = q[v];
}

__global__ void __launch_bounds__(kBlock) relax2_mixed_kernel(float* __restrict__ Qh, float* __restrict__ Ql,
                                                              int64_t pitch, int64_t n, Eos2 eos, int mode,
                                                              const double* t_in, double t_end, int bc, DevState* S) {
  if (!(*t_in < t_end)) return;
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (i >= n || (bc == HYP_BC_FROZEN && (i == 0 || i == n - 1))) return;
  if (!(Qh[i] >= (float)kRelaxMinAlpha && Qh[15 * pitch + i] >= (float)kRelaxMinAlpha)) return;
  double q[30];
  for (int v = 0; v < 30; ++v) q[v] = (double)Qh[v * pitch + i] + (double)Ql[v * pitch + i];
  const int st = relax_cell2(eos.e, mode, q);
  if (st) {
    record_relax_err(S, st, i);
    return;
  }
  for (int v = 0; v < 30; ++v) {
    const float h = (float)q[v];
    Qh[v * pitch + i] = h;
    Ql[v * pitch + i] = (float)(q[v] - (double)h);
  }
}

}  // namespace

namespace hyp {
cudaError_t launch_relax2(hyp_ctx* c, int p, double t_end) {
  const unsigned grid = (unsigned)((c->n + kBlock - 1) / kBlock);
  const int q = 1 - p;  // the state the step of parity p wrote
  if (c->cfg.precision == HYP_PREC_MIXED)
    relax2_mixed_kernel<<<grid, kBlock, 0, c->stream>>>(c->Qh[q], c->Ql[q], c->mpitch, c->n, c->eos2, c->relax,
                                                        &c->st->t[p], t_end, c->cfg.bc, c->st);
  else
    relax2_f64_kernel<<<grid, kBlock, 0, c->stream>>>(c->Q[q], c->n, c->eos2, c->relax, &c->st->t[p], t_end,
                                                      c->cfg.bc, c->st);
  return cudaGetLastError();
}
}  // namespace hyp

extern "C" int hyp_set_relaxation(hyp_ctx* c, int mode) {
  if (!c) return HYP_ERR_INVALID;
  if (mode != HYP_RELAX_NONE && mode != HYP_RELAX_PRESSURE && mode != HYP_RELAX_MECHANICAL)
    return ctx_set_err(c, HYP_ERR_INVALID, "relaxation mode");
  if (mode != HYP_RELAX_NONE && c->cfg.model != HYP_MODEL_MULTI)
    return ctx_set_err(c, HYP_ERR_UNSUPPORTED, "hyp_set_relaxation: two-phase contexts only");
  if (c->relax != mode) {
    c->relax = mode;
    for (auto& g : c->graph)  // captured steps no longer match
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }
  return HYP_OK;
}

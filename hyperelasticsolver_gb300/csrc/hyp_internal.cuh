// hyp_internal.cuh -- context, device-side step state and kernel launchers
// shared by the translation units of libhyperelastic_cuda.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "../../include/hyperelastic.h"
#include "hyp_physics.cuh"
#include "hyp_physics_mixed.cuh"
#include "hyp_physics_mph.cuh"
#include "hyp_tma.cuh"

namespace hyp {

constexpr int kBlock = 256;

// Device-resident loop control of one context. The step kernels read the
// input slot of t / lam_max and write the other slot, so a sequence of steps
// needs no host round trip (and can be captured in a CUDA graph).
struct DevState {
  double t[2];                        // time before the step of parity p is t[p]
  unsigned long long lam_bits[2];     // max wave speed of the state of parity p (bits of a double >= 0)
  unsigned long long lam_query;       // hyp_max_wavespeed slot
  unsigned long long lam_slots[3];    // mixed precision: FP32 max lambda (bits) of states k, k+1 (slot k%3)
  long long steps;                    // steps taken
  int err_code;                       // first HYP_CELL_* status raised (0 = none)
  int pad_;
  long long err_cell;                 // cell that raised it
};

// Per-cell flux components that are not identically zero for one phase:
// mass, momentum(3), energy and rows 2-3 of rho*A (row 1 of the rho*A flux is
// den*(u1 A[0,b] - u1 A[0,b]) = 0 exactly, HyperelasticityMPh.jl:172).
constexpr int kNFlux1 = 11;
__host__ __device__ __forceinline__ int flux_slot1(int v) {
  // v: index in the 14-vector [rho, rho u(3), rho E, rho A(9)]; -1 = zero flux
  if (v < 5) return v;
  int a = (v - 5) % 3;  // row of rho*A
  if (a == 0) return -1;
  int b = (v - 5) / 3;
  return 5 + 2 * b + (a - 1);
}

// The Rusanov face flux 0.5 (f_a + f_b) - h (q_b - q_a), h = max(lambda_a, lambda_b)/2
// (NumFluxes.jl:25-33, main.jl:45-48), with one fixed rounding sequence (explicit
// intrinsics, no compiler contraction), so the step commutes with x -> -x.
__device__ __forceinline__ double face_flux(double fa, double fb, double h, double qa, double qb) {
  return __fma_rn(-h, __dsub_rn(qb, qa), __dmul_rn(0.5, __dadd_rn(fa, fb)));
}

// Face f of a block's face table (between cells f - 1 and f of the problem [lo, hi),
// a zero-gradient ghost past either end) into slot k: its 14 flux components.
template <int kSlots>
__device__ __forceinline__ void rusanov_face(const double* __restrict__ Q, const double* __restrict__ F,
                                             const double* __restrict__ lam, int64_t n, int64_t lo, int64_t hi,
                                             int64_t f, bool lxf, double lam_lxf, double (*sF)[kSlots], int k) {
  const int64_t a = f > lo ? f - 1 : lo, b = f < hi ? f : hi - 1;
  double lf;
  if (lxf) {
    lf = lam_lxf;
  } else {
    const double la = lam[a], lb = lam[b];
    lf = la > lb ? la : lb;  // max(lambda_L, lambda_R) (main.jl:45-48)
  }
  const double h = lf * 0.5;
#pragma unroll
  for (int v = 0; v < 14; ++v) {
    const int sl = flux_slot1(v);
    const double fa = sl >= 0 ? F[sl * n + a] : 0.0, fb = sl >= 0 ? F[sl * n + b] : 0.0;
    sF[v][k] = face_flux(fa, fb, h, Q[v * n + a], Q[v * n + b]);
  }
}

// A step's dt = cfl dx / max lambda, the LxF lambda = dx / dt and dt/dx (main.jl:223-225;
// for LxF the update's dt/dx is 1 / lambda, main.jl:40), evaluated by lane 0 of each
// warp and broadcast: the same expressions, so the same bits, as evaluating them in
// every thread, at 1/32 of the FP64 divisions on the FP64 pipe that bounds the FP64
// kernels. Every lane of the warp must call it (no thread may have returned).
struct StepScalars {
  double dt, lam_lxf, dtdx;
};
__device__ __forceinline__ StepScalars step_scalars(double cfl, double dx, double lmax, bool lxf) {
  StepScalars s{0.0, 0.0, 0.0};
  if ((threadIdx.x & 31) == 0) {
    s.dt = (cfl * dx) / lmax;
    s.lam_lxf = dx / s.dt;
    s.dtdx = lxf ? 1.0 / s.lam_lxf : s.dt / dx;
  }
  s.dt = __shfl_sync(0xffffffffu, s.dt, 0);
  s.lam_lxf = __shfl_sync(0xffffffffu, s.lam_lxf, 0);
  s.dtdx = __shfl_sync(0xffffffffu, s.dtdx, 0);
  return s;
}

// Which end cells of a single-phase step are held (not updated). The step kernels
// take the context's bc: HYP_BC_FROZEN holds both ends (main.jl:219-220),
// HYP_BC_TRANSMISSIVE neither; a slab of a decomposed domain (hyp_slab.cu) also
// holds an end that is a ghost cell, whose value its neighbour supplies:
// kBcHoldFirst / kBcHoldLast hold only the first / last cell.
constexpr int kBcHoldFirst = 2, kBcHoldLast = 3;
__host__ __device__ __forceinline__ bool bc_holds(int bc, bool first, bool last) {
  return (first && (bc == HYP_BC_FROZEN || bc == kBcHoldFirst)) || (last && (bc == HYP_BC_FROZEN || bc == kBcHoldLast));
}

// The two phases' EOS, passed to the two-phase kernels by value.
struct Eos2 {
  EosC e[2];
};

struct StepTiming {
  float ms_total = 0.f, ms_cell = 0.f, ms_update = 0.f;
  int n_cell = 0, n_update = 0;
};

}  // namespace hyp

namespace hyp {
struct AdjTape;
struct SnapBuf;
// Mixed-precision state of one parity: kMixedRows rows per cell, rows 0-13 hi
// parts, 14-27 lo parts, 28 the cell's wave speed, 29-31 its island outputs.
// Row-major blocks (the batch solver, the two-phase step's 60 rows): row r of cell
// i at r * pitch + i. Tile-major blocks (the single-phase step): cells in tiles of
// kTileCells, each tile's 32 rows of kTileRow floats (its cells, then 2 unused)
// contiguous (32 KB, 128-byte aligned rows), so that the block that steps a tile
// reads and writes one contiguous span in whole 128-byte lines.
constexpr int kMixedRows = 32;
constexpr int kRowLo = 14, kRowLam = 28, kRowIsl = 29;
constexpr int kTileCells = 254;  // owned cells of a 256-thread tile
constexpr int kTileRow = 256;    // floats from one row of a tile to the next
constexpr int kTileFloats = kMixedRows * kTileRow;
__host__ __device__ __forceinline__ int64_t mixed_pitch(int64_t n) { return (n + 3) & ~int64_t(3); }
__host__ __device__ __forceinline__ int64_t mixed_tiles(int64_t n) { return (n + kTileCells - 1) / kTileCells; }
// Offset of cell i's row 0 in a tile-major block (row r at + r * kTileRow).
__host__ __device__ __forceinline__ int64_t tile_cell_off(int64_t i) {
  const unsigned t = (unsigned)i / kTileCells;  // cells < 2^31: the state of 2^31 cells exceeds the device
  return (int64_t)t * kTileFloats + (int64_t)((unsigned)i - t * kTileCells);
}
}

struct hyp_ctx {
  hyp_config cfg;
  hyp::EosC eos[2];
  int device = 0;
  int nvar = 14;
  int64_t n = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // downloads: device-to-host copies overlapping the next rows' join
  cudaEvent_t row_ev[30] = {};         // one per variable row of a pipelined download
  // FP64 state, double-buffered: Q[p] is the state before a step of parity p.
  double* Q[2] = {nullptr, nullptr};
  double* F = nullptr;     // per-cell fluxes (scratch)
  double* lam = nullptr;   // per-cell max wave speed (scratch)
  // mixed precision: per parity one block of floats, which also serves as the FP64
  // staging buffer of uploads and downloads. Single-phase: Qh[p] is a tile-major
  // block of the 32 rows (hi, lo, lambda, islands) of mixed_tiles(n) tiles; Ql is not
  // used. Two-phase: Qh[p] / Ql[p] the row-major hi / lo rows [30][mpitch].
  float* Qh[2] = {nullptr, nullptr};
  float* Ql[2] = {nullptr, nullptr};
  float* mixed_base = nullptr;          // one allocation holding both parities' blocks
  int64_t mpitch = 0;                   // two-phase: row pitch (floats, a multiple of 4)
  int mixed_kind = HYP_MIXED_TILE;      // kernel family (hyp_set_mixed_kernel)
  int wait_tries = hyp::kWaitTries;     // poll budget of the TMA kernel's barrier waits
  int tma_grid = 0;
  hyp::EosMixed eos_mixed;
  // two-phase (FP64): cell fluxes F [30][n], wave-speed bounds, face fluctuations [30][n+1]
  hyp::Eos2 eos2;
  hyp::Quad6D quad;        // Gauss-Legendre 6 on [0,1] (HLL path integrals)
  hyp::Quad6D lobatto;     // Gauss-Lobatto 6 on [0,1] (LxF path integrals)
  double* FF = nullptr;    // two-phase LxF: conservative face fluxes [30][n+1]
  // two-phase mixed precision (FP32): cell fluxes [30][n], speed bounds, face fluctuations [30][n+1]
  float* F32 = nullptr;
  float* smin32 = nullptr;
  float* smax32 = nullptr;
  float* DM32 = nullptr;
  float* DP32 = nullptr;
  float* FF32 = nullptr;
  double* smin = nullptr;
  double* smax = nullptr;
  double* DM = nullptr;
  double* DP = nullptr;
  hyp::DevState* st = nullptr;
  hyp::DevState* st_host = nullptr;  // pinned mirror
  int cur = 0;             // parity of the buffer that holds the current state
  int has_state = 0;       // a state was uploaded or installed
  long long steps_host = 0;
  double t_host = 0.0;
  int profiling = 0;
  cudaEvent_t ev[8];
  std::vector<cudaEvent_t> prof_ev;  // profiling: 3 events per step
  size_t prof_used = 0;
  hyp::StepTiming timing;
  // CUDA graph of an even number of steps, per starting parity
  // graphs keyed by the starting step index modulo the pattern period (2 for
  // FP64: buffer parity; 6 for mixed: parity x three max-lambda slots)
  cudaGraphExec_t graph[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  int graph_steps = 0;
  double* hist_dev = nullptr;  // hyp_step_times: device array of the per-step times
  long long hist_cap = 0;
  int hist_on = 0;             // set during hyp_step_times: steps launched one by one, each logged
  double graph_t_end = 0.0;
  std::string err;
  int64_t err_cell = -1;
  // one slab of a decomposed domain (hyp_slab.cu): ghost ends, the global dx
  int slab = 0;
  int slab_ghost[2] = {0, 0};  // the first / last cell is a ghost
  double slab_dx = 0.0;
  long long slab_cell_pass = -1;  // FP64: the step whose cell pass (fluxes, speeds) is done
  int relax = HYP_RELAX_NONE;     // two-phase pressure relaxation after each step (hyp_relax.cu)
  hyp::AdjTape* tape = nullptr;  // checkpoints and buffers of the adjoint (hyp_adjoint.cu)
  hyp::SnapBuf* snap = nullptr;  // snapshot buffers and writer (hyp_snapshot.cu)
};

// Context helpers shared by the C-ABI files (hyp_capi.cu): record an error
// message, copy the device status word to the host, turn a cell status into an
// error code.
int ctx_set_err(hyp_ctx* c, int code, const std::string& msg);
int ctx_sync_state(hyp_ctx* c);
int ctx_check_cell_error(hyp_ctx* c);
// Installing a state generated on the device (hyp_capi.cu): write it, FP64 [nvar][n],
// to ctx_install_target(c), then call ctx_finish_install(c, t0).
double* ctx_install_target(hyp_ctx* c);
int ctx_finish_install(hyp_ctx* c, double t0);
// The same from an FP64 state [nvar][n] at src: device memory, or host memory the
// device maps (mixed contexts read it in place, so the host link is the only transfer).
int ctx_finish_install_from(hyp_ctx* c, const double* src, double t0);
// The step's dx and kernel bc value of a context: the configuration's, or a slab's
// (its global dx and held ghost ends).
double ctx_dx(const hyp_ctx* c);
int ctx_bc(const hyp_ctx* c);

namespace hyp {
// adjoint buffers of a context (hyp_adjoint.cu)
void free_tape(hyp_ctx* c);
// snapshot buffers of a context (hyp_snapshot.cu)
void free_snap(hyp_ctx* c);
// single-phase FP64 step kernels (defined in hyp_step1.cu)
__global__ void __launch_bounds__(kBlock) cell1_f64_kernel(const double* __restrict__ Q, int64_t n, EosC e,
                                                           double* __restrict__ F, double* __restrict__ lam,
                                                           unsigned long long* lam_slot, const double* t_now,
                                                           double t_end, DevState* S);
__global__ void __launch_bounds__(kBlock) update1_f64_kernel(const double* __restrict__ Q, double* __restrict__ Qn,
                                                             int64_t n, const double* __restrict__ F,
                                                             const double* __restrict__ lam,
                                                             const unsigned long long* lam_in,
                                                             unsigned long long* lam_next, const double* t_in,
                                                             double* t_out, long long* steps, double t_end,
                                                             double cfl, double dx, int flux, int bc);
// single-phase FP64 launchers on a context (hyp_step1.cu)
cudaError_t launch_cell1_f64(hyp_ctx* c, int p, unsigned long long* lam_slot, const double* t_now, double t_end);
cudaError_t launch_update1_f64(hyp_ctx* c, int p, double t_end);
// single-phase mixed-precision launchers (hyp_step1_mixed.cu)
cudaError_t launch_split(hyp_ctx* c, const double* q, float* hi, float* lo);
cudaError_t launch_split_n(cudaStream_t s, const double* q, float* hi, float* lo, int rows, int64_t n, int64_t pitch);
cudaError_t launch_join_n(cudaStream_t s, const float* hi, const float* lo, double* q, int rows, int64_t n, int64_t pitch);
// two-phase mixed precision (hyp_step2_mixed.cu)
cudaError_t launch_cell2_mixed(hyp_ctx* c, int p, unsigned long long* lam_slot, const double* t_now, double t_end);
cudaError_t launch_face2_mixed(hyp_ctx* c, int p, double t_end);
cudaError_t launch_update2_mixed(hyp_ctx* c, int p, double t_end);
// the step's pair faces (HLL or LxF) and update in one kernel: replaces the two launches above
bool fused_face_update2_mixed(const hyp_ctx* c);
cudaError_t launch_face_update2_mixed(hyp_ctx* c, int p, double t_end);
int setup_mixed_tma(hyp_ctx* c);
cudaError_t launch_join(hyp_ctx* c, int p, double* q);
cudaError_t launch_join_rows(hyp_ctx* c, int p, double* q, int v0, int rows);
cudaError_t launch_lam1_mixed(hyp_ctx* c, int p, unsigned long long* slot);
cudaError_t launch_install1_mixed(hyp_ctx* c, const double* q, unsigned long long* slot);
cudaError_t launch_step1_mixed(hyp_ctx* c, long long k, double t_end);
// two-phase FP64 launchers (hyp_step2.cu)
cudaError_t launch_cell2_f64(hyp_ctx* c, int p, unsigned long long* lam_slot, const double* t_now, double t_end);
cudaError_t launch_face2_f64(hyp_ctx* c, int p, double t_end);
cudaError_t launch_update2_f64(hyp_ctx* c, int p, double t_end);
// two-phase pressure relaxation of the state the step of parity p wrote (hyp_relax.cu)
cudaError_t launch_relax2(hyp_ctx* c, int p, double t_end);
Quad6D gauss_legendre6();
Quad6D gauss_lobatto6();
}  // namespace hyp

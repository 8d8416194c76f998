// hyp_snapshot.cu -- solution snapshots and restart in the reference's file
// format (main.jl:62-95 save_data / read_data, :108 sol_%06i.csv, :174-198
// restart, :233-237 logging every log_freq steps).
//
// A snapshot is cons2prim of every cell on the device (the per-phase primitive
// 15-vectors [alpha, rho, u(3), S, A(9)] of HyperelasticityMPh.jl:106-133), copied
// to pinned host memory, then written as the reference writes it: a tab-separated
// header a1 r1 u11 u21 u31 S1 F111 ... F331 (and the a2 ... F332 columns of the
// second phase), one row per cell, each number in the shortest form that reads
// back to the same double, with Julia's fixed / scientific layout (1.0, 0.0001,
// 1.0e-5, 1.234567e6). A single-phase context writes the 15 columns of phase 1
// (alpha = 1).
//
// hyp_run_logged runs the main.jl time loop with logging: the initial state and
// every state whose step number is a multiple of log_freq are saved. The
// snapshot kernel runs on the context stream; its copy to the host runs on a
// second stream and the file is formatted and written by a host thread, so both
// overlap the steps that follow on the GPU.
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>
#include "hyp_internal.cuh"

namespace hyp {

struct SnapArg {
  EosC e[2];
  int model;  // HYP_MODEL_SINGLE: 15 columns, else 30
};

// prims [cols][n] of the FP64 state Q [nvar][n]
__global__ void snapshot_prims_kernel(SnapArg a, const double* __restrict__ Q, double* __restrict__ P, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double q[30], p[30];
  int np;
  if (a.model == HYP_MODEL_SINGLE) {
    q[0] = 1.0;
    for (int c = 0; c < 14; ++c) q[1 + c] = Q[c * n + i];
    np = 1;
  } else {
    for (int c = 0; c < 30; ++c) q[c] = Q[c * n + i];
    np = 2;
  }
  for (int ph = 0; ph < np; ++ph) phase_cons2prim(a.e[ph], q + 15 * ph, p + 15 * ph);
  for (int c = 0; c < 15 * np; ++c) P[c * n + i] = p[c];
}

// state Q [nvar][n] of prims P [cols][n] (prim2cons, HyperelasticityMPh.jl:63-90)
__global__ void snapshot_cons_kernel(SnapArg a, const double* __restrict__ P, double* __restrict__ Q, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int np = a.model == HYP_MODEL_SINGLE ? 1 : 2;
  double p[30], q[30];
  for (int c = 0; c < 15 * np; ++c) p[c] = P[c * n + i];
  for (int ph = 0; ph < np; ++ph) phase_prim2cons(a.e[ph], p + 15 * ph, q + 15 * ph);
  if (a.model == HYP_MODEL_SINGLE) {
    for (int c = 0; c < 14; ++c) Q[c * n + i] = q[1 + c];
  } else {
    for (int c = 0; c < 30; ++c) Q[c * n + i] = q[c];
  }
}

// ---- host: text format --------------------------------------------------------

// The shortest decimal that reads back to x, laid out as Julia prints a Float64:
// fixed notation for decimal exponents -5 < e < 6 (always with a fractional part,
// "1.0"), otherwise d.ddde[-]x ("1.0e-5", "1.234567e6"); NaN, Inf, -Inf.
static int format_double(double x, char* out) {
  if (std::isnan(x)) return (int)(std::strcpy(out, "NaN"), 3);
  if (std::isinf(x)) return x > 0 ? (int)(std::strcpy(out, "Inf"), 3) : (int)(std::strcpy(out, "-Inf"), 4);
  char* o = out;
  if (std::signbit(x)) {
    *o++ = '-';
    x = -x;
  }
  if (x == 0.0) {
    std::memcpy(o, "0.0", 3);
    return (int)(o - out) + 3;
  }
  char buf[40];
  const auto r = std::to_chars(buf, buf + sizeof buf - 1, x, std::chars_format::scientific);
  *r.ptr = '\0';
  // buf: d[.ddd]e(+|-)xx -> digits and decimal exponent
  char digits[24];
  int nd = 0;
  const char* p = buf;
  for (; p < r.ptr && *p != 'e'; ++p)
    if (*p != '.') digits[nd++] = *p;
  const int e = std::atoi(p + 1);
  while (nd > 1 && digits[nd - 1] == '0') --nd;
  if (e > -5 && e < 6) {
    if (e >= 0) {
      for (int k = 0; k <= e; ++k) *o++ = k < nd ? digits[k] : '0';
      *o++ = '.';
      if (nd > e + 1)
        for (int k = e + 1; k < nd; ++k) *o++ = digits[k];
      else
        *o++ = '0';
    } else {
      *o++ = '0';
      *o++ = '.';
      for (int k = 0; k < -e - 1; ++k) *o++ = '0';
      for (int k = 0; k < nd; ++k) *o++ = digits[k];
    }
  } else {
    *o++ = digits[0];
    *o++ = '.';
    if (nd > 1)
      for (int k = 1; k < nd; ++k) *o++ = digits[k];
    else
      *o++ = '0';
    *o++ = 'e';
    o += std::snprintf(o, 8, "%d", e);
  }
  return (int)(o - out);
}

static const char* kHeader30 =
    "a1\tr1\tu11\tu21\tu31\tS1\tF111\tF211\tF311\tF121\tF221\tF321\tF131\tF231\tF331\t"
    "a2\tr2\tu12\tu22\tu32\tS2\tF112\tF212\tF312\tF122\tF222\tF322\tF132\tF232\tF332";

// Writes prims P [cols][n] as the reference's TSV; rows formatted by up to 16 threads.
static int write_tsv(const char* path, const double* P, int64_t n, int cols) {
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return HYP_ERR_INVALID;
  std::string head(kHeader30);
  if (cols == 15) head = head.substr(0, head.find("\ta2"));
  head += "\n";
  bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
  const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(16, n / 4096));
  const int64_t rows_per = 65536;  // rows per formatted block, written in order
  std::vector<std::string> blk(nt);
  for (int64_t r0 = 0; ok && r0 < n; r0 += rows_per * nt) {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t]() {
        std::string& s = blk[t];
        s.clear();
        const int64_t a = r0 + t * rows_per, b = std::min<int64_t>(n, a + rows_per);
        char num[40];
        for (int64_t i = a; i < b; ++i) {
          for (int c = 0; c < cols; ++c) {
            if (c) s.push_back('\t');
            s.append(num, (size_t)format_double(P[(int64_t)c * n + i], num));
          }
          s.push_back('\n');
        }
      });
    for (auto& x : th) x.join();
    for (int t = 0; ok && t < nt; ++t) ok = std::fwrite(blk[t].data(), 1, blk[t].size(), f) == blk[t].size();
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? HYP_OK : HYP_ERR_INVALID;
}

// Reads the reference's TSV (header line, then n rows of `cols` numbers) into P [cols][n];
// HYP_ERR_INVALID for a missing file, a row with fewer or more numbers, or a row count
// other than n.
static int read_tsv(const char* path, double* P, int64_t n, int cols) {
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return HYP_ERR_INVALID;
  std::string line;
  int rc = HYP_OK;
  int64_t row = -1;
  char buf[1 << 16];
  std::string acc;
  auto take = [&](const std::string& l) {
    if (row < 0) {  // header
      row = 0;
      return;
    }
    if (l.empty()) return;
    if (row >= n) {
      rc = HYP_ERR_INVALID;
      return;
    }
    const char* p = l.c_str();
    for (int c = 0; c < cols; ++c) {
      char* end = nullptr;
      const double v = std::strtod(p, &end);
      if (end == p) {
        rc = HYP_ERR_INVALID;
        return;
      }
      P[(int64_t)c * n + row] = v;
      p = end;
    }
    while (*p == ' ' || *p == '\t' || *p == '\r') ++p;
    if (*p != '\0') {  // more columns than the context's model has
      rc = HYP_ERR_INVALID;
      return;
    }
    ++row;
  };
  size_t got;
  while (rc == HYP_OK && (got = std::fread(buf, 1, sizeof buf, f)) > 0) {
    size_t s0 = 0;
    for (size_t k = 0; k < got; ++k)
      if (buf[k] == '\n') {
        acc.append(buf + s0, k - s0);
        take(acc);
        acc.clear();
        s0 = k + 1;
      }
    acc.append(buf + s0, got - s0);
  }
  if (rc == HYP_OK && !acc.empty()) take(acc);
  std::fclose(f);
  if (rc == HYP_OK && row != n) rc = HYP_ERR_INVALID;
  return rc;
}

}  // namespace hyp

namespace hyp {

struct SnapBuf {
  int cols = 0;
  int64_t n = 0;
  double* dev[2] = {nullptr, nullptr};   // prims [cols][n]
  double* host[2] = {nullptr, nullptr};  // pinned copies
  cudaStream_t copy = nullptr;           // device-to-host copies, off the stepping stream
  cudaEvent_t ready[2] = {nullptr, nullptr};
  cudaEvent_t copied[2] = {nullptr, nullptr};
  std::thread writer;
  int writer_rc = HYP_OK;
};

void free_snap(hyp_ctx* c) {
  SnapBuf* s = c->snap;
  if (!s) return;
  if (s->writer.joinable()) s->writer.join();
  if (s->copy) cudaStreamSynchronize(s->copy);
  for (int k = 0; k < 2; ++k) {
    cudaFree(s->dev[k]);
    if (s->host[k]) cudaFreeHost(s->host[k]);
    if (s->ready[k]) cudaEventDestroy(s->ready[k]);
    if (s->copied[k]) cudaEventDestroy(s->copied[k]);
  }
  if (s->copy) cudaStreamDestroy(s->copy);
  delete s;
  c->snap = nullptr;
}

static SnapArg snap_arg(const hyp_ctx* c) {
  SnapArg a;
  a.e[0] = c->eos[0];
  a.e[1] = c->eos[1];
  a.model = c->cfg.model;
  return a;
}

static int snap_cols(const hyp_ctx* c) { return c->cfg.model == HYP_MODEL_SINGLE ? 15 : 30; }

}  // namespace hyp

using namespace hyp;

#define SCK(call)                                                                             \
  do {                                                                                        \
    cudaError_t _e = (call);                                                                  \
    if (_e != cudaSuccess) return ctx_set_err(c, HYP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

static int ensure_snap(hyp_ctx* c) {
  if (c->snap) return HYP_OK;
  SnapBuf* s = c->snap = new SnapBuf();
  s->cols = snap_cols(c);
  s->n = c->n;
  const size_t bytes = (size_t)s->cols * c->n * sizeof(double);
  for (int k = 0; k < 2; ++k) {
    SCK(cudaMalloc(&s->dev[k], bytes));
    SCK(cudaMallocHost(&s->host[k], bytes));
    SCK(cudaEventCreateWithFlags(&s->ready[k], cudaEventDisableTiming));
    SCK(cudaEventCreateWithFlags(&s->copied[k], cudaEventDisableTiming));
  }
  SCK(cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking));
  return HYP_OK;
}

// Enqueues cons2prim of the current state into dev[slot] (context stream) and its
// copy into host[slot] (copy stream); returns without waiting.
static int enqueue_snapshot(hyp_ctx* c, int slot) {
  SnapBuf* s = c->snap;
  const double* src = c->Q[c->cur];
  if (c->cfg.precision == HYP_PREC_MIXED) {  // (hi, lo) -> FP64 in the other parity's block
    double* stage = (double*)c->Qh[1 - c->cur];
    SCK(launch_join(c, c->cur, stage));
    src = stage;
  }
  snapshot_prims_kernel<<<(unsigned)((c->n + 127) / 128), 128, 0, c->stream>>>(snap_arg(c), src, s->dev[slot], c->n);
  SCK(cudaGetLastError());
  SCK(cudaEventRecord(s->ready[slot], c->stream));
  SCK(cudaStreamWaitEvent(s->copy, s->ready[slot], 0));
  SCK(cudaMemcpyAsync(s->host[slot], s->dev[slot], (size_t)s->cols * c->n * sizeof(double), cudaMemcpyDeviceToHost,
                      s->copy));
  SCK(cudaEventRecord(s->copied[slot], s->copy));
  return HYP_OK;
}

// Writes host[slot] to `path` on a host thread once its copy has landed; the previous
// writer is joined first (its status is kept).
static void start_writer(hyp_ctx* c, int slot, const std::string& path) {
  SnapBuf* s = c->snap;
  if (s->writer.joinable()) s->writer.join();
  const int dev = c->device;
  s->writer = std::thread([s, slot, path, dev]() {
    cudaSetDevice(dev);
    int rc = cudaEventSynchronize(s->copied[slot]) == cudaSuccess ? HYP_OK : HYP_ERR_CUDA;
    if (rc == HYP_OK) rc = write_tsv(path.c_str(), s->host[slot], s->n, s->cols);
    if (rc != HYP_OK && s->writer_rc == HYP_OK) s->writer_rc = rc;
  });
}

static int finish_writer(hyp_ctx* c) {
  SnapBuf* s = c->snap;
  if (s->writer.joinable()) s->writer.join();
  const int rc = s->writer_rc;
  s->writer_rc = HYP_OK;
  if (rc != HYP_OK) return ctx_set_err(c, rc, "writing a snapshot file failed");
  return HYP_OK;
}

extern "C" int hyp_snapshot(hyp_ctx* c, double* P) {
  if (!c || !P) return HYP_ERR_INVALID;
  SCK(cudaSetDevice(c->device));
  int rc = ensure_snap(c);
  if (rc != HYP_OK) return rc;
  if ((rc = finish_writer(c)) != HYP_OK) return rc;
  if ((rc = enqueue_snapshot(c, 0)) != HYP_OK) return rc;
  SCK(cudaEventSynchronize(c->snap->copied[0]));
  std::memcpy(P, c->snap->host[0], (size_t)c->snap->cols * c->n * sizeof(double));
  return HYP_OK;
}

extern "C" int hyp_save_snapshot(hyp_ctx* c, const char* path) {
  if (!c || !path) return HYP_ERR_INVALID;
  SCK(cudaSetDevice(c->device));
  int rc = ensure_snap(c);
  if (rc != HYP_OK) return rc;
  if ((rc = finish_writer(c)) != HYP_OK) return rc;
  if ((rc = enqueue_snapshot(c, 0)) != HYP_OK) return rc;
  start_writer(c, 0, path);
  return finish_writer(c);
}

extern "C" int hyp_load_snapshot(hyp_ctx* c, const char* path, double t0) {
  if (!c || !path) return HYP_ERR_INVALID;
  SCK(cudaSetDevice(c->device));
  const int cols = snap_cols(c);
  std::vector<double> P((size_t)cols * c->n), Q((size_t)c->nvar * c->n);
  if (read_tsv(path, P.data(), c->n, cols) != HYP_OK)
    return ctx_set_err(c, HYP_ERR_INVALID, std::string("hyp_load_snapshot: cannot read ") + path);
  double *dP = nullptr, *dQ = nullptr;
  int rc = HYP_OK;
  if (cudaMalloc(&dP, P.size() * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dQ, Q.size() * sizeof(double)) != cudaSuccess)
    rc = ctx_set_err(c, HYP_ERR_CUDA, "hyp_load_snapshot: cudaMalloc");
  if (rc == HYP_OK &&
      cudaMemcpyAsync(dP, P.data(), P.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
    rc = ctx_set_err(c, HYP_ERR_CUDA, "hyp_load_snapshot: copy");
  if (rc == HYP_OK) {
    snapshot_cons_kernel<<<(unsigned)((c->n + 127) / 128), 128, 0, c->stream>>>(snap_arg(c), dP, dQ, c->n);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(Q.data(), dQ, Q.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
      rc = ctx_set_err(c, HYP_ERR_CUDA, "hyp_load_snapshot: prim2cons");
  }
  cudaFree(dP);
  cudaFree(dQ);
  if (rc != HYP_OK) return rc;
  return hyp_upload(c, Q.data(), c->n, c->nvar, t0);
}

extern "C" int hyp_run_logged(hyp_ctx* c, double t_end, int max_steps, int log_freq, const char* dir,
                              int64_t first_step, int* steps_done, double* t_out) {
  if (!c || !dir || log_freq <= 0 || first_step < 0) return HYP_ERR_INVALID;
  if (max_steps <= 0 && std::isinf(t_end))
    return ctx_set_err(c, HYP_ERR_INVALID, "hyp_run_logged: neither max_steps nor t_end bounds the run");
  SCK(cudaSetDevice(c->device));
  int rc = ensure_snap(c);
  if (rc != HYP_OK) return rc;
  if ((rc = finish_writer(c)) != HYP_OK) return rc;
  auto file = [&](int64_t step) {
    char name[32];
    std::snprintf(name, sizeof name, "sol_%06lld.csv", (long long)step);  // main.jl:108
    std::string d(dir);
    if (!d.empty() && d.back() != '/') d += '/';
    return d + name;
  };
  int slot = 0;
  int64_t step = first_step;
  long long done = 0;
  double t = c->t_host;
  // the initial state is saved (main.jl:196-197)
  if ((rc = enqueue_snapshot(c, slot)) != HYP_OK) return rc;
  start_writer(c, slot, file(step));
  slot ^= 1;
  while (rc == HYP_OK && t < t_end && (max_steps <= 0 || done < max_steps)) {
    long long chunk = log_freq - (step % log_freq);
    if (max_steps > 0 && chunk > max_steps - done) chunk = max_steps - done;
    int sd = 0;
    if ((rc = hyp_step(c, (int)chunk, t_end, &sd, &t)) != HYP_OK) break;
    done += sd;
    step += sd;
    if (sd > 0 && step % log_freq == 0) {  // main.jl:233-237
      if ((rc = enqueue_snapshot(c, slot)) != HYP_OK) break;
      start_writer(c, slot, file(step));
      slot ^= 1;
    }
    if (sd < chunk) break;  // t reached t_end
  }
  if (rc == HYP_OK && !(t < t_end)) {  // the run reached T: result.csv (main.jl:242-244)
    std::string d(dir);
    if (!d.empty() && d.back() != '/') d += '/';
    if ((rc = enqueue_snapshot(c, slot)) == HYP_OK) start_writer(c, slot, d + "result.csv");
  }
  const int wrc = finish_writer(c);
  if (rc == HYP_OK) rc = wrc;
  if (steps_done) *steps_done = (int)done;
  if (t_out) *t_out = c->t_host;
  return rc;
}

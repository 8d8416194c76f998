// Floating-point operations per cell-update of the step's formulation, counted by
// running the product's FP64 physics (hyp_physics.cuh, hyp_physics_mph.cuh) on the
// host with `double` replaced by a scalar type that counts every add, multiply,
// divide, square root, transcendental and compare it executes. Built and run by
// tests/test_flop_count.py; prints one JSON object.
//
// A cell-update of the single-phase Rusanov step: the cell's pass (cons2prim, stress,
// flux, acoustic tensor, spectral radius), one face (0.5 (f_L + f_R) - 0.5 lambda
// (Q_R - Q_L) over 14 variables) and the update (14 variables). Of the two-phase
// path-conservative HLL step: the cell's pass for both phases (flux and speed
// bounds), one face (midpoint speeds, three six-node path integrals of B) and the
// update of 30 variables. Flops: add + mul + div + sqrt (a fused multiply-add counts
// two); the FP32 seed of the spectral radius is outside the count.
#include <cmath>
#include <cstdio>

struct Ops {
  long add = 0, mul = 0, div = 0, sqrt = 0, trans = 0, cmp = 0;
};
static Ops ops;

struct Cnt {
  double v;
  Cnt() = default;
  Cnt(double x) : v(x) {}
  Cnt(float x) : v(x) {}
  Cnt(int x) : v(x) {}
  Cnt(long x) : v((double)x) {}
  Cnt(long long x) : v((double)x) {}
  explicit operator float() const { return (float)v; }
  explicit operator int() const { return (int)v; }
  explicit operator long long() const { return (long long)v; }
  Cnt& operator+=(Cnt b) { ops.add++; v += b.v; return *this; }
  Cnt& operator-=(Cnt b) { ops.add++; v -= b.v; return *this; }
  Cnt& operator*=(Cnt b) { ops.mul++; v *= b.v; return *this; }
  Cnt& operator/=(Cnt b) { ops.div++; v /= b.v; return *this; }
};
inline Cnt operator+(Cnt a, Cnt b) { ops.add++; return a.v + b.v; }
inline Cnt operator-(Cnt a, Cnt b) { ops.add++; return a.v - b.v; }
inline Cnt operator*(Cnt a, Cnt b) { ops.mul++; return a.v * b.v; }
inline Cnt operator/(Cnt a, Cnt b) { ops.div++; return a.v / b.v; }
inline Cnt operator-(Cnt a) { return -a.v; }
inline Cnt operator+(Cnt a) { return a; }
inline bool operator<(Cnt a, Cnt b) { ops.cmp++; return a.v < b.v; }
inline bool operator>(Cnt a, Cnt b) { ops.cmp++; return a.v > b.v; }
inline bool operator<=(Cnt a, Cnt b) { ops.cmp++; return a.v <= b.v; }
inline bool operator>=(Cnt a, Cnt b) { ops.cmp++; return a.v >= b.v; }
inline bool operator==(Cnt a, Cnt b) { return a.v == b.v; }
inline bool operator!=(Cnt a, Cnt b) { return a.v != b.v; }
inline Cnt sqrt(Cnt a) { ops.sqrt++; return std::sqrt(a.v); }
inline Cnt fabs(Cnt a) { return std::fabs(a.v); }
inline Cnt fmax(Cnt a, Cnt b) { ops.cmp++; return std::fmax(a.v, b.v); }
inline Cnt fmin(Cnt a, Cnt b) { ops.cmp++; return std::fmin(a.v, b.v); }
inline Cnt fma(Cnt a, Cnt b, Cnt c) { ops.mul++; ops.add++; return std::fma(a.v, b.v, c.v); }
inline Cnt exp(Cnt a) { ops.trans++; return std::exp(a.v); }
inline Cnt log(Cnt a) { ops.trans++; return std::log(a.v); }
inline Cnt expm1(Cnt a) { ops.trans++; return std::expm1(a.v); }
inline Cnt log1p(Cnt a) { ops.trans++; return std::log1p(a.v); }
inline Cnt pow(Cnt a, Cnt b) { ops.trans++; return std::pow(a.v, b.v); }
inline Cnt cbrt(Cnt a) { ops.trans++; return std::cbrt(a.v); }
inline Cnt copysign(Cnt a, Cnt b) { return std::copysign(a.v, b.v); }
inline bool isfinite(Cnt a) { return std::isfinite(a.v); }
inline bool isnan(Cnt a) { return std::isnan(a.v); }

#define double Cnt
#include "../hyperelasticsolver_gb300/csrc/hyp_physics.cuh"
#include "../hyperelasticsolver_gb300/csrc/hyp_physics_mph.cuh"
#undef double

using namespace hyp;

static long flops(const Ops& o) { return o.add + o.mul + o.div + o.sqrt; }
static Ops diff(const Ops& a, const Ops& b) {
  Ops d;
  d.add = a.add - b.add;
  d.mul = a.mul - b.mul;
  d.div = a.div - b.div;
  d.sqrt = a.sqrt - b.sqrt;
  d.trans = a.trans - b.trans;
  d.cmp = a.cmp - b.cmp;
  return d;
}
static void print(const char* name, const Ops& o, bool last) {
  printf("\"%s\": {\"flops\": %ld, \"add\": %ld, \"mul\": %ld, \"div\": %ld, \"sqrt\": %ld, \"transcendental\": %ld, "
         "\"compare\": %ld}%s\n",
         name, flops(o), o.add, o.mul, o.div, o.sqrt, o.trans, o.cmp, last ? "" : ",");
}

// one phase's conservative state (15) from primitives: alpha, rho_true, u, S = 0, A
static void phase_state(const EosC& e, Cnt alpha, Cnt rho, Cnt u0, Cnt u1, Cnt u2, Cnt strain, Cnt* q) {
  Cnt p[15];
  p[0] = alpha;
  p[1] = rho;
  p[2] = u0;
  p[3] = u1;
  p[4] = u2;
  p[5] = 0.0;
  const Cnt s = std::cbrt((e.rho0 / rho).v);  // det A = rho0 / rho
  const double off[9] = {0, 0.3, -0.2, 0.1, 0, 0.25, -0.15, 0.05, 0};
  for (int k = 0; k < 9; ++k) p[6 + k] = (k % 4 == 0 ? s : Cnt(0.0)) + strain * off[k];
  phase_prim2cons(e, p, q);
}

int main() {
  const EosC e = make_eos(8.93, 4.6, 3.9e-4, 300.0, 2.1, 1.0, 3.0, 2.0);
  const EosC e2 = make_eos(8.93, 4.6, 3.9e-4, 300.0, 2.1 * std::sqrt(0.1), 1.0, 3.0, 2.0);
  printf("{\n");
  // ---- single phase, Rusanov --------------------------------------------------
  {
    Cnt qa[15], qb[15];
    phase_state(e, 1.0, 8.93 * 1.02, 0.3, -0.2, 0.1, 0.03, qa);
    phase_state(e, 1.0, 8.93 * 0.99, -0.1, 0.4, 0.2, 0.02, qb);
    Cnt fb[14], s0b[3], lamb;  // the right neighbour's pass, outside the count
    {
      Prim P;
      cons_to_prim(e, qb[0], qb + 2, qb[5], qb + 6, P);
      const StressC c = stress_coeffs(e, P.k, P.w, P.xm1);
      phase_flux(e, qb[0], P, c, fb, s0b);
      lamb = fabs(P.u[0]) + phase_cmax(e, P, c);
    }
    const Ops o0 = ops;
    Prim P;
    cons_to_prim(e, qa[0], qa + 2, qa[5], qa + 6, P);
    const StressC c = stress_coeffs(e, P.k, P.w, P.xm1);
    Cnt f[14], s0[3];
    phase_flux(e, qa[0], P, c, f, s0);
    const Cnt lam = fabs(P.u[0]) + phase_cmax(e, P, c);
    const Ops o1 = ops;
    // one Rusanov face over the 14 variables
    const Cnt hl = 0.5 * fmax(lam, lamb);
    Cnt face[14];
    for (int v = 0; v < 14; ++v) face[v] = 0.5 * (f[v] + fb[v]) - hl * (qb[1 + v] - qa[1 + v]);
    const Ops o2 = ops;
    const Cnt dtdx = 0.5 / lam;  // cfl / max lambda
    Cnt qn[14];
    for (int v = 0; v < 14; ++v) qn[v] = qa[1 + v] - dtdx * (face[v] - f[v]);  // F_{i+1/2} - F_{i-1/2}
    const Ops o3 = ops;
    (void)qn;
    Ops t = diff(o3, o0);
    print("single_cell_pass", diff(o1, o0), false);
    print("single_face", diff(o2, o1), false);
    print("single_update", diff(o3, o2), false);
    print("single_cell_update", t, false);
  }
  // ---- two phases, path-conservative HLL ---------------------------------------
  {
    EosC eos[2] = {e, e2};
    Cnt QL[30], QR[30];
    phase_state(e, 0.7, 8.93 * 1.01, 0.2, -0.1, 0.05, 0.02, QL);
    phase_state(e2, 0.3, 8.93 * 0.99, 0.1, 0.2, -0.1, 0.03, QL + 15);
    phase_state(e, 0.4, 8.93 * 0.995, -0.1, 0.3, 0.1, 0.01, QR);
    phase_state(e2, 0.6, 8.93 * 1.005, 0.05, -0.2, 0.2, 0.02, QR + 15);
    Quad6D qd;
    const double gx[6] = {0.0337652428984240, 0.1693953067668677, 0.3806904069584015,
                          0.6193095930415985, 0.8306046932331323, 0.9662347571015760};
    const double gw[6] = {0.0856622461895852, 0.1803807865240693, 0.2339569672863455,
                          0.2339569672863455, 0.1803807865240693, 0.0856622461895852};
    for (int i = 0; i < 6; ++i) {
      qd.x[i] = gx[i];
      qd.w[i] = gw[i];
    }
    const Ops o0 = ops;
    Cnt FL[30], FR[30];
    flux2(eos, QL, FL);
    Cnt sminL, smaxL;
    speeds2(eos, QL, sminL, smaxL);
    const Ops o1 = ops;
    flux2(eos, QR, FR);
    Cnt sminR, smaxR;
    speeds2(eos, QR, sminR, smaxR);
    const Ops o1b = ops;
    Cnt dm[30], dp[30];
    hll_face2(eos, qd, QL, QR, FL, FR, sminL, smaxR, dm, dp);
    const Ops o2 = ops;
    const Cnt dtdx = 0.5 / fmax(smaxL, -sminL);
    Cnt qn[30];
    for (int v = 0; v < 30; ++v) qn[v] = QL[v] - dtdx * (dm[v] + dp[v]);
    const Ops o3 = ops;
    (void)qn;
    Ops cell = diff(o1, o0), face = diff(o2, o1b), upd = diff(o3, o2), t;
    t.add = cell.add + face.add + upd.add;
    t.mul = cell.mul + face.mul + upd.mul;
    t.div = cell.div + face.div + upd.div;
    t.sqrt = cell.sqrt + face.sqrt + upd.sqrt;
    t.trans = cell.trans + face.trans + upd.trans;
    t.cmp = cell.cmp + face.cmp + upd.cmp;
    print("twophase_cell_pass", cell, false);
    print("twophase_hll_face", face, false);
    print("twophase_update", upd, false);
    print("twophase_cell_update", t, true);
  }
  printf("}\n");
  return 0;
}

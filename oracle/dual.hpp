// oracle/dual.hpp -- forward-mode dual numbers for the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY. This header belongs to the oracle: a CPU
// restatement of BlackSiberian/HyperelasticSolver used by tests/, by
// __graft_entry__.smoke() and by bench.py's cpu_baseline / reference arm
// as the checker. Nothing in the product (hyperelasticsolver_gb300/) includes it.
//
// The reference differentiates its energy and stress with ForwardDiff.jl
// (EquationsOfState.jl:169,183 `gradient`, :200,226 `jacobian`;
// HyperelasticityMPh.jl:212 `derivative`; NumFluxes.jl:41,100 `derivative`).
// ForwardDiff is not vendored in the reference and its version is not pinned
// (no Manifest.toml). Its published algorithm is forward-mode AD with dual
// numbers: each elementary operation propagates a value and a vector of
// partials with the rules below (ForwardDiff's `dual.jl`, with DiffRules for
// the unary functions). Nested duals (`Dual<Dual<double,9>,9>`) restate the
// reference's jacobian-of-gradient in `acoustic` (EquationsOfState.jl:223-246).
#pragma once
#include <cmath>
#include <type_traits>

namespace hyp_oracle {

template <class T, int N>
struct Dual {
  T v;
  T d[N];
  Dual() : v(0.0) {
    for (int i = 0; i < N; ++i) d[i] = T(0.0);
  }
  Dual(double x) : v(x) {  // constants carry zero partials
    for (int i = 0; i < N; ++i) d[i] = T(0.0);
  }
  template <class U, class = std::enable_if_t<!std::is_same<U, double>::value &&
                                                std::is_convertible<U, T>::value>>
  Dual(const U& x) : v(x) {
    for (int i = 0; i < N; ++i) d[i] = T(0.0);
  }
};

template <class X> struct is_dual : std::false_type {};
template <class T, int N> struct is_dual<Dual<T, N>> : std::true_type {};

// value of the innermost scalar (for comparisons such as LU pivoting and the
// entropy clamp, which ForwardDiff performs on values)
inline double value_of(double x) { return x; }
template <class T, int N> double value_of(const Dual<T, N>& x) { return value_of(x.v); }

// ---- arithmetic: Dual (op) Dual ------------------------------------------
template <class T, int N> Dual<T, N> operator-(const Dual<T, N>& x) {
  Dual<T, N> r; r.v = -x.v;
  for (int i = 0; i < N; ++i) r.d[i] = -x.d[i];
  return r;
}
template <class T, int N> Dual<T, N> operator+(const Dual<T, N>& x, const Dual<T, N>& y) {
  Dual<T, N> r; r.v = x.v + y.v;
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] + y.d[i];
  return r;
}
template <class T, int N> Dual<T, N> operator-(const Dual<T, N>& x, const Dual<T, N>& y) {
  Dual<T, N> r; r.v = x.v - y.v;
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] - y.d[i];
  return r;
}
// ForwardDiff: partials(x)*value(y) + partials(y)*value(x)
template <class T, int N> Dual<T, N> operator*(const Dual<T, N>& x, const Dual<T, N>& y) {
  Dual<T, N> r; r.v = x.v * y.v;
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] * y.v + y.d[i] * x.v;
  return r;
}
// ForwardDiff: partials(x)*inv(vy) + partials(y)*(-(vx/(vy*vy)))
template <class T, int N> Dual<T, N> operator/(const Dual<T, N>& x, const Dual<T, N>& y) {
  Dual<T, N> r; r.v = x.v / y.v;
  T a = T(1.0) / y.v;
  T b = -(x.v / (y.v * y.v));
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] * a + y.d[i] * b;
  return r;
}
// ---- Dual (op) scalar of the value type or double ------------------------
template <class T, int N, class S, class = std::enable_if_t<!is_dual<S>::value || std::is_same<S, T>::value>>
Dual<T, N> operator+(const Dual<T, N>& x, const S& y) {
  Dual<T, N> r = x; r.v = x.v + y; return r;
}
template <class T, int N, class S, class = std::enable_if_t<!is_dual<S>::value || std::is_same<S, T>::value>>
Dual<T, N> operator+(const S& y, const Dual<T, N>& x) {
  Dual<T, N> r = x; r.v = y + x.v; return r;
}
template <class T, int N, class S, class = std::enable_if_t<!is_dual<S>::value || std::is_same<S, T>::value>>
Dual<T, N> operator-(const Dual<T, N>& x, const S& y) {
  Dual<T, N> r = x; r.v = x.v - y; return r;
}
template <class T, int N, class S, class = std::enable_if_t<!is_dual<S>::value || std::is_same<S, T>::value>>
Dual<T, N> operator-(const S& y, const Dual<T, N>& x) {
  Dual<T, N> r; r.v = y - x.v;
  for (int i = 0; i < N; ++i) r.d[i] = -x.d[i];
  return r;
}
template <class T, int N, class S, class = std::enable_if_t<!is_dual<S>::value || std::is_same<S, T>::value>>
Dual<T, N> operator*(const Dual<T, N>& x, const S& y) {
  Dual<T, N> r; r.v = x.v * y;
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] * y;
  return r;
}
template <class T, int N, class S, class = std::enable_if_t<!is_dual<S>::value || std::is_same<S, T>::value>>
Dual<T, N> operator*(const S& y, const Dual<T, N>& x) {
  Dual<T, N> r; r.v = y * x.v;
  for (int i = 0; i < N; ++i) r.d[i] = y * x.d[i];
  return r;
}
template <class T, int N, class S, class = std::enable_if_t<!is_dual<S>::value || std::is_same<S, T>::value>>
Dual<T, N> operator/(const Dual<T, N>& x, const S& y) {
  Dual<T, N> r; r.v = x.v / y;
  for (int i = 0; i < N; ++i) r.d[i] = x.d[i] / y;
  return r;
}
template <class T, int N, class S, class = std::enable_if_t<!is_dual<S>::value || std::is_same<S, T>::value>>
Dual<T, N> operator/(const S& x, const Dual<T, N>& y) {
  Dual<T, N> r; r.v = x / y.v;
  T b = -(x / (y.v * y.v));
  for (int i = 0; i < N; ++i) r.d[i] = y.d[i] * b;
  return r;
}
template <class T, int N, class S> Dual<T, N>& operator+=(Dual<T, N>& x, const S& y) { x = x + y; return x; }
template <class T, int N, class S> Dual<T, N>& operator-=(Dual<T, N>& x, const S& y) { x = x - y; return x; }
template <class T, int N, class S> Dual<T, N>& operator*=(Dual<T, N>& x, const S& y) { x = x * y; return x; }

// ---- a dual of a lower nesting level (S convertible to T) is lifted into T --
// (a constant with respect to the inner partials): lets an EOS modulus that
// carries outer partials multiply the nested duals of the stress derivatives.
template <class T, int N, class S>
using lift_r = std::enable_if_t<is_dual<S>::value && !std::is_same<S, T>::value && std::is_convertible<S, T>::value,
                                Dual<T, N>>;
template <class T, int N, class S> lift_r<T, N, S> operator+(const Dual<T, N>& x, const S& y) { return x + T(y); }
template <class T, int N, class S> lift_r<T, N, S> operator+(const S& y, const Dual<T, N>& x) { return T(y) + x; }
template <class T, int N, class S> lift_r<T, N, S> operator-(const Dual<T, N>& x, const S& y) { return x - T(y); }
template <class T, int N, class S> lift_r<T, N, S> operator-(const S& y, const Dual<T, N>& x) { return T(y) - x; }
template <class T, int N, class S> lift_r<T, N, S> operator*(const Dual<T, N>& x, const S& y) { return x * T(y); }
template <class T, int N, class S> lift_r<T, N, S> operator*(const S& y, const Dual<T, N>& x) { return T(y) * x; }
template <class T, int N, class S> lift_r<T, N, S> operator/(const Dual<T, N>& x, const S& y) { return x / T(y); }
template <class T, int N, class S> lift_r<T, N, S> operator/(const S& y, const Dual<T, N>& x) { return T(y) / x; }

// ---- comparisons act on values --------------------------------------------
template <class A, class B, class = std::enable_if_t<is_dual<A>::value || is_dual<B>::value>>
bool operator<(const A& a, const B& b) { return value_of(a) < value_of(b); }
template <class A, class B, class = std::enable_if_t<is_dual<A>::value || is_dual<B>::value>>
bool operator>(const A& a, const B& b) { return value_of(a) > value_of(b); }

// ---- unary functions (DiffRules) ------------------------------------------
using std::sqrt; using std::exp; using std::log; using std::pow; using std::abs;

template <class T, int N> Dual<T, N> sqrt(const Dual<T, N>& x) {
  Dual<T, N> r; r.v = sqrt(x.v);
  T k = T(1.0) / (2.0 * r.v);  // inv(2*sqrt(x))
  for (int i = 0; i < N; ++i) r.d[i] = k * x.d[i];
  return r;
}
template <class T, int N> Dual<T, N> exp(const Dual<T, N>& x) {
  Dual<T, N> r; r.v = exp(x.v);
  for (int i = 0; i < N; ++i) r.d[i] = r.v * x.d[i];
  return r;
}
template <class T, int N> Dual<T, N> log(const Dual<T, N>& x) {
  Dual<T, N> r; r.v = log(x.v);
  T k = T(1.0) / x.v;
  for (int i = 0; i < N; ++i) r.d[i] = k * x.d[i];
  return r;
}
// x^y for real y (ForwardDiff: partials(x) * y * v^(y-1))
template <class T, int N> Dual<T, N> pow(const Dual<T, N>& x, double y) {
  Dual<T, N> r; r.v = pow(x.v, y);
  if (y == 0.0) return r;
  T k = pow(x.v, y - 1.0);
  for (int i = 0; i < N; ++i) r.d[i] = (x.d[i] * y) * k;
  return r;
}
template <class T, int N> Dual<T, N> abs(const Dual<T, N>& x) {
  return value_of(x) < 0.0 ? -x : x;
}
template <class T, int N> Dual<T, N> inv(const Dual<T, N>& x) {  // -abs2(inv(x))
  Dual<T, N> r; r.v = T(1.0) / x.v;
  T k = -(r.v * r.v);
  for (int i = 0; i < N; ++i) r.d[i] = k * x.d[i];
  return r;
}
inline double inv(double x) { return 1.0 / x; }

// x^n for integer n as Julia evaluates it: Float64 x^2 is x*x (literal_pow);
// for duals ForwardDiff uses v^n and n*v^(n-1)*partials.
inline double ipow2(double x) { return x * x; }
template <class T, int N> Dual<T, N> ipow2(const Dual<T, N>& x) {
  Dual<T, N> r; r.v = ipow2(x.v);
  for (int i = 0; i < N; ++i) r.d[i] = (x.d[i] * 2.0) * x.v;
  return r;
}

}  // namespace hyp_oracle

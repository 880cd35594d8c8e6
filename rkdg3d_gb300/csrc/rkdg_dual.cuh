// Forward-mode dual numbers for the discrete adjoint.
//
// Dual<N> carries a value and N directional derivatives.  The physics and
// Riemann-solver templates (rkdg_physics.cuh) are instantiated with it to get
// exact Jacobians of the nodal Euler flux, the numerical fluxes (including
// the boundary ghost states) and the limiter indicator.  Branches (min/max,
// HLL/HLLC cases, TRRS shock/rarefaction switches, the indicator's
// thresholds) follow the primal values, which is the derivative of the
// active branch.
#pragma once

#include <cuda_runtime.h>

namespace rkdg {

// keep the scalar overloads visible next to the Dual ones
using ::fabs;
using ::fmax;
using ::fmin;
using ::pow;
using ::sqrt;

template <int N>
struct Dual {
  double v;
  double d[N];
  __host__ __device__ Dual() : v(0.0) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  __host__ __device__ Dual(double x) : v(x) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  __host__ __device__ static Dual var(double x, int i) {
    Dual r(x);
    r.d[i] = 1.0;
    return r;
  }
  __host__ __device__ Dual& operator+=(const Dual& o) {
    v += o.v;
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] += o.d[i];
    return *this;
  }
  __host__ __device__ Dual& operator-=(const Dual& o) {
    v -= o.v;
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] -= o.d[i];
    return *this;
  }
  __host__ __device__ Dual& operator*=(const Dual& o) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = d[i] * o.v + v * o.d[i];
    v *= o.v;
    return *this;
  }
  __host__ __device__ Dual& operator/=(const Dual& o) {
    const double inv = 1.0 / o.v;
    const double q = v * inv;
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = (d[i] - q * o.d[i]) * inv;
    v = q;
    return *this;
  }
};

template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator+(Dual<N> a, const Dual<N>& b) { return a += b; }
template <int N>
__host__ __device__ inline Dual<N> operator-(Dual<N> a, const Dual<N>& b) { return a -= b; }
template <int N>
__host__ __device__ inline Dual<N> operator*(Dual<N> a, const Dual<N>& b) { return a *= b; }
template <int N>
__host__ __device__ inline Dual<N> operator/(Dual<N> a, const Dual<N>& b) { return a /= b; }
template <int N>
__host__ __device__ inline Dual<N> operator+(Dual<N> a, double b) { a.v += b; return a; }
template <int N>
__host__ __device__ inline Dual<N> operator+(double b, Dual<N> a) { a.v += b; return a; }
template <int N>
__host__ __device__ inline Dual<N> operator-(Dual<N> a, double b) { a.v -= b; return a; }
template <int N>
__host__ __device__ inline Dual<N> operator-(double b, const Dual<N>& a) { return Dual<N>(b) - a; }
template <int N>
__host__ __device__ inline Dual<N> operator*(Dual<N> a, double b) {
  a.v *= b;
#pragma unroll
  for (int i = 0; i < N; ++i) a.d[i] *= b;
  return a;
}
template <int N>
__host__ __device__ inline Dual<N> operator*(double b, Dual<N> a) { return a * b; }
template <int N>
__host__ __device__ inline Dual<N> operator/(Dual<N> a, double b) { return a * (1.0 / b); }
template <int N>
__host__ __device__ inline Dual<N> operator/(double b, const Dual<N>& a) { return Dual<N>(b) / a; }

template <int N> __host__ __device__ inline bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> __host__ __device__ inline bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> __host__ __device__ inline bool operator<=(const Dual<N>& a, const Dual<N>& b) { return a.v <= b.v; }
template <int N> __host__ __device__ inline bool operator>=(const Dual<N>& a, const Dual<N>& b) { return a.v >= b.v; }
template <int N> __host__ __device__ inline bool operator!=(const Dual<N>& a, const Dual<N>& b) { return a.v != b.v; }
template <int N> __host__ __device__ inline bool operator==(const Dual<N>& a, const Dual<N>& b) { return a.v == b.v; }

template <int N>
__device__ inline Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = ::sqrt(a.v);
  const double h = r.v > 0.0 ? 0.5 / r.v : 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * h;
  return r;
}
template <int N>
__device__ inline Dual<N> fabs(const Dual<N>& a) { return a.v < 0.0 ? -a : a; }
template <int N>
__device__ inline Dual<N> fmax(const Dual<N>& a, const Dual<N>& b) { return a.v >= b.v ? a : b; }
template <int N>
__device__ inline Dual<N> fmin(const Dual<N>& a, const Dual<N>& b) { return a.v <= b.v ? a : b; }
// a^e for a > 0
template <int N>
__device__ inline Dual<N> pow(const Dual<N>& a, const Dual<N>& e) {
  Dual<N> r;
  r.v = ::pow(a.v, e.v);
  const double la = ::log(a.v);
  const double da = e.v * ::pow(a.v, e.v - 1.0);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = da * a.d[i] + r.v * la * e.d[i];
  return r;
}

}  // namespace rkdg

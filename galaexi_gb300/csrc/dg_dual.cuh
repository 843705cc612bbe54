// Forward-mode dual numbers for the tangent-linear operator and the local Jacobians of the adjoint.
//
// Dual<K> carries a value and K directional derivatives.  Instantiating the pointwise physics
// (dg_physics.cuh) and the forward kernels with R = Dual<1> gives the exact tangent-linear model of
// the FP64 operator (same branches, same operation order for the values); Dual<K> with K > 1 gives
// the K-column Jacobian of a pointwise function in one evaluation.  The default constructor is
// trivial so that Dual arrays may live in shared memory.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace gx {

// the Dual overloads below would hide the global math functions inside namespace gx
using ::sqrt;
using ::fabs;
using ::fmax;
using ::fmin;

template <int K>
struct Dual {
  double v;
  double d[K];
  Dual() = default;
  __host__ __device__ __forceinline__ Dual(double x) : v(x) {
#pragma unroll
    for (int k = 0; k < K; ++k) d[k] = 0.;
  }
  __host__ __device__ __forceinline__ explicit operator double() const { return v; }
  __host__ __device__ __forceinline__ Dual& operator+=(const Dual& b) {
    v += b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) d[k] += b.d[k];
    return *this;
  }
  __host__ __device__ __forceinline__ Dual& operator-=(const Dual& b) {
    v -= b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) d[k] -= b.d[k];
    return *this;
  }
  __host__ __device__ __forceinline__ Dual& operator*=(const Dual& b) {
#pragma unroll
    for (int k = 0; k < K; ++k) d[k] = d[k] * b.v + v * b.d[k];
    v *= b.v;
    return *this;
  }
};

template <int K>
__host__ __device__ __forceinline__ Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int K>
__host__ __device__ __forceinline__ Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int K>
__host__ __device__ __forceinline__ Dual<K> operator-(const Dual<K>& a) {
  Dual<K> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int K>
__host__ __device__ __forceinline__ Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int K>
__host__ __device__ __forceinline__ Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r;
  r.v = a.v / b.v;  // the value rounds as the primal division does
  const double s = 1. / b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * s;
  return r;
}
// mixed operands (double promoted to a constant)
template <int K> __host__ __device__ __forceinline__ Dual<K> operator+(const Dual<K>& a, double b) { return a + Dual<K>(b); }
template <int K> __host__ __device__ __forceinline__ Dual<K> operator+(double a, const Dual<K>& b) { return Dual<K>(a) + b; }
template <int K> __host__ __device__ __forceinline__ Dual<K> operator-(const Dual<K>& a, double b) { return a - Dual<K>(b); }
template <int K> __host__ __device__ __forceinline__ Dual<K> operator-(double a, const Dual<K>& b) { return Dual<K>(a) - b; }
template <int K> __host__ __device__ __forceinline__ Dual<K> operator*(const Dual<K>& a, double b) {
  Dual<K> r;
  r.v = a.v * b;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b;
  return r;
}
template <int K> __host__ __device__ __forceinline__ Dual<K> operator*(double a, const Dual<K>& b) { return b * a; }
template <int K> __host__ __device__ __forceinline__ Dual<K> operator/(const Dual<K>& a, double b) { return a / Dual<K>(b); }
template <int K> __host__ __device__ __forceinline__ Dual<K> operator/(double a, const Dual<K>& b) { return Dual<K>(a) / b; }

// comparisons act on the values (the branch taken is the primal one)
template <int K> __host__ __device__ __forceinline__ bool operator<(const Dual<K>& a, const Dual<K>& b) { return a.v < b.v; }
template <int K> __host__ __device__ __forceinline__ bool operator>(const Dual<K>& a, const Dual<K>& b) { return a.v > b.v; }
template <int K> __host__ __device__ __forceinline__ bool operator<=(const Dual<K>& a, const Dual<K>& b) { return a.v <= b.v; }
template <int K> __host__ __device__ __forceinline__ bool operator>=(const Dual<K>& a, const Dual<K>& b) { return a.v >= b.v; }

template <int K>
__device__ __forceinline__ Dual<K> sqrt(const Dual<K>& a) {
  Dual<K> r;
  r.v = ::sqrt(a.v);
  const double h = 0.5 / r.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * h;
  return r;
}
template <int K>
__device__ __forceinline__ Dual<K> fabs(const Dual<K>& a) {
  return a.v < 0. ? -a : a;
}
// fmax/fmin pick one operand (ties go to the first, as in the value path)
template <int K>
__device__ __forceinline__ Dual<K> fmax(const Dual<K>& a, const Dual<K>& b) {
  return (b.v > a.v) ? b : a;
}
template <int K>
__device__ __forceinline__ Dual<K> fmin(const Dual<K>& a, const Dual<K>& b) {
  return (b.v < a.v) ? b : a;
}

template <typename T> struct IsDual { static constexpr bool v = false; };
template <int K> struct IsDual<Dual<K>> { static constexpr bool v = true; };

}  // namespace gx

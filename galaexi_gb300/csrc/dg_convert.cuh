// FP64 <-> FP32 conversions of the mixed form on the integer pipes.
//
// On this GPU the conversion instructions between FP64 and FP32 issue on the FP64 unit (2 per clock
// per SM), which made them most of the FP64 work of the mixed form's ConsToPrim.  These functions
// rebuild the IEEE-754 fields with integer operations and give the same bits as the conversion
// instructions (round to nearest, ties to even), zeros included.  Subnormal, out-of-range, infinite
// and NaN inputs call the conversion instruction in a function of its own: a call is not turned into
// a predicated instruction, so warps without such an input issue no conversion at all.
//
// Host-callable as well (the word access then goes through memcpy), so that the same source is
// checked against the host's IEEE conversions by the CPU tests.
#pragma once
#include <cuda_runtime.h>
#include <string.h>

#ifdef __CUDACC__
#define GX_NOINLINE __noinline__
#else
#define GX_NOINLINE __attribute__((noinline))
#endif

namespace gx {

__host__ __device__ __forceinline__ unsigned cv_hi(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2hiint(x);
#else
  unsigned long long b;
  memcpy(&b, &x, 8);
  return (unsigned)(b >> 32);
#endif
}
__host__ __device__ __forceinline__ unsigned cv_lo(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2loint(x);
#else
  unsigned long long b;
  memcpy(&b, &x, 8);
  return (unsigned)b;
#endif
}
__host__ __device__ __forceinline__ double cv_double(unsigned hi, unsigned lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const unsigned long long b = ((unsigned long long)hi << 32) | lo;
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
__host__ __device__ __forceinline__ float cv_float(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}
__host__ __device__ __forceinline__ unsigned cv_bits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  unsigned u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

static __host__ __device__ GX_NOINLINE float f64_to_f32_rare(double x) { return (float)x; }
static __host__ __device__ GX_NOINLINE double f32_to_f64_rare(float f) { return (double)f; }

__host__ __device__ __forceinline__ float f64_to_f32_rn(double x) {
  const unsigned hi = cv_hi(x), lo = cv_lo(x);
  const unsigned ahi = hi & 0x7fffffffu;
  const bool zero = (ahi | lo) == 0u;
  const int e = (int)(ahi >> 20) - (1023 - 127);
  if (!zero && (e < 1 || e > 254)) return f64_to_f32_rare(x);
  // 23 mantissa bits kept: the 20 of the high word and the top 3 of the low word; 29 bits rounded off
  unsigned r = ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rest = lo & 0x1fffffffu;
  r += (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) ? 1u : 0u;  // a carry into e is exact
  return cv_float((zero ? 0u : r) | (hi & 0x80000000u));
}
__host__ __device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = cv_bits(f);
  const unsigned au = u & 0x7fffffffu;
  const bool zero = au == 0u;
  const unsigned e = au >> 23;
  if (!zero && (e == 0u || e == 255u)) return f32_to_f64_rare(f);
  const unsigned hi = (u & 0x80000000u) | (zero ? 0u : (((e + (1023u - 127u)) << 20) | ((au & 0x7fffffu) >> 3)));
  return cv_double(hi, u << 29);
}

}  // namespace gx

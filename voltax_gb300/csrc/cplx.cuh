// Complex FP64 scalar for the AC small-signal factorization and solves
// (A = G + j w C). Interleaved (re, im) in memory, like std::complex<double>.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace vxg {

struct cplx {
  double re, im;
  __host__ __device__ cplx() : re(0.0), im(0.0) {}
  __host__ __device__ cplx(double r) : re(r), im(0.0) {}  // NOLINT: real -> complex
  __host__ __device__ cplx(double r, double i) : re(r), im(i) {}
};

__host__ __device__ __forceinline__ cplx operator+(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ cplx operator-(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ __forceinline__ cplx operator-(cplx a) { return {-a.re, -a.im}; }
__host__ __device__ __forceinline__ cplx operator*(cplx a, cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
// Smith's algorithm (no overflow for large |b|)
__host__ __device__ __forceinline__ cplx operator/(cplx a, cplx b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, den = b.re + b.im * r;
    return {(a.re + a.im * r) / den, (a.im - a.re * r) / den};
  }
  const double r = b.re / b.im, den = b.re * r + b.im;
  return {(a.re * r + a.im) / den, (a.im * r - a.re) / den};
}
__host__ __device__ __forceinline__ cplx& operator+=(cplx& a, cplx b) { return a = a + b; }
__host__ __device__ __forceinline__ cplx& operator-=(cplx& a, cplx b) { return a = a - b; }
__host__ __device__ __forceinline__ bool operator==(cplx a, cplx b) {
  return a.re == b.re && a.im == b.im;
}

// Pivot magnitude: |x| for reals, |re| + |im| for complex (the measure of
// LAPACK's complex pivot search).
__device__ __forceinline__ float pmag(float x) { return fabsf(x); }
__device__ __forceinline__ double pmag(double x) { return fabs(x); }
__device__ __forceinline__ double pmag(cplx x) { return fabs(x.re) + fabs(x.im); }

__device__ __forceinline__ cplx shfl_xor(cplx v, int off) {
  return {__shfl_xor_sync(0xffffffffu, v.re, off), __shfl_xor_sync(0xffffffffu, v.im, off)};
}
__device__ __forceinline__ float shfl_xor(float v, int off) {
  return __shfl_xor_sync(0xffffffffu, v, off);
}
__device__ __forceinline__ double shfl_xor(double v, int off) {
  return __shfl_xor_sync(0xffffffffu, v, off);
}

}  // namespace vxg

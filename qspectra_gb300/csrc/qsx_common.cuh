// Shared device helpers for the qsx kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/qsx.h"

namespace qsx {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);

#define QSX_CHECK_ARG(cond, ...)                 \
  do {                                           \
    if (!(cond)) {                               \
      ::qsx::set_error(__VA_ARGS__);             \
      return QSX_ERR_INVALID_ARG;                \
    }                                            \
  } while (0)

#define QSX_LAUNCH_CHECK(where)                                       \
  do {                                                                \
    cudaError_t _e = cudaGetLastError();                              \
    if (_e != cudaSuccess) return ::qsx::cuda_status(_e, where);      \
  } while (0)

// ------------------------------------------------------ complex arithmetic
// complex128 is double2 {re, im} and complex64 is float2, the interleaved
// layouts of torch.complex128 / torch.complex64.
template <typename T> struct cplx;
template <> struct cplx<double> { using type = double2; };
template <> struct cplx<float> { using type = float2; };

__host__ __device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ float2 cmk(float r, float i) { return make_float2(r, i); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return cmk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return cmk(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return cmk(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  // Smith's algorithm keeps the scale of |b| out of the intermediate products.
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return cmk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    double r = b.x / b.y, d = b.y + b.x * r;
    return cmk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}
__host__ __device__ __forceinline__ double2 crecip(double2 b) { return cdiv(cmk(1.0, 0.0), b); }
// single-precision counterparts
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return cmk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return cmk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return cmk(a.x, -a.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return cmk(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 cdiv(float2 a, float2 b) {
  if (fabsf(b.x) >= fabsf(b.y)) {
    float r = b.y / b.x, d = b.x + b.y * r;
    return cmk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    float r = b.x / b.y, d = b.y + b.x * r;
    return cmk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}
__host__ __device__ __forceinline__ float2 crecip(float2 b) { return cdiv(cmk(1.0f, 0.0f), b); }

// acc += a * b  (complex multiply-accumulate, 4 FMAs)
__device__ __forceinline__ void cfma(double2& acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}

// Knuth's error-free sum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bp = s - a;
  float ap = s - bp;
  e = (a - ap) + (b - bp);
}

// (hi, lo) += z as a split-word (double-float) accumulator.
__device__ __forceinline__ void dd_add(float& hi, float& lo, float z) {
  float s, e;
  two_sum(hi, z, s, e);
  e += lo;
  hi = s + e;
  lo = e - (hi - s);
}

__host__ __device__ __forceinline__ float2 cadd2(float2 a, float2 b) { return cmk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 cadd2(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }

__device__ __forceinline__ bool finite2(double2 a) { return isfinite(a.x) && isfinite(a.y); }

// Whether a select table can drive the blocked loops: every entry in
// [0, m) and no entry twice (a repeated entry would leave an output slot
// unfilled, an entry outside [0, m) would index past the state).  Every
// thread of the CTA must call it (it ends in a barrier); the result is the
// same in all threads, and a bad table sets QSX_ERR_INVALID_ARG in *status.
__device__ __forceinline__ bool select_table_valid(const int* __restrict__ sel, int nsel, int m,
                                                   int* status) {
  int bad = 0;
  for (int q = threadIdx.x; q < nsel; q += blockDim.x) {
    const int v = sel[q];
    if (v < 0 || v >= m) {
      bad = 1;
    } else {
      for (int j = 0; j < q; ++j)
        if (sel[j] == v) {
          bad = 1;
          break;
        }
    }
  }
  bad = __syncthreads_or(bad);
  if (bad && threadIdx.x == 0 && status) atomicOr(status, QSX_ERR_INVALID_ARG);
  return !bad;
}

}  // namespace qsx

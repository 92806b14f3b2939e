// CUDA-core FMA throughput probe for the benchmark's roofline denominators.
// Not part of libqsx.so: it is built into its own small library,
// libqsx_probe.so, which only bench.py loads.  Each thread runs `iters`
// iterations of 16 x 8 independent FMA chains (FP32 or FP64) and writes one
// value to out[thread], so one launch performs
// blocks * threads * iters * 128 FMAs.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

// Eight independent FMA chains per thread so one warp can issue back to back.
template <typename T>
__global__ void probe_fma_kernel(int iters, T* out) {
  T a[8];
  const T m = T(0.999999), c = T(1e-7);
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = T(threadIdx.x + k) * T(1e-3);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int r = 0; r < 16; ++r) {
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = a[k] * m + c;
    }
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

// precision 1 = FP32, 0 = FP64.  Returns 0, 1 for a bad launch shape, or 2
// for a launch error.
extern "C" int qsx_probe_fma(int precision, int64_t blocks, int threads, int iters,
                             void* out, void* stream) {
  if (!(blocks > 0 && threads > 0 && threads <= 1024 && iters > 0 && out)) return 1;
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == 1)
    probe_fma_kernel<float><<<(unsigned)blocks, threads, 0, s>>>(iters, (float*)out);
  else
    probe_fma_kernel<double><<<(unsigned)blocks, threads, 0, s>>>(iters, (double*)out);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

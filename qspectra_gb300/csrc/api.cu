// Error plumbing, version and the FMA-throughput probe of the qsx C ABI.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "qsx_common.cuh"

namespace qsx {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char* where) {
  set_error("%s: CUDA error %d (%s)", where, (int)e, cudaGetErrorString(e));
  return QSX_ERR_CUDA;
}

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

}  // namespace qsx

extern "C" {

const char* qsx_last_error_string(void) { return qsx::g_err; }

int qsx_version(void) { return 100; }

// Each thread performs iters * 16 * 8 FMAs.
int qsx_probe_fma(int precision, int64_t blocks, int threads, int iters,
                  void* out, void* stream) {
  QSX_CHECK_ARG(blocks > 0 && threads > 0 && threads <= 1024 && iters > 0 && out,
                "qsx_probe_fma: bad launch shape");
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == QSX_FP32)
    qsx::probe_fma_kernel<float><<<(unsigned)blocks, threads, 0, s>>>(iters, (float*)out);
  else
    qsx::probe_fma_kernel<double><<<(unsigned)blocks, threads, 0, s>>>(iters, (double*)out);
  QSX_LAUNCH_CHECK("qsx_probe_fma");
  return QSX_OK;
}

}  // extern "C"

// Batched dense products for the third-order engine's many-right-hand-side
// steps: the f-manifold transform M_q = U Y_q U^T, the RK4 propagator
// polynomial and powers of the 'ee' block, their application to all t1
// states, and the signal contraction against the t3 states
// (qspectra/simulate/response.py:321-336: the t2 integrate over len(t1)
// vectors and einsum('ci,abi')).
//
// Complex products run as real products of the interleaved {re, im} views:
// a complex M x K matrix stored row-major is a real M x 2K matrix, and with
// every complex b = (br, bi) of the right operand expanded to the 2 x 2 real
// block [[br, bi], [-bi, br]] (a real b to [[b, 0], [0, b]]), the real
// product of the views is the interleaved complex product.  So one real GEMM
// kernel serves real x real, complex x complex, complex x real and
// real x complex (the last is a real product with the complex right operand
// read as a real matrix of twice the columns).
//
// FP32: 5th-generation tensor cores, 3xTF32 (hi/lo TF32 split of both
// operands, A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi, FP32 accumulation in
// tensor memory).  Each CTA owns a 128 x 128 tile of C, two CTAs per SM; the
// K loop moves in chunks of 16 through three buffers: while the tensor core
// multiplies the previous chunks, all threads split and store the chunk
// their registers hold (loaded from global memory two chunks ahead: 16-byte
// loads of A rows, 8-byte loads of complex B) in the K-major core-matrix
// layout of a free buffer.  One thread issues the
// MMAs and commits them to the buffer's mbarrier; every wait is bounded and a
// timeout sets QSX_ERR_CUDA in the status word.
// FP64: CUDA cores, 64 x 64 tiles of C, 4 x 4 per thread, the same views.
#include <stdint.h>

#include <algorithm>

#include "qsx_common.cuh"
#include "qsx_tc.cuh"

namespace qsx {

// right-operand expansion of the real view
enum { GB_REAL = 0, GB_CPLX = 1, GB_REAL_AS_CPLX = 2 };

struct GemmP {
  int M, N, K;          // real-view sizes: C M x N, A M x K, B' K x N
  int bmode;
  const void* A;
  int64_t lda, sA;      // in real elements
  const void* B;
  int64_t ldb, sB;      // in source elements: real (GB_REAL, GB_REAL_AS_CPLX) or complex
  const void* Cin;
  int64_t ldcin, sCin;
  void* C;
  int64_t ldc, sC;
  double alpha, beta;
  int avec;             // A rows 16-byte aligned (vector loads allowed)
  int* status;
};

// element (k, n) of the expanded right operand B'
template <typename T>
__device__ __forceinline__ T b_elem(const GemmP& p, const T* B, int k, int n) {
  if (k >= p.K || n >= p.N) return (T)0;
  if (p.bmode == GB_REAL) return B[(int64_t)k * p.ldb + n];
  const int kk = k >> 1, nn = n >> 1, t = k & 1, u = n & 1;
  if (p.bmode == GB_REAL_AS_CPLX) return t == u ? B[(int64_t)kk * p.ldb + nn] : (T)0;
  const T* z = B + 2 * ((int64_t)kk * p.ldb + nn);   // complex (re, im)
  if (t == 0) return u == 0 ? z[0] : z[1];
  return u == 0 ? -z[1] : z[0];
}

template <typename T>
__device__ __forceinline__ T a_elem(const GemmP& p, const T* A, int m, int k) {
  return (m < p.M && k < p.K) ? A[(int64_t)m * p.lda + k] : (T)0;
}

// ------------------------------------------------------------ FP32, tcgen05
constexpr int GT_BM = 128, GT_BN = 128, GT_BK = 16, GT_THREADS = 256, GT_STAGES = 3;
constexpr uint32_t GT_PLANE = GT_BM * GT_BK * 4;             // 8 KB
constexpr uint32_t GT_SBO = GT_BK * 32;                       // 512 B
constexpr uint32_t GT_BUF = 4 * GT_PLANE;                     // A hi/lo, B hi/lo
constexpr size_t GT_SMEM = GT_STAGES * (size_t)GT_BUF + 64;
constexpr uint32_t GT_TMEM_COLS = 128;

// Four consecutive k of row m of A (real view): one 16-byte load when the
// rows are 16-byte aligned and the quad lies inside the matrix.
__device__ __forceinline__ float4 a_quad(const GemmP& p, const float* A, int m, int k) {
  if (m < p.M && k + 3 < p.K && p.avec)
    return __ldg(reinterpret_cast<const float4*>(A + (int64_t)m * p.lda + k));
  return make_float4(a_elem(p, A, m, k), a_elem(p, A, m, k + 1), a_elem(p, A, m, k + 2),
                     a_elem(p, A, m, k + 3));
}

// Four consecutive k (k a multiple of 4) of column n of the expanded right
// operand B': for a complex source two 8-byte loads give the whole quad.
__device__ __forceinline__ float4 b_quad(const GemmP& p, const float* B, int k, int n) {
  if (p.bmode == GB_REAL || n >= p.N || k + 3 >= p.K)
    return make_float4(b_elem(p, B, k, n), b_elem(p, B, k + 1, n), b_elem(p, B, k + 2, n),
                       b_elem(p, B, k + 3, n));
  const int kk = k >> 1, nn = n >> 1, u = n & 1;
  if (p.bmode == GB_REAL_AS_CPLX) {
    const float z0 = __ldg(B + (int64_t)kk * p.ldb + nn);
    const float z1 = __ldg(B + (int64_t)(kk + 1) * p.ldb + nn);
    return u == 0 ? make_float4(z0, 0.f, z1, 0.f) : make_float4(0.f, z0, 0.f, z1);
  }
  const float2 z0 = __ldg(reinterpret_cast<const float2*>(B) + (int64_t)kk * p.ldb + nn);
  const float2 z1 = __ldg(reinterpret_cast<const float2*>(B) + (int64_t)(kk + 1) * p.ldb + nn);
  // rows 2kk, 2kk + 1 of the 2 x 2 blocks [[br, bi], [-bi, br]]
  return u == 0 ? make_float4(z0.x, -z0.y, z1.x, -z1.y) : make_float4(z0.y, z0.x, z1.y, z1.x);
}

__global__ void __launch_bounds__(GT_THREADS, 2) gemm_tc_kernel(GemmP p) {
  using namespace tc;
  extern __shared__ __align__(128) unsigned char smraw[];
  uint64_t* mbar_p = reinterpret_cast<uint64_t*>(smraw + GT_STAGES * GT_BUF);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar_p + GT_STAGES);
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * GT_BM, n0 = blockIdx.x * GT_BN;
  const int64_t bz = blockIdx.z;
  const float* A = (const float*)p.A + bz * p.sA;
  const float* B = (const float*)p.B + bz * p.sB * (p.bmode == GB_CPLX ? 2 : 1);
  if (tid == 0) {
    s_abort = 0;
    for (int i = 0; i < GT_STAGES; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
                       (uint32_t)__cvta_generic_to_shared(mbar_p + i))
                   : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(tmem_slot)),
                 "r"(GT_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = make_idesc(GT_BN);
  const int nk = (p.K + GT_BK - 1) / GT_BK;
  int issued = 0;   // chunks whose MMAs were issued (uniform across threads)
  // Each thread's quads of a chunk: two of A (a warp covers 8 rows x 16 k,
  // 64 contiguous bytes per row; its 16-byte stores fill 32 distinct bank
  // groups) and two of B'^T (rows n fastest, coalesced along the columns of
  // B).  The global loads run two chunks ahead of the split and store, in
  // registers, so their latency hides behind two iterations of work.
  constexpr int QA = (GT_BM / 8) / (GT_THREADS / 32), QB = (GT_BN * GT_BK / 4) / GT_THREADS;
  auto load_chunk = [&](int kc, float4 (&va)[QA], float4 (&vb)[QB]) {
    const int k0 = kc * GT_BK;
#pragma unroll
    for (int i = 0; i < QA; ++i) {
      const int r = 8 * (warp + (GT_THREADS / 32) * i) + (lane & 7), j = lane >> 3;
      va[i] = a_quad(p, A, m0 + r, k0 + 4 * j);
    }
#pragma unroll
    for (int i = 0; i < QB; ++i) {
      const int idx = tid + i * GT_THREADS;
      const int n = idx & (GT_BN - 1), j = idx >> 7;
      vb[i] = b_quad(p, B, k0 + 4 * j, n0 + n);
    }
  };
  float4 ca[QA], cb[QB], na[QA], nb[QB], fa[QA], fb[QB];
  if (nk > 0) load_chunk(0, ca, cb);
  if (nk > 1) load_chunk(1, na, nb);
  for (int kc = 0; kc < nk; ++kc) {
    if (kc + 2 < nk) load_chunk(kc + 2, fa, fb);
    const int buf = kc % GT_STAGES;
    unsigned char* base = smraw + buf * GT_BUF;
    unsigned char* a_hi = base;
    unsigned char* a_lo = base + GT_PLANE;
    unsigned char* b_hi = base + 2 * GT_PLANE;
    unsigned char* b_lo = base + 3 * GT_PLANE;
    if (kc >= GT_STAGES) {   // the MMAs of chunk kc - GT_STAGES read this buffer
      if (tid == 0) {
        const uint32_t mb = (uint32_t)__cvta_generic_to_shared(mbar_p + buf);
        if (!wait_parity(mb, (uint32_t)(((kc - GT_STAGES) / GT_STAGES) & 1))) {
          if (p.status) atomicOr(p.status, QSX_ERR_CUDA);
          s_abort = 1;
        }
      }
      __syncthreads();
      if (s_abort) break;
    }
#pragma unroll
    for (int i = 0; i < QA; ++i) {
      const int r = 8 * (warp + (GT_THREADS / 32) * i) + (lane & 7), j = lane >> 3;
      st_split4(a_hi, a_lo, op_offset(r, 4 * j, GT_SBO), ca[i].x, ca[i].y, ca[i].z, ca[i].w);
    }
#pragma unroll
    for (int i = 0; i < QB; ++i) {
      const int idx = tid + i * GT_THREADS;
      const int n = idx & (GT_BN - 1), j = idx >> 7;
      st_split4(b_hi, b_lo, op_offset(n, 4 * j, GT_SBO), cb[i].x, cb[i].y, cb[i].z, cb[i].w);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      const uint64_t dah = smem_desc((uint32_t)__cvta_generic_to_shared(a_hi), GT_SBO);
      const uint64_t dal = smem_desc((uint32_t)__cvta_generic_to_shared(a_lo), GT_SBO);
      const uint64_t dbh = smem_desc((uint32_t)__cvta_generic_to_shared(b_hi), GT_SBO);
      const uint64_t dbl = smem_desc((uint32_t)__cvta_generic_to_shared(b_lo), GT_SBO);
      issue_product(tmem, dah, dal, dbh, dbl, GT_BK / 8, idesc,
                    (uint32_t)__cvta_generic_to_shared(mbar_p + buf), kc > 0 ? 1u : 0u);
    }
    issued = kc + 1;
#pragma unroll
    for (int i = 0; i < QA; ++i) ca[i] = na[i], na[i] = fa[i];
#pragma unroll
    for (int i = 0; i < QB; ++i) cb[i] = nb[i], nb[i] = fb[i];
  }
  // the last commit covers every MMA issued before it
  if (tid == 0 && !s_abort && issued > 0) {
    const int last = issued - 1;
    const uint32_t mb = (uint32_t)__cvta_generic_to_shared(mbar_p + (last % GT_STAGES));
    if (!wait_parity(mb, (uint32_t)((last / GT_STAGES) & 1))) {
      if (p.status) atomicOr(p.status, QSX_ERR_CUDA);
      s_abort = 1;
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!s_abort) {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows) and
    // columns 64 (w / 4) .. + 63
    const int q = warp & 3, half = warp >> 2;
    const int m = m0 + 32 * q + lane;
    const float al = (float)p.alpha, be = (float)p.beta;
    float* C = (float*)p.C + bz * p.sC + (int64_t)m * p.ldc;
    const float* Ci = p.Cin ? (const float*)p.Cin + bz * p.sCin + (int64_t)m * p.ldcin : nullptr;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      float v[32];
      const int c0 = 64 * half + 32 * g;
      tmem_load(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0, v);
      if (m < p.M) {
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          const int n = n0 + c0 + c;
          if (n < p.N) C[n] = al * v[c] + (Ci ? be * Ci[n] : 0.f);
        }
      }
    }
  } else if (tid == 0 && issued > 0) {
    // let an unfinished chain drain (bounded) before the memory is freed
    const int last = issued - 1;
    wait_parity((uint32_t)__cvta_generic_to_shared(mbar_p + (last % GT_STAGES)),
                (uint32_t)((last / GT_STAGES) & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(GT_TMEM_COLS)
                 : "memory");
}

// ------------------------------------------------------------ FP64, CUDA cores
constexpr int GD_BM = 64, GD_BN = 64, GD_BK = 16;

__global__ void __launch_bounds__(256) gemm_f64_kernel(GemmP p) {
  __shared__ double sA[GD_BK][GD_BM + 1];
  __shared__ double sB[GD_BK][GD_BN + 1];
  const int tid = threadIdx.x;
  const int tr = tid / 16, tc = tid % 16;   // 4 x 4 outputs per thread
  const int m0 = blockIdx.y * GD_BM, n0 = blockIdx.x * GD_BN;
  const int64_t bz = blockIdx.z;
  const double* A = (const double*)p.A + bz * p.sA;
  const double* B = (const double*)p.B + bz * p.sB * (p.bmode == GB_CPLX ? 2 : 1);
  double acc[4][4] = {};
  for (int k0 = 0; k0 < p.K; k0 += GD_BK) {
    for (int e = tid; e < GD_BK * GD_BM; e += 256) {
      const int r = e / GD_BK, k = e % GD_BK;
      sA[k][r] = a_elem(p, A, m0 + r, k0 + k);
    }
    for (int e = tid; e < GD_BK * GD_BN; e += 256) {
      const int k = e / GD_BN, n = e % GD_BN;
      sB[k][n] = b_elem(p, B, k0 + k, n0 + n);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < GD_BK; ++k) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[k][tr + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[k][tc + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  double* C = (double*)p.C + bz * p.sC;
  const double* Ci = p.Cin ? (const double*)p.Cin + bz * p.sCin : nullptr;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + tr + 16 * i;
    if (m >= p.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tc + 16 * j;
      if (n < p.N)
        C[(int64_t)m * p.ldc + n] =
            p.alpha * acc[i][j] + (Ci ? p.beta * Ci[(int64_t)m * p.ldcin + n] : 0.0);
    }
  }
}

}  // namespace qsx

using namespace qsx;

extern "C" int qsx_gemm_batched(int precision, int mode, int64_t batch, int M, int N, int K,
                                const void* A, int64_t lda, int64_t strideA, const void* B,
                                int64_t ldb, int64_t strideB, const void* Cin, int64_t ldcin,
                                int64_t strideCin, double beta, void* C, int64_t ldc,
                                int64_t strideC, double alpha, int32_t* status, void* stream) {
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64, "qsx_gemm_batched: bad precision");
  QSX_CHECK_ARG(mode >= 0 && mode <= 3, "qsx_gemm_batched: mode must be 0..3");
  QSX_CHECK_ARG(batch >= 0 && batch <= 65535 && M >= 0 && N >= 0 && K >= 0,
                "qsx_gemm_batched: bad sizes (batch <= 65535)");
  if (batch == 0 || M == 0 || N == 0) return QSX_OK;
  QSX_CHECK_ARG(A && B && C, "qsx_gemm_batched: null operand");
  QSX_CHECK_ARG(K >= 1, "qsx_gemm_batched: K must be at least 1");
  QSX_CHECK_ARG(C != A && C != B, "qsx_gemm_batched: C must not alias A or B");
  QSX_CHECK_ARG(Cin == nullptr || Cin != C || (ldcin == ldc && strideCin == strideC),
                "qsx_gemm_batched: Cin may alias C only element for element");
  // real views: complex sizes and leading dimensions double
  GemmP p;
  const bool ca = mode == 1 || mode == 2;   // complex A (and C)
  const bool cb = mode == 1 || mode == 3;   // complex B
  const bool cc = mode != 0;                // complex C
  p.M = M;
  p.K = ca ? 2 * K : K;
  p.N = cc ? 2 * N : N;
  p.bmode = mode == 1 ? GB_CPLX : (mode == 2 ? GB_REAL_AS_CPLX : GB_REAL);
  p.A = A;
  p.lda = ca ? 2 * lda : lda;
  p.sA = ca ? 2 * strideA : strideA;
  p.B = B;
  // mode 3: the complex right operand is read as a real K x 2N matrix
  p.ldb = mode == 3 ? 2 * ldb : ldb;
  p.sB = mode == 3 ? 2 * strideB : strideB;
  p.Cin = Cin;
  p.ldcin = cc ? 2 * ldcin : ldcin;
  p.sCin = cc ? 2 * strideCin : strideCin;
  p.C = C;
  p.ldc = cc ? 2 * ldc : ldc;
  p.sC = cc ? 2 * strideC : strideC;
  p.alpha = alpha;
  p.beta = beta;
  p.status = status;
  p.avec = precision == QSX_FP32 && (reinterpret_cast<uintptr_t>(A) & 15) == 0 &&
           p.lda % 4 == 0 && p.sA % 4 == 0;
  (void)cb;
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == QSX_FP32) {
    cudaError_t e = cudaFuncSetAttribute(gemm_tc_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)GT_SMEM);
    if (e != cudaSuccess) return cuda_status(e, "qsx_gemm_batched");
    dim3 grid((unsigned)((p.N + GT_BN - 1) / GT_BN), (unsigned)((p.M + GT_BM - 1) / GT_BM),
              (unsigned)batch);
    gemm_tc_kernel<<<grid, GT_THREADS, GT_SMEM, s>>>(p);
  } else {
    dim3 grid((unsigned)((p.N + GD_BN - 1) / GD_BN), (unsigned)((p.M + GD_BM - 1) / GD_BM),
              (unsigned)batch);
    gemm_f64_kernel<<<grid, 256, 0, s>>>(p);
  }
  QSX_LAUNCH_CHECK("qsx_gemm_batched");
  return QSX_OK;
}

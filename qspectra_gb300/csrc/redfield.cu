// Redfield Liouvillian construction on the GPU (FP64): bath correlation
// function, batched Jacobi eigensolver, operator-form Redfield tensor, dense
// Liouvillian blocks and the RK4 one-step propagator.
#include <algorithm>
#include <cmath>

#include "qsx_bath.cuh"
#include <type_traits>

#include "qsx_common.cuh"

namespace qsx {

// ------------------------------------------------------------------ C(x)
__global__ void debye_corr_kernel(const double* x, int64_t n, DebyeParams p,
                                  double2* out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = debye_corr(p, x[i]);
}

// ------------------------------------------------------------ eigensolver
// One warp per matrix, matrix and eigenvectors in shared memory.  Cyclic
// Jacobi sweeps (Golub & Van Loan, Alg. 8.4.3): for each pair (p, q) every
// lane updates one row/column.  Block-diagonal inputs stay exactly block
// diagonal because rotations of an exactly zero pair are skipped.
constexpr int EIGH_NMAX = 32;
constexpr int EIGH_WARPS = 4;

struct BlockTable {
  int v[EIGH_NMAX + 1];
};

// Classical Jacobi rotation zeroing a_pq (Golub & Van Loan, Alg. 8.4.1):
// returns c = cos, s = sin and t = tan of the angle.
__device__ __forceinline__ void jacobi_rotation(double app, double aqq, double apq,
                                                double& c, double& s, double& t) {
  const double tau = (aqq - app) / (2.0 * apq);
  t = fabs(tau) < 1e100
          ? (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(fma(tau, tau, 1.0)))
          : 0.5 / tau;
  c = rsqrt(fma(t, t, 1.0));
  s = t * c;
}
__device__ __forceinline__ void jacobi_rotation(double app, double aqq, double apq,
                                                double& c, double& s) {
  double t;
  jacobi_rotation(app, aqq, apq, c, s, t);
}
__device__ __forceinline__ void jacobi_rotation(float app, float aqq, float apq, float& c,
                                                float& s, float& t) {
  const float tau = (aqq - app) / (2.0f * apq);
  t = fabsf(tau) < 1e18f ? (tau >= 0.0f ? 1.0f : -1.0f) / (fabsf(tau) + sqrtf(fmaf(tau, tau, 1.0f)))
                         : 0.5f / tau;
  c = rsqrtf(fmaf(t, t, 1.0f));
  s = t * c;
}

// One thread per matrix for a diagonal block of size NB <= 8 starting at
// row/column `off` of each n x n input: the upper triangle of the block and
// its eigenvectors live in registers (fully unrolled sweeps, compile-time
// indices).  Symmetric update: a_pp -= t a_pq, a_qq += t a_pq, and for
// k != p, q the pair (a_kp, a_kq) rotates by (c, s).
// T = float runs the same sweeps in FP32 (for builds feeding FP32
// propagation; stops at off-diagonal mass below 1e-13 of the diagonal).
template <typename T, int NB>
__global__ void __launch_bounds__(64)
    eigh_block_kernel(const double* __restrict__ H, int n, int off, int64_t batch,
                      double* E, double* U) {
#define AS(i, j) A[(i) < (j) ? (i) : (j)][(i) < (j) ? (j) : (i)]
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  T A[NB][NB], V[NB][NB];
  const double* h = H + b * n * n;
  const T tol = sizeof(T) == 4 ? (T)1e-13 : (T)1e-32;
#pragma unroll
  for (int i = 0; i < NB; ++i)
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      if (j >= i) A[i][j] = (T)h[(off + i) * n + off + j];
      V[i][j] = i == j ? (T)1 : (T)0;
    }
  for (int sweep = 0; sweep < 30; ++sweep) {
    T offd = (T)0, dia = (T)0;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      dia = fma(A[i][i], A[i][i], dia);
#pragma unroll
      for (int j = i + 1; j < NB; ++j) offd = fma(A[i][j], A[i][j], offd);
    }
    if (!(offd > tol * dia)) break;
#pragma unroll
    for (int p = 0; p < NB - 1; ++p) {
#pragma unroll
      for (int q = p + 1; q < NB; ++q) {
        const T apq = A[p][q];
        if (apq != (T)0) {
          T c, s, t;
          jacobi_rotation(A[p][p], A[q][q], apq, c, s, t);
          A[p][p] = fma(-t, apq, A[p][p]);
          A[q][q] = fma(t, apq, A[q][q]);
          A[p][q] = (T)0;
#pragma unroll
          for (int k = 0; k < NB; ++k) {
            if (k == p || k == q) continue;
            const T g = AS(k, p), hh = AS(k, q);
            AS(k, p) = c * g - s * hh;
            AS(k, q) = s * g + c * hh;
          }
#pragma unroll
          for (int k = 0; k < NB; ++k) {  // V <- V J
            const T vkp = V[k][p], vkq = V[k][q];
            V[k][p] = c * vkp - s * vkq;
            V[k][q] = s * vkp + c * vkq;
          }
        }
      }
    }
  }
  // ascending order inside the block (stable on ties)
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    int rank = 0;
#pragma unroll
    for (int j = 0; j < NB; ++j)
      rank += (A[j][j] < A[i][i] || (A[j][j] == A[i][i] && j < i)) ? 1 : 0;
    E[b * n + off + rank] = (double)A[i][i];
#pragma unroll
    for (int r = 0; r < NB; ++r) U[b * n * n + (off + r) * n + off + rank] = (double)V[r][i];
  }
#undef AS
}

// zero the off-block entries of U (the block kernels write only their blocks)
__global__ void zero_kernel(double* p, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.0;
}

__global__ void __launch_bounds__(32 * EIGH_WARPS)
    eigh_jacobi_kernel(const double* __restrict__ H, int n, int64_t batch,
                       int nblocks, BlockTable blocks, double* E, double* U) {
  __shared__ double sA[EIGH_WARPS][EIGH_NMAX][EIGH_NMAX + 1];
  __shared__ double sV[EIGH_WARPS][EIGH_NMAX][EIGH_NMAX + 1];
  __shared__ int sBlk[EIGH_NMAX + 1];
  const int w = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int64_t b = (int64_t)blockIdx.x * EIGH_WARPS + w;
  if (threadIdx.x <= nblocks && threadIdx.x <= EIGH_NMAX) sBlk[threadIdx.x] = blocks.v[threadIdx.x];
  __syncthreads();
  if (b >= batch) return;
  double(*A)[EIGH_NMAX + 1] = sA[w];
  double(*V)[EIGH_NMAX + 1] = sV[w];
  const double* h = H + b * n * n;
  for (int r = 0; r < n; ++r) {
    if (lane < n) {
      A[r][lane] = h[r * n + lane];
      V[r][lane] = (r == lane) ? 1.0 : 0.0;
    }
  }
  __syncwarp();
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, dia = 0.0;
    if (lane < n) {
      for (int c = 0; c < n; ++c) {
        double v = A[lane][c];
        if (c == lane) dia += v * v; else off += v * v;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dia += __shfl_xor_sync(0xffffffffu, dia, o);
    }
    if (!(off > 1e-30 * dia) || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p) {
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p][q];
        if (apq == 0.0) continue;
        // one lane evaluates the rotation (FP64 divide/sqrt are scarce here)
        double c = 1.0, s = 0.0;
        if (lane == 0) jacobi_rotation(A[p][p], A[q][q], apq, c, s);
        c = __shfl_sync(0xffffffffu, c, 0);
        s = __shfl_sync(0xffffffffu, s, 0);
        __syncwarp();
        if (lane < n) {  // A <- A J and V <- V J on row `lane`
          double akp = A[lane][p], akq = A[lane][q];
          A[lane][p] = c * akp - s * akq;
          A[lane][q] = s * akp + c * akq;
          double vkp = V[lane][p], vkq = V[lane][q];
          V[lane][p] = c * vkp - s * vkq;
          V[lane][q] = s * vkp + c * vkq;
        }
        __syncwarp();
        if (lane < n) {  // A <- J^T A on column `lane`
          double apk = A[p][lane], aqk = A[q][lane];
          A[p][lane] = c * apk - s * aqk;
          A[q][lane] = s * apk + c * aqk;
        }
        __syncwarp();
        if (lane == 0) {
          A[p][q] = 0.0;
          A[q][p] = 0.0;
        }
        __syncwarp();
      }
    }
  }
  // sort ascending inside each block (stable on ties)
  if (lane < n) {
    int blk = 0;
    while (blk < nblocks - 1 && lane >= sBlk[blk + 1]) ++blk;
    const int lo = sBlk[blk], hi = sBlk[blk + 1];
    const double ev = A[lane][lane];
    int rank = lo;
    for (int j = lo; j < hi; ++j) {
      double ej = A[j][j];
      if (ej < ev || (ej == ev && j < lane)) ++rank;
    }
    E[b * n + rank] = ev;
    for (int r = 0; r < n; ++r) U[b * n * n + r * n + rank] = V[r][lane];
  }
}

// ------------------------------------------------- Redfield operator form
// One CTA per sample.  Shared layout (n <= 32): U, Kt real; Cw, Mt, GS, T1
// complex.  See qsx_redfield_operators_batched in qsx.h for the algebra.
// T = double is the FP64 build; T = float evaluates the same formulas in FP32
// for generators that feed the FP32 split-word propagation (outputs are
// stored as complex128 either way).
template <typename T>
__device__ __forceinline__ void smem_matmul_rc(const T* A, const typename cplx<T>::type* B,
                                               typename cplx<T>::type* C, int n, bool accumulate) {
  // C = A (real) * B (complex)
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int r = e / n, c = e % n;
    typename cplx<T>::type acc = accumulate ? C[e] : cmk((T)0, (T)0);
    for (int k = 0; k < n; ++k) {
      const T a = A[r * n + k];
      const typename cplx<T>::type bb = B[k * n + c];
      acc.x = fma(a, bb.x, acc.x);
      acc.y = fma(a, bb.y, acc.y);
    }
    C[e] = acc;
  }
}

template <typename T>
__device__ __forceinline__ void smem_matmul_crT(const typename cplx<T>::type* A, const T* B,
                                                typename cplx<T>::type* C, int n) {
  // C = A (complex) * B^T (real)
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int r = e / n, c = e % n;
    typename cplx<T>::type acc = cmk((T)0, (T)0);
    for (int k = 0; k < n; ++k) {
      const T bb = B[c * n + k];
      const typename cplx<T>::type a = A[r * n + k];
      acc.x = fma(a.x, bb, acc.x);
      acc.y = fma(a.y, bb, acc.y);
    }
    C[e] = acc;
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
    redfield_operators_kernel(const double* __restrict__ E, const double* __restrict__ U,
                              int n, int64_t batch, const double* __restrict__ occ,
                              int n_sites, DebyeParams bath, double uc, int site_basis,
                              double2* G, double2* M, double* K) {
  using Cx = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nn = n * n;
  Cx* sC = (Cx*)smraw;               // nn   (complex arrays first)
  Cx* sMt = sC + nn;                 // nn
  Cx* sGS = sMt + nn;                // nn
  Cx* sT1 = sGS + nn;                // nn
  T* sU = (T*)(sT1 + nn);            // nn
  T* sUt = sU + nn;                  // nn, U^T
  T* sKt = sUt + nn;                 // nn
  T* sE = sKt + nn;                  // n (<= 32), then 32 coupling weights of eigenvectors
  T* sOcc = sE + 64;                 // [n_sites][n]
  // occupied states of each site (occ != 0), found once per CTA so the
  // element loops below issue no compares on the occupations
  int* sOccN = (int*)(sOcc + n_sites * n);  // [n_sites]
  int* sOccS = sOccN + 32;                   // [n_sites][n] state indices
  const int64_t b = blockIdx.x;
  const double* u = U + b * nn;
  for (int e = threadIdx.x; e < nn; e += blockDim.x) {
    int r = e / n, c = e % n;
    const T v = (T)u[e];
    sU[e] = v;
    sUt[c * n + r] = v;
    sGS[e] = cmk((T)0, (T)0);
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) sE[i] = (T)E[b * n + i];
  for (int e = threadIdx.x; e < n_sites * n; e += blockDim.x) sOcc[e] = (T)occ[e];
  for (int i = threadIdx.x; i < n_sites; i += blockDim.x) {
    int cnt = 0;
    for (int st = 0; st < n; ++st)
      if (occ[i * n + st] != 0.0) sOccS[i * n + cnt++] = st;
    sOccN[i] = cnt;
  }
  __syncthreads();
  // coupling weight of eigenvector c: sum_s U[s][c]^2 (sum_i occ_i(s)^2)
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    T wsum = (T)0;
    for (int i = 0; i < n_sites; ++i)
      for (int k = 0; k < sOccN[i]; ++k) {
        const int st = sOccS[i * n + k];
        const T o = sOcc[i * n + st], x = sU[st * n + c];
        wsum = fma(o * o, x * x, wsum);
      }
    sE[32 + c] = wsum;
  }
  __syncthreads();
  // correlation function only for pairs of bath-coupled eigenvectors (any
  // Kt_i[c][d] vanishes otherwise); the pair (c, d), (d, c) shares one
  // Matsubara evaluation (C(E_d - E_c) and C(E_c - E_d)), computed by the
  // thread with c <= d.
  for (int e = threadIdx.x; e < nn; e += blockDim.x) {
    int c = e / n, d = e % n;
    if (c > d) continue;
    if (sE[32 + c] > (T)0 && sE[32 + d] > (T)0) {
      Cx cp, cn;
      debye_corr_pair_t(bath, sE[d] - sE[c], cp, cn);
      sC[e] = cp;
      sC[d * n + c] = cn;
    } else {
      sC[e] = cmk((T)0, (T)0);
      sC[d * n + c] = cmk((T)0, (T)0);
    }
  }
  __syncthreads();
  const T uct = (T)uc;
  for (int i = 0; i < n_sites; ++i) {
    const T* oc = sOcc + i * n;
    const int cnt = sOccN[i];
    const int* ost = sOccS + i * n;
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      int c = e / n, d = e % n;
      T acc = (T)0;
      for (int k = 0; k < cnt; ++k) {
        const int st = ost[k];
        acc = fma(sU[st * n + c] * oc[st], sU[st * n + d], acc);
      }
      sKt[e] = acc;
      const Cx cw = sC[e];
      sMt[e] = cmk(acc * cw.x, acc * cw.y);
    }
    __syncthreads();
    double2* Mi = M + (b * n_sites + i) * nn;
    if (site_basis) {
      smem_matmul_rc<T>(sU, sMt, sT1, n, false);  // T1 = U Mt_i
      __syncthreads();
      smem_matmul_crT<T>(sT1, sU, sMt, n);        // Mt_i <- T1 U^T (site basis)
      __syncthreads();
      // G_site = sum_i diag(occ_i) M_i: row s of G gathers row s of every M_i
      for (int e = threadIdx.x; e < nn; e += blockDim.x)
        Mi[e] = make_double2((double)(sMt[e].x * uct), (double)(sMt[e].y * uct));
      for (int k = 0; k < cnt; ++k) {
        const int st = ost[k];
        const T o = oc[st];
        for (int c = threadIdx.x; c < n; c += blockDim.x)
          sGS[st * n + c] = cadd(sGS[st * n + c], cscale(sMt[st * n + c], o));
      }
    } else {
      smem_matmul_rc<T>(sKt, sMt, sGS, n, true);  // GS += Kt_i Mt_i (eigenbasis)
      __syncthreads();
      double* Ki = K + (b * n_sites + i) * nn;
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        Mi[e] = make_double2((double)(sMt[e].x * uct), (double)(sMt[e].y * uct));
        Ki[e] = (double)sKt[e];
      }
    }
    __syncthreads();
  }
  double2* g = G + b * nn;
  for (int e = threadIdx.x; e < nn; e += blockDim.x)
    g[e] = make_double2((double)(sGS[e].x * uct), (double)(sGS[e].y * uct));
}

// ----------------------------------------------- dense Liouvillian block
__global__ void liouvillian_kernel(const double* __restrict__ H, int64_t H_stride,
                                   const double2* __restrict__ G,
                                   const double2* __restrict__ M,
                                   const double* __restrict__ K, int64_t K_stride,
                                   const double* __restrict__ occ, int n, int n_sites,
                                   double uc, const int* __restrict__ idx, int m,
                                   int secular, int transpose, double2* L) {
  const int64_t b = blockIdx.y;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)m * m) return;
  int r = (int)(e / m), cc = (int)(e % m);
  if (transpose) { int t = r; r = cc; cc = t; }
  const int ir = idx[r], ic = idx[cc];
  const int nn = n * n;
  if (ir < 0 || ir >= nn || ic < 0 || ic >= nn) {  // bad index table: no access
    L[b * (int64_t)m * m + e] = cmk(nan(""), nan(""));
    return;
  }
  const int a = ir % n, bb = ir / n, c = ic % n, d = ic / n;
  const double* h = H + b * H_stride;
  const double2* g = G + b * nn;
  const double2* mm = M + b * (int64_t)n_sites * nn;
  // coherent part: -i uc (H_ac d_bd - d_ac H_db)
  double hre = 0.0;
  if (bb == d) hre += h[a * n + c];
  if (a == c) hre -= h[d * n + bb];
  double2 val = cmk(0.0, -uc * hre);
  double2 R = cmk(0.0, 0.0);
  if (bb == d) R = cadd(R, g[a * n + c]);
  if (a == c) R = cadd(R, cconj(g[bb * n + d]));
  if (K == nullptr) {
    // site basis, K_i = diag(occ_i)
    if (a == c) {
      for (int i = 0; i < n_sites; ++i) {
        double o = occ[i * n + a];
        if (o != 0.0) R = csub(R, cscale(cconj(mm[i * nn + bb * n + d]), o));
      }
    }
    if (bb == d) {
      for (int i = 0; i < n_sites; ++i) {
        double o = occ[i * n + bb];
        if (o != 0.0) R = csub(R, cscale(mm[i * nn + a * n + c], o));
      }
    }
  } else {
    const double* k = K + b * K_stride;
    for (int i = 0; i < n_sites; ++i) {
      double kac = k[i * nn + a * n + c], kbd = k[i * nn + bb * n + d];
      if (kac != 0.0) R = csub(R, cscale(cconj(mm[i * nn + bb * n + d]), kac));
      if (kbd != 0.0) R = csub(R, cscale(mm[i * nn + a * n + c], kbd));
    }
  }
  if (secular && !((a == bb && c == d) || (a == c && bb == d))) R = cmk(0.0, 0.0);
  L[b * (int64_t)m * m + e] = csub(val, R);
}

// ------------------------------------------------ RK4 one-step propagator
// C = A * B for m x m complex tiles in shared memory.  Each thread owns a 4 x 4
// block of C (8 shared loads per 16 complex MACs); `store(e, acc)` writes the
// result element e = row * m + col.
template <int TR, int TC, typename C, typename Store>
__device__ __forceinline__ void cgemm_tiled(const C* __restrict__ A, const C* __restrict__ B,
                                            int m, Store store) {
  // Thread (r', c') owns rows r' + i nbr (i < TR) and columns c' + j nbc
  // (j < TC): consecutive threads read consecutive B columns (conflict-free)
  // and share A rows (broadcast).
  using T = decltype(A[0].x);
  const int nbr = (m + TR - 1) / TR, nbc = (m + TC - 1) / TC;
  for (int blk = threadIdx.x; blk < nbr * nbc; blk += blockDim.x) {
    const int r0 = blk / nbc, c0 = blk % nbc;
    C acc[TR][TC];
#pragma unroll
    for (int i = 0; i < TR; ++i)
#pragma unroll
      for (int j = 0; j < TC; ++j) acc[i][j] = cmk((T)0, (T)0);
    for (int k = 0; k < m; ++k) {
      C a[TR], b[TC];
#pragma unroll
      for (int i = 0; i < TR; ++i)
        a[i] = (r0 + i * nbr < m) ? A[(r0 + i * nbr) * m + k] : cmk((T)0, (T)0);
#pragma unroll
      for (int j = 0; j < TC; ++j)
        b[j] = (c0 + j * nbc < m) ? B[k * m + c0 + j * nbc] : cmk((T)0, (T)0);
#pragma unroll
      for (int i = 0; i < TR; ++i)
#pragma unroll
        for (int j = 0; j < TC; ++j) cfma(acc[i][j], a[i], b[j]);
    }
#pragma unroll
    for (int i = 0; i < TR; ++i)
#pragma unroll
      for (int j = 0; j < TC; ++j)
        if (r0 + i * nbr < m && c0 + j * nbc < m)
          store((r0 + i * nbr) * m + c0 + j * nbc, acc[i][j]);
  }
}

// C = A B for m x m complex tiles in shared memory, results handed to
// store(index, value).  The register tile TR x TC is chosen per m to keep
// every thread busy: estimated issue cost per k = passes * (4 TR TC FMA +
// TR + TC loads), e.g. 5 x 2 tiles (250 threads) at m = 49, 4 x 4 at m = 64.
template <typename C, typename Store>
__device__ __forceinline__ void smem_cgemm(const C* __restrict__ A, const C* __restrict__ B,
                                           int m, Store store) {
  constexpr int NC = 8;
  const int tr[NC] = {1, 2, 2, 3, 4, 3, 4, 5};
  const int tc[NC] = {1, 1, 2, 2, 2, 3, 4, 2};
  int best = 0, bestc = 0x7fffffff;
  const int nt = blockDim.x;
  for (int i = 0; i < NC; ++i) {
    const int tiles = ((m + tr[i] - 1) / tr[i]) * ((m + tc[i] - 1) / tc[i]);
    const int cost = ((tiles + nt - 1) / nt) * (4 * tr[i] * tc[i] + tr[i] + tc[i]);
    if (cost < bestc) {
      bestc = cost;
      best = i;
    }
  }
  switch (best) {
    case 0: cgemm_tiled<1, 1>(A, B, m, store); break;
    case 1: cgemm_tiled<2, 1>(A, B, m, store); break;
    case 2: cgemm_tiled<2, 2>(A, B, m, store); break;
    case 3: cgemm_tiled<3, 2>(A, B, m, store); break;
    case 4: cgemm_tiled<4, 2>(A, B, m, store); break;
    case 5: cgemm_tiled<3, 3>(A, B, m, store); break;
    case 6: cgemm_tiled<4, 4>(A, B, m, store); break;
    default: cgemm_tiled<5, 2>(A, B, m, store); break;
  }
}

// C = A B for real matrices in shared memory with row stride ld (a multiple
// of 4, columns beyond the data zero): A has `rows` rows (a multiple of 4),
// B is ld x ld.  Each thread owns a 4 x 4 block of C and per four k reads four
// float4 of A rows and four float4 of B rows (64 FMA per 8 vector loads, no
// bounds tests in the loop); store(r0, c0, acc) receives the block.
struct Quad {
  float x, y, z, w;
};
struct QuadD {
  double x, y, z, w;
};
// four consecutive values from 16-byte aligned shared memory
__device__ __forceinline__ Quad load4(const float* p) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ QuadD load4(const double* p) {
  const double2 a = *reinterpret_cast<const double2*>(p);
  const double2 b = *reinterpret_cast<const double2*>(p + 2);
  return {a.x, a.y, b.x, b.y};
}

template <typename T, typename Store>
__device__ __forceinline__ void rgemm_4x4(const T* __restrict__ A, const T* __restrict__ B,
                                          int ld, int rows, Store store) {
  using V4 = typename std::conditional<sizeof(T) == 4, Quad, QuadD>::type;
  const int nct = ld / 4;
  const int ntiles = (rows / 4) * nct;
  for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
    const int r0 = (t / nct) * 4, c0 = (t % nct) * 4;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = (T)0;
    for (int k = 0; k < ld; k += 4) {
      V4 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = load4(A + (r0 + i) * ld + k);
#pragma unroll
      for (int q = 0; q < 4; ++q) b[q] = load4(B + (k + q) * ld + c0);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const T av[4] = {a[i].x, a[i].y, a[i].z, a[i].w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          acc[i][0] = fma(av[q], b[q].x, acc[i][0]);
          acc[i][1] = fma(av[q], b[q].y, acc[i][1]);
          acc[i][2] = fma(av[q], b[q].z, acc[i][2]);
          acc[i][3] = fma(av[q], b[q].w, acc[i][3]);
        }
      }
    }
    store(r0, c0, acc);
  }
}

// (I + X)(I + Y) - I = X + Y + X Y for padded ld x ld shared matrices (rows
// of X: `rows`); Z may be global (ldz, only the first m rows/cols written)
// or shared.
template <typename T>
__device__ __forceinline__ void compose_into(const T* X, const T* Y, int ld, int rows, int m,
                                             T* Z, int ldz) {
  rgemm_4x4<T>(X, Y, ld, rows, [&](int r0, int c0, T (&acc)[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int r = r0 + i, c = c0 + j;
        if (r < m && c < m) Z[r * ldz + c] = (X[r * ld + c] + Y[r * ld + c]) + acc[i][j];
      }
  });
}

// Real form of a Hermiticity-preserving map on n x n matrices (m = n^2,
// column-stacked).  Coordinates of a Hermitian rho: x[a + n b] = Re rho_ab
// for a <= b and Im rho_ba for a > b.  Input coordinate l = c + n d is the
// Hermitian basis matrix E_cc (c = d), E_cd + E_dc (c < d) or
// i E_dc - i E_cd (c > d); R[k][l] is coordinate k of A applied to it.
template <typename C>
__device__ __forceinline__ auto hermitian_entry(const C* __restrict__ A, int lda, int n, int k,
                                                int l) -> decltype(A[0].x) {
  const int a = k % n, b = k / n, c = l % n, d = l / n;
  const int row = a <= b ? a + n * b : b + n * a;
  const C* Ar = A + (size_t)row * lda;
  C v;
  if (c == d) {
    v = Ar[l];
  } else if (c < d) {
    v = cadd2(Ar[c + n * d], Ar[d + n * c]);
  } else {  // i (A[:, d + n c] - A[:, c + n d])
    const C u = Ar[d + n * c], w = Ar[c + n * d];
    v = cmk(-(u.y - w.y), u.x - w.x);
  }
  return a <= b ? v.x : v.y;
}

// Rows of complex column-stacked n x n matrices V to and from Hermitian
// coordinates of their Hermitian and anti-Hermitian parts: V = V_h + i V_a
// with V_h = (V + V^H) / 2 and V_a = (V - V^H) / 2i, coordinates as above.
// Split: in complex [batch][rows][m] -> out real [batch][2 rows][m] (the
// V_h rows, then the V_a rows); merge: the inverse.
template <typename T>
__global__ void hermitian_rows_kernel(const void* __restrict__ in, int n, int64_t rows,
                                      int merge, void* __restrict__ out) {
  using C = typename cplx<T>::type;
  const int m = n * n;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= rows * m) return;
  const int64_t b = blockIdx.y, r = e / m;
  const int k = (int)(e % m), a = k % n, c = k / n;
  const int q = c + n * a;   // the transposed entry
  if (!merge) {
    const C* v = (const C*)in + (b * rows + r) * m;
    const C vp = v[k], vq = v[q];
    T xh, xa;
    if (a <= c) {
      xh = (T)0.5 * (vp.x + vq.x);
      xa = (T)0.5 * (vp.y + vq.y);
    } else {
      xh = (T)0.5 * (vq.y - vp.y);
      xa = (T)0.5 * (vp.x - vq.x);
    }
    T* o = (T*)out + (b * 2 * rows + r) * m;
    o[k] = xh;
    o[rows * m + k] = xa;
  } else {
    const T* xh = (const T*)in + (b * 2 * rows + r) * m;
    const T* xa = xh + rows * m;
    // V_h[a][c] and V_a[a][c] from their coordinates
    T hr, hi, ar, ai;
    if (a == c) {
      hr = xh[k]; hi = (T)0; ar = xa[k]; ai = (T)0;
    } else if (a < c) {
      hr = xh[k]; hi = xh[q]; ar = xa[k]; ai = xa[q];
    } else {
      hr = xh[q]; hi = -xh[k]; ar = xa[q]; ai = -xa[k];
    }
    C* o = (C*)out + (b * rows + r) * m;
    o[k] = cmk(hr - ai, hi + ar);
  }
}

// D = P - I for one RK4 step, P = sum_{k<=4} A^k / k!, A = h L, evaluated
// Paterson-Stockmeyer style with two products:
//   A2 = A A,   D = A + A2 / 2 + A2 (A / 6 + A2 / 24).
// On entry sA holds L; sA, sB, sC are m x m shared tiles.
template <typename T>
__device__ void rk4_polynomial(typename cplx<T>::type* sA, typename cplx<T>::type* sB,
                               typename cplx<T>::type* sC, int m, double h,
                               typename cplx<T>::type* D) {
  using C = typename cplx<T>::type;
  const int mm = m * m;
  const T ht = (T)h;
  for (int e = threadIdx.x; e < mm; e += blockDim.x) sA[e] = cmk(ht * sA[e].x, ht * sA[e].y);
  __syncthreads();
  smem_cgemm(sA, sA, m, [&](int e, C v) { sB[e] = v; });  // A2
  __syncthreads();
  const T c6 = (T)(1.0 / 6.0), c24 = (T)(1.0 / 24.0), c2 = (T)0.5;
  for (int e = threadIdx.x; e < mm; e += blockDim.x)
    sC[e] = cmk(c6 * sA[e].x + c24 * sB[e].x, c6 * sA[e].y + c24 * sB[e].y);
  __syncthreads();
  smem_cgemm(sB, sC, m, [&](int e, C z) {
    D[e] = cmk(sA[e].x + c2 * sB[e].x + z.x, sA[e].y + c2 * sB[e].y + z.y);
  });
}

// Fused: site-basis generator block -> shared memory -> RK4 polynomial.
// The block is assembled from the per-state operators
//   B[s] = G - sum_i occ_is M_i,
//   L[(a,b),(c,d)] = d_bd (-B[b]_ac - i uc H_ac) + d_ac (-conj(B[a]_bd) + i uc H_db),
// which is the K == NULL branch of liouvillian_kernel regrouped.
template <typename T>
__global__ void __launch_bounds__(256, 2)
    redfield_propagator_kernel(const double* __restrict__ H, int64_t H_stride,
                               const double2* __restrict__ G, const double2* __restrict__ Mo,
                               const double* __restrict__ occ, int n, int n_sites, double uc,
                               const int* __restrict__ idx, int m, int transpose, double h,
                               typename cplx<T>::type* D) {
  using C = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nn = n * n;
  C* sB = (C*)smraw;                  // n * n * n
  C* sHs = sB + (size_t)n * nn;       // n * n, i * uc * H stored as (0, uc H)
  C* sL = sHs + nn;                   // m * m
  C* sX = sL + m * m;
  C* sY = sX + m * m;
  int* sIdx = (int*)(sY + m * m);     // m
  C* sGM = (C*)(sIdx + ((m + 3) & ~3));  // (1 + n_sites) n^2: G, M_i (16-byte aligned)
  T* sOcc = (T*)(sGM + (size_t)(1 + n_sites) * nn);  // n_sites n
  const int64_t b = blockIdx.x;
  const double2* g = G + b * nn;
  const double2* mo = Mo + b * (int64_t)n_sites * nn;
  // every FP64 operator entry is converted once
  for (int e = threadIdx.x; e < (1 + n_sites) * nn; e += blockDim.x) {
    const double2 v = e < nn ? g[e] : mo[e - nn];
    sGM[e] = cmk((T)v.x, (T)v.y);
  }
  for (int e = threadIdx.x; e < n_sites * n; e += blockDim.x) sOcc[e] = (T)occ[e];
  __syncthreads();
  // B[s] = G - sum_i occ_is M_i
  for (int e = threadIdx.x; e < n * nn; e += blockDim.x) {
    const int st = e / nn, xy = e % nn;
    C v = sGM[xy];
    for (int i = 0; i < n_sites; ++i) {
      const T o = sOcc[i * n + st];
      if (o != (T)0) {
        const C mv = sGM[(1 + i) * nn + xy];
        v = cmk(v.x - o * mv.x, v.y - o * mv.y);
      }
    }
    sB[e] = v;
  }
  for (int e = threadIdx.x; e < nn; e += blockDim.x) sHs[e] = cmk((T)0, (T)(uc * H[b * H_stride + e]));
  for (int e = threadIdx.x; e < m; e += blockDim.x) {
    const int v = idx[e];
    sIdx[e] = (v >= 0 && v < nn) ? v : -1;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    int r = e / m, cc = e % m;
    if (transpose) { const int t = r; r = cc; cc = t; }
    const int ir = sIdx[r], ic = sIdx[cc];
    C v = cmk((T)0, (T)0);
    if (ir < 0 || ic < 0) {
      v = cmk((T)nan(""), (T)nan(""));
    } else {
      const int a = ir % n, bb = ir / n, c = ic % n, d = ic / n;
      if (bb == d) {  // -B[b]_ac - i uc H_ac
        const C x = sB[bb * nn + a * n + c], hh = sHs[a * n + c];
        v = cmk(v.x - x.x - hh.x, v.y - x.y - hh.y);
      }
      if (a == c) {  // -conj(B[a]_bd) + i uc H_db
        const C x = sB[a * nn + bb * n + d], hh = sHs[d * n + bb];
        v = cmk(v.x - x.x + hh.x, v.y + x.y + hh.y);
      }
    }
    sL[e] = v;
  }
  __syncthreads();
  rk4_polynomial<T>(sL, sX, sY, m, h, D + b * (int64_t)m * m);
}

// The same propagator for small blocks (m <= 8, n <= 8), one warp per
// sample and eight samples per CTA: the warp stages its operators in shared
// memory (coalesced, converted once), forms each generator entry with its
// B[s] sums on the fly, and evaluates the RK4 polynomial with __syncwarp
// between the dependent products, no CTA barrier.
constexpr int RPW_WARPS = 8;

template <typename T>
struct RpwSlice {
  typename cplx<T>::type gm[9 * 64];   // G, M_i (i < n_sites <= 8) on n^2 <= 64 entries
  typename cplx<T>::type hs[64];       // (0, uc H)
  typename cplx<T>::type a[64], a2[64], c[64];
  T occ[8 * 8];
  int idx[8];
};

template <typename T>
__global__ void __launch_bounds__(32 * RPW_WARPS)
    redfield_propagator_w_kernel(const double* __restrict__ H, int64_t H_stride,
                                 const double2* __restrict__ G, const double2* __restrict__ Mo,
                                 const double* __restrict__ occ, int n, int n_sites, double uc,
                                 const int* __restrict__ idx, int m, int transpose, double h,
                                 int64_t batch, typename cplx<T>::type* D) {
  using C = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t b = (int64_t)blockIdx.x * RPW_WARPS + w;
  if (b >= batch) return;   // whole warps only: no CTA barrier follows
  RpwSlice<T>& S = reinterpret_cast<RpwSlice<T>*>(smraw)[w];
  const int nn = n * n, mm = m * m;
  const double2* g = G + b * nn;
  const double2* mo = Mo + b * (int64_t)n_sites * nn;
  for (int e = lane; e < (1 + n_sites) * nn; e += 32) {
    const double2 v = e < nn ? g[e] : mo[e - nn];
    S.gm[e] = cmk((T)v.x, (T)v.y);
  }
  for (int e = lane; e < n_sites * n; e += 32) S.occ[e] = (T)occ[e];
  for (int e = lane; e < nn; e += 32) S.hs[e] = cmk((T)0, (T)(uc * H[b * H_stride + e]));
  if (lane < m) {
    const int v = idx[lane];
    S.idx[lane] = (v >= 0 && v < nn) ? v : -1;
  }
  __syncwarp();
  // B[s]_xy = G_xy - sum_i occ_is M_i,xy, in the CTA kernel's order
  auto bval = [&](int st, int xy) -> C {
    C v = S.gm[xy];
    for (int i = 0; i < n_sites; ++i) {
      const T o = S.occ[i * n + st];
      if (o != (T)0) {
        const C mv = S.gm[(1 + i) * nn + xy];
        v = cmk(v.x - o * mv.x, v.y - o * mv.y);
      }
    }
    return v;
  };
  const T ht = (T)h;
  for (int e = lane; e < mm; e += 32) {
    int r = e / m, cc = e % m;
    if (transpose) { const int t = r; r = cc; cc = t; }
    const int ir = S.idx[r], ic = S.idx[cc];
    C v = cmk((T)0, (T)0);
    if (ir < 0 || ic < 0) {
      v = cmk((T)nan(""), (T)nan(""));
    } else {
      const int a = ir % n, bb = ir / n, c = ic % n, d = ic / n;
      if (bb == d) {  // -B[b]_ac - i uc H_ac
        const C x = bval(bb, a * n + c), hh = S.hs[a * n + c];
        v = cmk(v.x - x.x - hh.x, v.y - x.y - hh.y);
      }
      if (a == c) {  // -conj(B[a]_bd) + i uc H_db
        const C x = bval(a, bb * n + d), hh = S.hs[d * n + bb];
        v = cmk(v.x - x.x + hh.x, v.y + x.y + hh.y);
      }
    }
    S.a[e] = cmk(ht * v.x, ht * v.y);
  }
  __syncwarp();
  for (int e = lane; e < mm; e += 32) {  // A2 = A A
    const int r = e / m, cc = e % m;
    C acc = cmk((T)0, (T)0);
    for (int j = 0; j < m; ++j) cfma(acc, S.a[r * m + j], S.a[j * m + cc]);
    S.a2[e] = acc;
  }
  __syncwarp();
  const T c6 = (T)(1.0 / 6.0), c24 = (T)(1.0 / 24.0), c2 = (T)0.5;
  for (int e = lane; e < mm; e += 32)
    S.c[e] = cmk(c6 * S.a[e].x + c24 * S.a2[e].x, c6 * S.a[e].y + c24 * S.a2[e].y);
  __syncwarp();
  C* Dr = D + b * (int64_t)mm;
  for (int e = lane; e < mm; e += 32) {  // D = A + A2 / 2 + A2 (A / 6 + A2 / 24)
    const int r = e / m, cc = e % m;
    C z = cmk((T)0, (T)0);
    for (int j = 0; j < m; ++j) cfma(z, S.a2[r * m + j], S.c[j * m + cc]);
    Dr[e] = cmk(S.a[e].x + c2 * S.a2[e].x + z.x, S.a[e].y + c2 * S.a2[e].y + z.y);
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
    propagator_kernel(const double2* __restrict__ L, int m, double h,
                      typename cplx<T>::type* D) {
  using C = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sL = (C*)smraw;
  C* sX = sL + m * m;
  C* sY = sX + m * m;
  const int64_t b = blockIdx.x;
  const int mm = m * m;
  const double2* l = L + b * mm;
  for (int e = threadIdx.x; e < mm; e += blockDim.x) {
    double2 v = l[e];
    sL[e] = cmk((T)v.x, (T)v.y);
  }
  __syncthreads();
  rk4_polynomial<T>(sL, sX, sY, m, h, D + b * mm);
}

// ------------------------------------------- K-step blocked propagators
// From D = P - I (one RK4 step) build, per sample, the (m + nsel (K-1)) x m
// matrix whose first m rows are D_K = P^K - I and whose row m + (k-1) nsel + q
// is row select[q] of D_k = P^k - I (k = 1 .. K-1).  D_K comes from binary
// powering with (I + X)(I + Y) = I + X + Y + X Y; the selected rows follow
// R_{k+1} = R_k + R_1 + R_k D.
template <typename T>
__global__ void __launch_bounds__(256)
    block_matrix_kernel(const typename cplx<T>::type* __restrict__ D, int m, int K,
                        const int* __restrict__ sel, int nsel,
                        typename cplx<T>::type* __restrict__ out) {
  using C = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int mm = m * m;
  C* bufs[3];
  bufs[0] = (C*)smraw;             // D, then a rotating buffer
  bufs[1] = bufs[0] + mm;
  bufs[2] = bufs[1] + mm;
  C* sR = bufs[2] + mm;            // current selected rows R_k  [nsel][m]
  C* sR2 = sR + nsel * m;          // next selected rows
  const C* sD = bufs[0];
  const int64_t b = blockIdx.x;
  const int rows = m + nsel * (K - 1);
  const C* d = D + b * mm;
  C* o = out + b * (int64_t)rows * m;
  for (int e = threadIdx.x; e < mm; e += blockDim.x) bufs[0][e] = d[e];
  for (int e = threadIdx.x; e < nsel * m; e += blockDim.x) {
    const int q = e / m, c = e % m;
    int r = sel[q];
    r = (r >= 0 && r < m) ? r : 0;
    sR[e] = d[r * m + c];
    if (K > 1) o[(int64_t)(m + q) * m + c] = d[r * m + c];
  }
  __syncthreads();
  // selected rows of D_2 .. D_{K-1}: R_{k+1} = R_k + R_1 + R_k D
  for (int k = 2; k < K; ++k) {
    for (int e = threadIdx.x; e < nsel * m; e += blockDim.x) {
      const int q = e / m, c = e % m;
      int r = sel[q];
      r = (r >= 0 && r < m) ? r : 0;
      const C* rq = sR + q * m;
      C a0 = cadd2(sR[e], sD[r * m + c]), a1 = cmk((T)0, (T)0), a2 = a1, a3 = a1;
      int j = 0;
      for (; j + 3 < m; j += 4) {
        cfma(a0, rq[j], sD[j * m + c]);
        cfma(a1, rq[j + 1], sD[(j + 1) * m + c]);
        cfma(a2, rq[j + 2], sD[(j + 2) * m + c]);
        cfma(a3, rq[j + 3], sD[(j + 3) * m + c]);
      }
      for (; j < m; ++j) cfma(a0, rq[j], sD[j * m + c]);
      const C v = cadd2(cadd2(a0, a1), cadd2(a2, a3));
      sR2[e] = v;
      o[(int64_t)(m + (k - 1) * nsel + q) * m + c] = v;
    }
    __syncthreads();
    C* t = sR;
    sR = sR2;
    sR2 = t;
  }
  // D_K = P^K - I by binary powering over three rotating shared buffers;
  // each product folds (I + X)(I + Y) - I = X + Y + X Y into its store
  int res = -1, base = 0;
  for (int kk = K; kk > 0; kk >>= 1) {
    const bool last = (kk >> 1) == 0;
    if (kk & 1) {
      if (res < 0) {
        res = base;
        if (last)
          for (int e = threadIdx.x; e < mm; e += blockDim.x) o[e] = bufs[res][e];
      } else {
        const C* X = bufs[res];
        const C* Y = bufs[base];
        if (last) {
          smem_cgemm(X, Y, m, [&](int e, C v) { o[e] = cadd2(cadd2(X[e], Y[e]), v); });
        } else {
          const int f = 3 - res - base;
          C* Z = bufs[f];
          smem_cgemm(X, Y, m, [&](int e, C v) { Z[e] = cadd2(cadd2(X[e], Y[e]), v); });
          __syncthreads();
          res = f;
        }
      }
    }
    if (kk > 1) {
      const int f = (res != 1 && base != 1) ? 1 : ((res != 2 && base != 2) ? 2 : 0);
      const C* X = bufs[base];
      C* Z = bufs[f];
      smem_cgemm(X, X, m, [&](int e, C v) { Z[e] = cadd2(cadd2(X[e], X[e]), v); });
      __syncthreads();
      base = f;
    }
  }
}

// Real one-step propagator D_r = P_r - I of a Hermitian diagonal block of nb
// states (m = nb^2) from the per-sample operators.  The real generator is a
// fixed sparse linear map of the sources
//   S = [Re B[s]_xy, Im B[s]_xy (s, x, y < nb)], [uc H_xy (x, y < nb)],
// B[s] = G - sum_i occ_is M_i restricted to the block; every entry of the
// real generator combines at most four sources with coefficients in
// {0, +-1, +-2}, given per entry (row-major) as one int4: source indices
// (16 bits each) in .x, .y and four signed 8-bit coefficients in .z, built
// once by the host.  So the assembly is nb^3 operator sums in the working
// precision plus one 16-byte load and four multiply-adds per entry.
//
// NB > 0 fixes the block size at compile time (the index divisions and the
// product loops then fold to constants); NB = 0 takes nb at run time.
template <typename T, int NB>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2)
    hermitian_propagator_kernel(const double* __restrict__ H, int64_t H_stride,
                                const double2* __restrict__ G, const double2* __restrict__ Mo,
                                const double* __restrict__ occ, int n, int n_sites,
                                const int* __restrict__ states, int nb_rt,
                                const int4* __restrict__ recipe, double uc, double h,
                                T* __restrict__ D) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int nb = NB ? NB : nb_rt;
  const int m = nb * nb, ld = (m + 3) & ~3, nb3 = nb * m;
  T* rA = (T*)smraw;
  T* rB = rA + ld * ld;
  T* rC = rB + ld * ld;
  T* src = rC + ld * ld;               // [2 nb^3 + nb^2]
  T* gm = src + 2 * nb3 + m;           // [1 + n_sites][2][nb^2]: G, M_i on the block
  T* so = gm + 2 * (1 + n_sites) * m;  // [n_sites][nb] occupations of the block states
  int* st = (int*)(so + n_sites * nb); // [nb]
  const int64_t b = blockIdx.x;
  const double2* g = G + b * (int64_t)n * n;
  const double2* mo = Mo + b * (int64_t)n_sites * n * n;
  // rA keeps zero padding (rB and rC are written whole by the steps below)
  for (int e = threadIdx.x; e < ld * ld * (int)sizeof(T) / 16; e += blockDim.x)
    reinterpret_cast<uint4*>(rA)[e] = make_uint4(0u, 0u, 0u, 0u);
  for (int e = threadIdx.x; e < nb; e += blockDim.x) st[e] = states[e];
  __syncthreads();
  // every FP64 operator entry of the block is converted once
  for (int e = threadIdx.x; e < (1 + n_sites) * m; e += blockDim.x) {
    const int i = e / m, xy = e % m;
    const int f = st[xy / nb] * n + st[xy % nb];
    const double2 v = i == 0 ? g[f] : mo[(int64_t)(i - 1) * n * n + f];
    gm[2 * i * m + xy] = (T)v.x;
    gm[(2 * i + 1) * m + xy] = (T)v.y;
  }
  for (int e = threadIdx.x; e < n_sites * nb; e += blockDim.x)
    so[e] = (T)occ[(e / nb) * n + st[e % nb]];
  for (int e = threadIdx.x; e < m; e += blockDim.x)
    src[2 * nb3 + e] = (T)(uc * H[b * H_stride + st[e / nb] * n + st[e % nb]]);
  __syncthreads();
  for (int e = threadIdx.x; e < nb3; e += blockDim.x) {
    const int s = e / m, xy = e % m;
    T vx = gm[xy], vy = gm[m + xy];
    for (int i = 0; i < n_sites; ++i) {
      const T o = so[i * nb + s];
      vx = fma(-o, gm[2 * (i + 1) * m + xy], vx);
      vy = fma(-o, gm[(2 * (i + 1) + 1) * m + xy], vy);
    }
    src[e] = vx;
    src[nb3 + e] = vy;
  }
  __syncthreads();
  const T ht = (T)h;
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int4 rq = recipe[e];
    const int cz = rq.z;
    T acc = (T)(signed char)(cz & 0xff) * src[rq.x & 0xffff];
    acc = fma((T)(signed char)((cz >> 8) & 0xff), src[(rq.x >> 16) & 0xffff], acc);
    acc = fma((T)(signed char)((cz >> 16) & 0xff), src[rq.y & 0xffff], acc);
    acc = fma((T)(signed char)((cz >> 24) & 0xff), src[(rq.y >> 16) & 0xffff], acc);
    rA[(e / m) * ld + e % m] = ht * acc;
  }
  __syncthreads();
  rgemm_4x4<T>(rA, rA, ld, ld, [&](int r0, int c0, T (&acc)[4][4]) {  // A2
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) rB[(r0 + i) * ld + c0 + j] = acc[i][j];
  });
  __syncthreads();
  const T c6 = (T)(1.0 / 6.0), c24 = (T)(1.0 / 24.0), c2 = (T)0.5;
  for (int e = threadIdx.x; e < ld * ld; e += blockDim.x) rC[e] = c6 * rA[e] + c24 * rB[e];
  __syncthreads();
  T* Dr = D + b * (int64_t)m * m;
  rgemm_4x4<T>(rB, rC, ld, ld, [&](int r0, int c0, T (&acc)[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int r = r0 + i, c = c0 + j;
        if (r < m && c < m) Dr[r * m + c] = rA[r * ld + c] + c2 * rB[r * ld + c] + acc[i][j];
      }
  });
}

// One 4 x 4 tile of C = A B (row stride ld for A, B), accumulators returned.
template <typename T>
__device__ __forceinline__ void rtile_4x4(const T* __restrict__ A, const T* __restrict__ B,
                                          int ld, int r0, int c0, T (&acc)[4][4]) {
  using V4 = typename std::conditional<sizeof(T) == 4, Quad, QuadD>::type;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = (T)0;
  for (int k = 0; k < ld; k += 4) {
    V4 a[4], bq[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = load4(A + (r0 + i) * ld + k);
#pragma unroll
    for (int q = 0; q < 4; ++q) bq[q] = load4(B + (k + q) * ld + c0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const T av[4] = {a[i].x, a[i].y, a[i].z, a[i].w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        acc[i][0] = fma(av[q], bq[q].x, acc[i][0]);
        acc[i][1] = fma(av[q], bq[q].y, acc[i][1]);
        acc[i][2] = fma(av[q], bq[q].z, acc[i][2]);
        acc[i][3] = fma(av[q], bq[q].w, acc[i][3]);
      }
    }
  }
}

// Real counterpart of block_matrix_kernel for the Hermitian real form:
// out rows 0..m-1 = D_K = P^K - I, then the selected rows R_k of D_k for
// k = 1..K-1 (row m + (k-1) nsel + q = row sel[q] of D_k).
// Shared memory holds the squares D_{2^j} (padded to ld = 4 ceil(m/4)), two
// accumulators for the binary powering of D_K, and the selected rows.  Phase
// j forms, from D_{2^j}, both the next square D_{2^{j+1}} = 2 D + D D and the
// rows R_{i + 2^j} = R_i + R_{2^j} + R_i D_{2^j} (i <= 2^j), the two products'
// 4 x 4 tiles spread over the whole CTA between one pair of barriers; D_K
// then follows from the squares by composition over the set bits of K.
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 2)
    block_matrix_real_kernel(const T* __restrict__ D, int m, int K, const int* __restrict__ sel,
                             int nsel, T* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ld = (m + 3) & ~3;
  const int mm = ld * ld;
  const int nct = ld / 4;
  int J = 0;
  while ((2 << J) <= K) ++J;                 // squares D_{2^0} .. D_{2^J}
  // composition buffers are needed only when K has more than two set bits
  const int nacc = __popc(K) > 2 ? 2 : 0;
  T* sq = (T*)smraw;                          // [J + 1][ld][ld]
  T* acc0 = sq + (size_t)(J + 1) * mm;        // [nacc][ld][ld]
  T* acc1 = acc0 + mm;
  const int rrows = ((nsel * (K - 1) + 3) & ~3) + 4;
  T* sR = acc0 + (size_t)nacc * mm;           // [rrows][ld] selected rows R_1 .. R_{K-1}
  const int64_t b = blockIdx.x;
  const int rows = m + nsel * (K - 1);
  const T* d = D + b * (int64_t)m * m;
  // samples are padded to a multiple of four values, so every sample starts
  // on a 16-byte boundary (the time loop prefetches them with 16-byte copies)
  T* o = out + b * (((int64_t)rows * m + 3) & ~(int64_t)3);
  // zero everything first: the padding rows and columns of every matrix
  // must stay zero because the tiled products read them
  const int total = (J + 1 + nacc) * mm + rrows * ld;
  for (int e = threadIdx.x; e < total; e += blockDim.x) sq[e] = (T)0;
  __syncthreads();
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) sq[(e / m) * ld + e % m] = d[e];
  __syncthreads();
  for (int e = threadIdx.x; e < nsel * ld; e += blockDim.x) {
    const int q = e / ld, c = e % ld;
    int r = sel[q];
    r = (r >= 0 && r < m) ? r : 0;
    sR[e] = sq[r * ld + c];
  }
  __syncthreads();
  int have = 1;  // R_1 .. R_have are in sR
  for (int j = 0; j < J || have < K - 1; ++j) {
    const T* Dj = sq + (size_t)j * mm;
    const bool square = j < J;                       // D_{2^{j+1}} still needed
    const int add = have < K - 1 ? min(1 << j, K - 1 - have) : 0;
    const int arows = (add * nsel + 3) & ~3;
    const int nsq = square ? nct * nct : 0;
    const int ntiles = nsq + (arows / 4) * nct;
    T* Z = sq + (size_t)(j + 1) * mm;
    T* dst = sR + (size_t)have * nsel * ld;
    const T* Rb = sR + (size_t)((1 << j) - 1) * nsel * ld;  // rows of D_{2^j}
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
      T acc[4][4];
      if (t < nsq) {
        const int r0 = (t / nct) * 4, c0 = (t % nct) * 4;
        rtile_4x4<T>(Dj, Dj, ld, r0, c0, acc);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int r = r0 + i, c = c0 + jj;
            if (r < m && c < m) Z[r * ld + c] = (Dj[r * ld + c] + Dj[r * ld + c]) + acc[i][jj];
          }
      } else {
        const int tt = t - nsq;
        const int r0 = (tt / nct) * 4, c0 = (tt % nct) * 4;
        rtile_4x4<T>(sR, Dj, ld, r0, c0, acc);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) {
            const int r = r0 + i, c = c0 + jj;
            if (r < add * nsel && c < m)
              dst[r * ld + c] = (sR[r * ld + c] + Rb[(r % nsel) * ld + c]) + acc[i][jj];
          }
      }
    }
    __syncthreads();
    have += add;
  }
  for (int e = threadIdx.x; e < nsel * (K - 1) * m; e += blockDim.x) {
    const int rr = e / m, c = e % m;
    o[(int64_t)(m + rr) * m + c] = sR[rr * ld + c];
  }
  // D_K by binary powering over the squares
  const T* cur = nullptr;
  T* bufs[2] = {acc0, acc1};
  int nb = 0;
  int bits = K, j = 0, remaining = 0;
  for (int t = K; t; t &= t - 1) ++remaining;
  for (; bits; bits >>= 1, ++j) {
    if (!(bits & 1)) continue;
    const T* S = sq + (size_t)j * mm;
    --remaining;
    if (cur == nullptr) {
      cur = S;
      if (remaining == 0)
        for (int e = threadIdx.x; e < m * m; e += blockDim.x) o[e] = S[(e / m) * ld + e % m];
    } else if (remaining == 0) {
      compose_into<T>(cur, S, ld, ld, m, o, m);
    } else {
      T* Z = bufs[nb];
      nb ^= 1;
      compose_into<T>(cur, S, ld, ld, m, Z, ld);
      __syncthreads();
      cur = Z;
    }
  }
}

// Real form of every sample's complex matrix (a Hermiticity-preserving map
// on n x n matrices), one thread per entry.
template <typename T>
__global__ void hermitian_form_kernel(const typename cplx<T>::type* __restrict__ A, int n,
                                      int64_t batch, T* __restrict__ R) {
  const int m = n * n;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= batch * m * m) return;
  const int64_t b = t / ((int64_t)m * m);
  const int e = (int)(t % ((int64_t)m * m));
  R[t] = hermitian_entry(A + b * (int64_t)m * m, m, n, e / m, e % m);
}

// H[s] = base + diag(offsets[s]) on rows/columns [off, off + n_sites):
// the rotating-frame Hamiltonian of disorder sample s (Hamiltonian.sample,
// hamiltonian.py:552-578, which shifts the site energies).
__global__ void disordered_hamiltonians_kernel(const double* __restrict__ base, int n,
                                               const double* __restrict__ offsets,
                                               int64_t batch, int n_sites, int off,
                                               double* __restrict__ H) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int nn = n * n;
  if (t >= batch * nn) return;
  const int64_t s = t / nn;
  const int e = (int)(t % nn), r = e / n, c = e % n;
  double v = base[e];
  if (r == c && r >= off && r < off + n_sites) v += offsets[s * n_sites + (r - off)];
  H[t] = v;
}

}  // namespace qsx

using namespace qsx;

extern "C" {

int qsx_disordered_hamiltonians(const double* base, int n, const double* offsets,
                                int64_t batch, int n_sites, int off, double* H, void* stream) {
  QSX_CHECK_ARG(n >= 1 && n_sites >= 0 && off >= 0 && off + n_sites <= n && batch >= 0,
                "qsx_disordered_hamiltonians: bad sizes");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(base && H && (n_sites == 0 || offsets),
                "qsx_disordered_hamiltonians: null pointer");
  const int64_t total = batch * (int64_t)n * n;
  disordered_hamiltonians_kernel<<<(unsigned)((total + 255) / 256), 256, 0,
                                   (cudaStream_t)stream>>>(base, n, offsets, batch, n_sites, off,
                                                           H);
  QSX_LAUNCH_CHECK("qsx_disordered_hamiltonians");
  return QSX_OK;
}

int qsx_hermitian_real_form(const void* A, int n, int64_t batch, int precision, void* R,
                            void* stream) {
  QSX_CHECK_ARG(n >= 1 && n <= 32 && batch >= 0 && (precision == QSX_FP32 || precision == QSX_FP64),
                "qsx_hermitian_real_form: bad arguments (n=%d)", n);
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(A && R, "qsx_hermitian_real_form: null pointer");
  const int64_t total = batch * (int64_t)n * n * n * n;
  const unsigned grid = (unsigned)((total + 255) / 256);
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == QSX_FP32)
    hermitian_form_kernel<float><<<grid, 256, 0, s>>>((const float2*)A, n, batch, (float*)R);
  else
    hermitian_form_kernel<double><<<grid, 256, 0, s>>>((const double2*)A, n, batch, (double*)R);
  QSX_LAUNCH_CHECK("qsx_hermitian_real_form");
  return QSX_OK;
}

int qsx_rk4_block_matrix_real_batched(const void* D, int m, int64_t batch, int precision, int K,
                                      const int* select, int nselect, void* out, void* stream) {
  QSX_CHECK_ARG(m >= 1 && m <= 64 && K >= 1 && K <= 64 && nselect >= 0 && nselect <= m,
                "qsx_rk4_block_matrix_real_batched: need m <= 64, 1 <= K <= 64, nselect <= m");
  QSX_CHECK_ARG(batch >= 0 && batch <= 0x7fffffff, "qsx_rk4_block_matrix_real_batched: bad batch");
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_rk4_block_matrix_real_batched: bad precision");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(D && out && (nselect == 0 || select),
                "qsx_rk4_block_matrix_real_batched: null pointer");
  const size_t rs = precision == QSX_FP32 ? sizeof(float) : sizeof(double);
  const size_t ld = ((size_t)m + 3) & ~(size_t)3;
  int J = 0;
  while ((2 << J) <= K) ++J;
  const size_t rrows = (((size_t)nselect * (K - 1) + 3) & ~(size_t)3) + 4;
  int bits = 0;
  for (int t = K; t; t &= t - 1) ++bits;
  const size_t nacc = bits > 2 ? 2 : 0;
  const size_t smem = ((size_t)(J + 1 + nacc) * ld * ld + rrows * ld) * rs;
  if (smem > 227 * 1024) {
    set_error("qsx_rk4_block_matrix_real_batched: %zu bytes of shared memory needed", smem);
    return QSX_ERR_UNSUPPORTED;
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (precision == QSX_FP32) {
    e = cudaFuncSetAttribute(block_matrix_real_kernel<float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_block_matrix_real_batched");
    block_matrix_real_kernel<float><<<(unsigned)batch, 256, smem, s>>>(
        (const float*)D, m, K, select, nselect, (float*)out);
  } else {
    e = cudaFuncSetAttribute(block_matrix_real_kernel<double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_block_matrix_real_batched");
    block_matrix_real_kernel<double><<<(unsigned)batch, 256, smem, s>>>(
        (const double*)D, m, K, select, nselect, (double*)out);
  }
  QSX_LAUNCH_CHECK("qsx_rk4_block_matrix_real_batched");
  return QSX_OK;
}

int qsx_debye_corr(const double* x, int64_t n, double temperature,
                   double reorg_energy, double cutoff_freq, int matsubara_cutoff,
                   int real_only, double* out, void* stream) {
  QSX_CHECK_ARG(n >= 0 && (n == 0 || (x && out)), "qsx_debye_corr: bad arguments");
  QSX_CHECK_ARG(temperature > 0 && cutoff_freq > 0 && matsubara_cutoff >= 1,
                "qsx_debye_corr: temperature, cutoff and matsubara_cutoff must be positive");
  if (n == 0) return QSX_OK;
  DebyeParams p = make_debye(temperature, reorg_energy, cutoff_freq,
                             matsubara_cutoff, real_only);
  debye_corr_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      x, n, p, (double2*)out);
  QSX_LAUNCH_CHECK("qsx_debye_corr");
  return QSX_OK;
}

int qsx_eigh_batched(const double* H, int n, int64_t batch, int nblocks,
                     const int* block_starts, double* E, double* U, void* stream) {
  return qsx_eigh_batched_prec(H, n, batch, nblocks, block_starts, QSX_FP64, E, U, stream);
}

int qsx_eigh_batched_prec(const double* H, int n, int64_t batch, int nblocks,
                          const int* block_starts, int precision, double* E, double* U,
                          void* stream) {
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_eigh_batched_prec: bad precision");
  QSX_CHECK_ARG(n >= 1 && n <= EIGH_NMAX, "qsx_eigh_batched: need 1 <= n <= %d (got %d)",
                EIGH_NMAX, n);
  QSX_CHECK_ARG(batch >= 0 && nblocks >= 1 && nblocks <= n && block_starts,
                "qsx_eigh_batched: bad batch/blocks");
  QSX_CHECK_ARG(block_starts[0] == 0 && block_starts[nblocks] == n,
                "qsx_eigh_batched: blocks must cover [0, n)");
  for (int k = 0; k < nblocks; ++k)
    QSX_CHECK_ARG(block_starts[k] < block_starts[k + 1],
                  "qsx_eigh_batched: blocks must be non-empty and increasing");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(H && E && U, "qsx_eigh_batched: null pointer");
  cudaStream_t st = (cudaStream_t)stream;
  int maxb = 0;
  for (int k = 0; k < nblocks; ++k) maxb = std::max(maxb, block_starts[k + 1] - block_starts[k]);
  if (maxb > 8) {
    BlockTable tb;
    for (int k = 0; k <= EIGH_NMAX; ++k) tb.v[k] = k <= nblocks ? block_starts[k] : n;
    unsigned grid = (unsigned)((batch + EIGH_WARPS - 1) / EIGH_WARPS);
    eigh_jacobi_kernel<<<grid, 32 * EIGH_WARPS, 0, st>>>(H, n, batch, nblocks, tb, E, U);
    QSX_LAUNCH_CHECK("qsx_eigh_batched");
    return QSX_OK;
  }
  const int64_t total = batch * n * n;
  zero_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(U, total);
  const unsigned grid = (unsigned)((batch + 63) / 64);
  for (int k = 0; k < nblocks; ++k) {
    const int off = block_starts[k], nb = block_starts[k + 1] - off;
    switch (nb) {
#define B(NB)                                                                        \
  case NB:                                                                           \
    if (precision == QSX_FP32)                                                       \
      eigh_block_kernel<float, NB><<<grid, 64, 0, st>>>(H, n, off, batch, E, U);     \
    else                                                                             \
      eigh_block_kernel<double, NB><<<grid, 64, 0, st>>>(H, n, off, batch, E, U);    \
    break;
      B(1) B(2) B(3) B(4) B(5) B(6) B(7) B(8)
#undef B
    }
  }
  QSX_LAUNCH_CHECK("qsx_eigh_batched");
  return QSX_OK;
}

int qsx_redfield_operators_batched(const double* E, const double* U, int n,
                                   int64_t batch, const double* occ, int n_sites,
                                   double temperature, double reorg_energy,
                                   double cutoff_freq, int matsubara_cutoff,
                                   int discard_imag_corr, double unit_convert,
                                   int site_basis, int precision, double* G, double* M,
                                   double* K, void* stream) {
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_redfield_operators_batched: bad precision");
  QSX_CHECK_ARG(n >= 1 && n <= 32 && n_sites >= 1 && n_sites <= 32,
                "qsx_redfield_operators_batched: need 1 <= n, n_sites <= 32 (got %d, %d)",
                n, n_sites);
  QSX_CHECK_ARG(temperature > 0 && cutoff_freq > 0 && matsubara_cutoff >= 1,
                "qsx_redfield_operators_batched: bad bath parameters");
  QSX_CHECK_ARG(batch >= 0, "qsx_redfield_operators_batched: negative batch");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(E && U && occ && G && M && (site_basis || K),
                "qsx_redfield_operators_batched: null pointer");
  QSX_CHECK_ARG(batch <= 0x7fffffff, "qsx_redfield_operators_batched: batch too large");
  DebyeParams p = make_debye(temperature, reorg_energy, cutoff_freq, matsubara_cutoff,
                             discard_imag_corr);
  const size_t nn = (size_t)n * n;
  const size_t rs = precision == QSX_FP32 ? sizeof(float) : sizeof(double);
  const size_t smem = (3 * nn + 64 + (size_t)n_sites * n) * rs + 4 * nn * 2 * rs +
                      (32 + (size_t)n_sites * n) * sizeof(int);
  // one thread per matrix element (n^2 <= 1024), rounded to whole warps
  const int threads = std::min(256, (int)((nn + 31) / 32) * 32);
  cudaError_t e;
  if (precision == QSX_FP32) {
    e = cudaFuncSetAttribute(redfield_operators_kernel<float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_operators_batched");
    redfield_operators_kernel<float><<<(unsigned)batch, threads, smem, (cudaStream_t)stream>>>(
        E, U, n, batch, occ, n_sites, p, unit_convert, site_basis, (double2*)G, (double2*)M, K);
  } else {
    e = cudaFuncSetAttribute(redfield_operators_kernel<double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_operators_batched");
    redfield_operators_kernel<double><<<(unsigned)batch, threads, smem, (cudaStream_t)stream>>>(
        E, U, n, batch, occ, n_sites, p, unit_convert, site_basis, (double2*)G, (double2*)M, K);
  }
  QSX_LAUNCH_CHECK("qsx_redfield_operators_batched");
  return QSX_OK;
}

int qsx_redfield_liouvillian_batched(const double* H, int64_t H_stride, const double* G,
                                     const double* M, const double* K, int64_t K_stride,
                                     const double* occ, int n, int n_sites, int64_t batch,
                                     double unit_convert, const int* idx, int m,
                                     int secular, int transpose, double* L, void* stream) {
  QSX_CHECK_ARG(n >= 1 && n_sites >= 1 && m >= 1 && (int64_t)m <= (int64_t)n * n,
                "qsx_redfield_liouvillian_batched: bad sizes n=%d n_sites=%d m=%d", n,
                n_sites, m);
  QSX_CHECK_ARG(batch >= 0 && batch <= 65535,
                "qsx_redfield_liouvillian_batched: batch must be in [0, 65535]");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(H && G && M && idx && L && (K || occ),
                "qsx_redfield_liouvillian_batched: null pointer");
  const int64_t mm = (int64_t)m * m;
  dim3 grid((unsigned)((mm + 255) / 256), (unsigned)batch);
  liouvillian_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
      H, H_stride, (const double2*)G, (const double2*)M, K, K_stride, occ, n, n_sites,
      unit_convert, idx, m, secular, transpose, (double2*)L);
  QSX_LAUNCH_CHECK("qsx_redfield_liouvillian_batched");
  return QSX_OK;
}


int qsx_redfield_propagator_hermitian_batched(const double* H, int64_t H_stride,
                                              const double* G, const double* M,
                                              const double* occ, int n, int n_sites,
                                              int64_t batch, double unit_convert,
                                              const int* states, int nb, const int* recipe,
                                              double h, int precision, void* D, void* stream) {
  QSX_CHECK_ARG(nb >= 1 && nb <= 8 && n >= nb && n_sites >= 1 && batch >= 0 &&
                    (precision == QSX_FP32 || precision == QSX_FP64),
                "qsx_redfield_propagator_hermitian_batched: bad sizes (n=%d, nb=%d)", n, nb);
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(H && G && M && occ && states && recipe && D,
                "qsx_redfield_propagator_hermitian_batched: null pointer");
  const int m = nb * nb, ld = (m + 3) & ~3;
  const size_t rs = precision == QSX_FP32 ? sizeof(float) : sizeof(double);
  const size_t smem = (3 * (size_t)ld * ld + 2 * (size_t)nb * m + m +
                       2 * (1 + (size_t)n_sites) * m + (size_t)n_sites * nb) * rs +
                      nb * sizeof(int);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  // one thread per 4 x 4 tile of the two products, whole warps, at most 256:
  // the 169 tiles of 7 sites take 192 threads in one round (256 threads left
  // 87 idle in every product), and five such CTAs fit an SM where four of
  // 256 did (64 registers a thread)
  const int tiles = (ld / 4) * (ld / 4);
  const int threads = std::min(256, (tiles + 31) / 32 * 32);
  auto launch = [&](auto kern, auto* Dt) -> cudaError_t {
    cudaError_t fe = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem);
    if (fe != cudaSuccess) return fe;
    kern<<<(unsigned)batch, threads, smem, s>>>(H, H_stride, (const double2*)G, (const double2*)M,
                                            occ, n, n_sites, states, nb, (const int4*)recipe,
                                            unit_convert, h, Dt);
    return cudaSuccess;
  };
  // the one-exciton blocks of 7 and 8 sites get compile-time sizes
  if (precision == QSX_FP32) {
    float* Df = (float*)D;
    e = nb == 7 ? launch(hermitian_propagator_kernel<float, 7>, Df)
        : nb == 8 ? launch(hermitian_propagator_kernel<float, 8>, Df)
                  : launch(hermitian_propagator_kernel<float, 0>, Df);
  } else {
    double* Dd = (double*)D;
    e = nb == 7 ? launch(hermitian_propagator_kernel<double, 7>, Dd)
        : nb == 8 ? launch(hermitian_propagator_kernel<double, 8>, Dd)
                  : launch(hermitian_propagator_kernel<double, 0>, Dd);
  }
  if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_propagator_hermitian_batched");
  QSX_LAUNCH_CHECK("qsx_redfield_propagator_hermitian_batched");
  return QSX_OK;
}

int qsx_redfield_propagator_batched(const double* H, int64_t H_stride, const double* G,
                                    const double* M, const double* occ, int n, int n_sites,
                                    int64_t batch, double unit_convert, const int* idx, int m,
                                    int transpose, double h, int precision, void* D,
                                    void* stream) {
  QSX_CHECK_ARG(n >= 1 && n_sites >= 1 && m >= 1 && m <= 64 && (int64_t)m <= (int64_t)n * n,
                "qsx_redfield_propagator_batched: bad sizes n=%d n_sites=%d m=%d", n, n_sites,
                m);
  QSX_CHECK_ARG(batch >= 0 && batch <= 0x7fffffff,
                "qsx_redfield_propagator_batched: bad batch");
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_redfield_propagator_batched: bad precision");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(H && G && M && occ && idx && D,
                "qsx_redfield_propagator_batched: null pointer");
  const size_t nn = (size_t)n * n;
  const size_t cs = precision == QSX_FP32 ? sizeof(float2) : sizeof(double2);
  const size_t smem = ((size_t)n * nn + nn + 3 * (size_t)m * m) * cs +
                      (((size_t)m + 3) & ~(size_t)3) * sizeof(int) +
                      (1 + (size_t)n_sites) * nn * cs +
                      (size_t)n_sites * n * (cs / 2);
  if (smem > 227 * 1024) {
    set_error("qsx_redfield_propagator_batched: %zu bytes of shared memory needed; use "
              "qsx_redfield_liouvillian_batched + qsx_rk4_propagator_batched", smem);
    return QSX_ERR_UNSUPPORTED;
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (m <= 8 && n <= 8 && n_sites <= 8) {
    // small blocks: one warp per sample
    const unsigned grid = (unsigned)((batch + RPW_WARPS - 1) / RPW_WARPS);
    if (precision == QSX_FP32) {
      const size_t sm = RPW_WARPS * sizeof(RpwSlice<float>);
      e = cudaFuncSetAttribute(redfield_propagator_w_kernel<float>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_propagator_batched");
      redfield_propagator_w_kernel<float><<<grid, 32 * RPW_WARPS, sm, s>>>(
          H, H_stride, (const double2*)G, (const double2*)M, occ, n, n_sites, unit_convert, idx,
          m, transpose, h, batch, (float2*)D);
    } else {
      const size_t sm = RPW_WARPS * sizeof(RpwSlice<double>);
      e = cudaFuncSetAttribute(redfield_propagator_w_kernel<double>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_propagator_batched");
      redfield_propagator_w_kernel<double><<<grid, 32 * RPW_WARPS, sm, s>>>(
          H, H_stride, (const double2*)G, (const double2*)M, occ, n, n_sites, unit_convert, idx,
          m, transpose, h, batch, (double2*)D);
    }
    QSX_LAUNCH_CHECK("qsx_redfield_propagator_batched");
    return QSX_OK;
  }
  if (precision == QSX_FP32) {
    e = cudaFuncSetAttribute(redfield_propagator_kernel<float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_propagator_batched");
    redfield_propagator_kernel<float><<<(unsigned)batch, 256, smem, s>>>(
        H, H_stride, (const double2*)G, (const double2*)M, occ, n, n_sites, unit_convert, idx, m,
        transpose, h, (float2*)D);
  } else {
    e = cudaFuncSetAttribute(redfield_propagator_kernel<double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_propagator_batched");
    redfield_propagator_kernel<double><<<(unsigned)batch, 256, smem, s>>>(
        H, H_stride, (const double2*)G, (const double2*)M, occ, n, n_sites, unit_convert, idx, m,
        transpose, h, (double2*)D);
  }
  QSX_LAUNCH_CHECK("qsx_redfield_propagator_batched");
  return QSX_OK;
}

int qsx_rk4_block_matrix_batched(const void* D, int m, int64_t batch, int precision, int K,
                                 const int* select, int nselect, void* out, void* stream) {
  QSX_CHECK_ARG(m >= 1 && m <= 64 && K >= 1 && K <= 64 && nselect >= 0 && nselect <= m,
                "qsx_rk4_block_matrix_batched: need m <= 64, 1 <= K <= 64, nselect <= m");
  QSX_CHECK_ARG(batch >= 0 && batch <= 0x7fffffff, "qsx_rk4_block_matrix_batched: bad batch");
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_rk4_block_matrix_batched: bad precision");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(D && out && (nselect == 0 || select),
                "qsx_rk4_block_matrix_batched: null pointer");
  const size_t cs = precision == QSX_FP32 ? sizeof(float2) : sizeof(double2);
  const size_t smem = (3 * (size_t)m * m + 2 * (size_t)nselect * m) * cs;
  if (smem > 227 * 1024) {
    set_error("qsx_rk4_block_matrix_batched: %zu bytes of shared memory needed", smem);
    return QSX_ERR_UNSUPPORTED;
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (precision == QSX_FP32) {
    e = cudaFuncSetAttribute(block_matrix_kernel<float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_block_matrix_batched");
    block_matrix_kernel<float><<<(unsigned)batch, 256, smem, s>>>((const float2*)D, m, K, select,
                                                                 nselect, (float2*)out);
  } else {
    e = cudaFuncSetAttribute(block_matrix_kernel<double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_block_matrix_batched");
    block_matrix_kernel<double><<<(unsigned)batch, 256, smem, s>>>(
        (const double2*)D, m, K, select, nselect, (double2*)out);
  }
  QSX_LAUNCH_CHECK("qsx_rk4_block_matrix_batched");
  return QSX_OK;
}

int qsx_rk4_propagator_batched(const double* L, int m, int64_t batch, double h,
                               int precision, void* D, void* stream) {
  QSX_CHECK_ARG(m >= 1 && m <= 64, "qsx_rk4_propagator_batched: need 1 <= m <= 64 (got %d)",
                m);
  QSX_CHECK_ARG(batch >= 0 && batch <= 0x7fffffff, "qsx_rk4_propagator_batched: bad batch");
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_rk4_propagator_batched: bad precision");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(L && D, "qsx_rk4_propagator_batched: null pointer");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t mm = (size_t)m * m;
  if (precision == QSX_FP32) {
    size_t smem = 3 * mm * sizeof(float2);
    cudaError_t e = cudaFuncSetAttribute(propagator_kernel<float>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_propagator_batched");
    propagator_kernel<float><<<(unsigned)batch, 256, smem, s>>>((const double2*)L, m, h,
                                                                (float2*)D);
  } else {
    size_t smem = 3 * mm * sizeof(double2);
    cudaError_t e = cudaFuncSetAttribute(propagator_kernel<double>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_propagator_batched");
    propagator_kernel<double><<<(unsigned)batch, 256, smem, s>>>((const double2*)L, m, h,
                                                                 (double2*)D);
  }
  QSX_LAUNCH_CHECK("qsx_rk4_propagator_batched");
  return QSX_OK;
}

int qsx_hermitian_rows(const void* in, int n, int64_t rows, int64_t batch, int precision,
                       int merge, void* out, void* stream) {
  QSX_CHECK_ARG(n >= 1 && n <= 64 && rows >= 0 && batch >= 0 && batch <= 65535 &&
                    (merge == 0 || merge == 1) &&
                    (precision == QSX_FP32 || precision == QSX_FP64),
                "qsx_hermitian_rows: bad arguments (n=%d)", n);
  if (batch == 0 || rows == 0) return QSX_OK;
  QSX_CHECK_ARG(in && out && in != out, "qsx_hermitian_rows: null or aliased pointer");
  const int64_t total = rows * n * n;
  const dim3 grid((unsigned)((total + 255) / 256), (unsigned)batch);
  if (precision == QSX_FP32)
    hermitian_rows_kernel<float><<<grid, 256, 0, (cudaStream_t)stream>>>(in, n, rows, merge, out);
  else
    hermitian_rows_kernel<double><<<grid, 256, 0, (cudaStream_t)stream>>>(in, n, rows, merge,
                                                                         out);
  QSX_LAUNCH_CHECK("qsx_hermitian_rows");
  return QSX_OK;
}

}  // extern "C"

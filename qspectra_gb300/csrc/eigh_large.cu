// Batched FP64 symmetric eigensolver for matrices too large for the
// register Jacobi kernels (the two-exciton block: 276 states at 24 sites).
// The reference diagonalises each sample's Hamiltonian with scipy.linalg.eigh
// (qspectra/hamiltonian.py:310-328).
//
// Four kernels over a global-memory workspace:
//   1. Householder reduction to tridiagonal form (one CTA per matrix),
//      A = Q T Q^T: for each
//      column k, v with (I - tau v v^T) x = alpha e_1 and the two-sided
//      update B <- B - v w^T - w v^T, w = p - (tau/2)(v^T p) v, p = tau B v.
//   2. Eigenvalues of T by bisection on Sturm counts (one thread per
//      eigenvalue of every matrix; O(n) per count, about 50 counts).
//   3. Eigenvectors of T by inverse iteration (one thread per eigenvalue of
//      every matrix): LU with partial pivoting of
//      T - lambda I, three solves from a vector of ones; eigenvalues closer
//      than 1e-3 |T| form a cluster handled by one thread with modified
//      Gram-Schmidt against the cluster's earlier vectors.
//   4. Back-transform by the Householder reflectors, U = H_0 ... H_{n-3} Z
//      (one CTA per matrix).
// This keeps the FP64 work near 2 n^3 multiply-adds per matrix (no Givens
// rotations accumulated into Q).  Eigenvalues are returned ascending with
// U[:, k] the k-th eigenvector.  Every loop is bounded (bisection stops after
// 128 halvings, inverse iteration runs three solves).
#include <algorithm>
#include <cfloat>

#include "qsx_common.cuh"

namespace qsx {

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  const int nw = blockDim.x >> 5;
  for (int i = 0; i < nw; ++i) t += red[i];
  return t;
}

// sum_j x[j * ld] v[j]: four independent chains, eight loads in flight
__device__ __forceinline__ double col_dot(const double* __restrict__ x, int ld,
                                          const double* __restrict__ v, int m) {
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  int j = 0;
  for (; j + 7 < m; j += 8) {
    double t[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) t[q] = x[(int64_t)(j + q) * ld];
    a0 = fma(t[0], v[j], a0);
    a1 = fma(t[1], v[j + 1], a1);
    a2 = fma(t[2], v[j + 2], a2);
    a3 = fma(t[3], v[j + 3], a3);
    a0 = fma(t[4], v[j + 4], a0);
    a1 = fma(t[5], v[j + 5], a1);
    a2 = fma(t[6], v[j + 6], a2);
    a3 = fma(t[7], v[j + 7], a3);
  }
  for (; j < m; ++j) a0 = fma(x[(int64_t)j * ld], v[j], a0);
  return (a0 + a1) + (a2 + a3);
}

// x[i * ld] -= a[i] * bc + b[i] * ac for i < m, eight rows loaded before
// any is stored (the shared vectors a, b cannot alias x)
__device__ __forceinline__ void col_rank2(double* __restrict__ x, int ld,
                                          const double* __restrict__ a,
                                          const double* __restrict__ b, double bc, double ac,
                                          int m) {
  int i = 0;
  for (; i + 7 < m; i += 8) {
    double t[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) t[q] = x[(int64_t)(i + q) * ld];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      x[(int64_t)(i + q) * ld] = fma(-a[i + q], bc, fma(-b[i + q], ac, t[q]));
  }
  for (; i < m; ++i) x[(int64_t)i * ld] = fma(-a[i], bc, fma(-b[i], ac, x[(int64_t)i * ld]));
}

constexpr int TQ_THREADS = 320;

// ---- A. Householder tridiagonalisation: one CTA per matrix.  Writes the
// diagonal and sub-diagonal to de[b] = {d[0..n), e[0..n)} and keeps, in the
// work matrix W, each reflector v_k in row k right of the diagonal with
// tau_k on the diagonal.
__global__ void __launch_bounds__(TQ_THREADS, 2)
    eigh_tridiag_kernel(const double* __restrict__ A, int n, double* W, double* de) {
  extern __shared__ __align__(16) double sm[];
  double* v = sm;          // [n] Householder vector
  double* w = v + n;       // [n]
  double* red = w + n;     // [32]
  const int tid = threadIdx.x, bd = blockDim.x;
  const int64_t b = blockIdx.x;
  const int64_t nn = (int64_t)n * n;
  const double* a = A + b * nn;
  double* Wm = W + b * nn;
  double* d = de + b * 2 * (int64_t)n;
  double* e = d + n;
  for (int64_t i = tid; i < nn; i += bd) Wm[i] = a[i];
  __syncthreads();
  for (int k = 0; k < n - 2; ++k) {
    const int m = n - k - 1;
    const double* rowk = Wm + (int64_t)k * n + k + 1;
    double part = 0.0;
    for (int i = tid; i < m; i += bd) {
      const double x = rowk[i];
      v[i] = x;
      part += x * x;
    }
    const double sigma = block_sum(part, red);
    const double x0 = v[0];
    double tau = 0.0;
    if (tid == 0) d[k] = Wm[(int64_t)k * n + k];
    if (sigma - x0 * x0 > 0.0) {
      const double alpha = -copysign(sqrt(sigma), x0);
      const double v0 = x0 - alpha;
      tau = 2.0 / (sigma - x0 * x0 + v0 * v0);
      __syncthreads();
      if (tid == 0) {
        v[0] = v0;
        e[k] = alpha;
      }
      __syncthreads();
      double* B = Wm + (int64_t)(k + 1) * n + k + 1;
      // p = tau B v (B symmetric: column r read across threads)
      double vp = 0.0;
      for (int r = tid; r < m; r += bd) {
        const double wr = tau * col_dot(B + r, n, v, m);
        w[r] = wr;
        vp += v[r] * wr;
      }
      const double K = 0.5 * tau * block_sum(vp, red);
      for (int r = tid; r < m; r += bd) w[r] -= K * v[r];
      __syncthreads();
      for (int c = tid; c < m; c += bd) col_rank2(B + c, n, v, w, w[c], v[c], m);
    } else {
      if (tid == 0) e[k] = x0;
    }
    __syncthreads();
    for (int i = tid; i < m; i += bd) Wm[(int64_t)k * n + k + 1 + i] = tau != 0.0 ? v[i] : 0.0;
    if (tid == 0) Wm[(int64_t)k * n + k] = tau;
    __syncthreads();
  }
  if (tid == 0) {
    if (n >= 2) {
      d[n - 2] = Wm[(int64_t)(n - 2) * n + n - 2];
      e[n - 2] = Wm[(int64_t)(n - 1) * n + n - 2];
    }
    d[n - 1] = Wm[(int64_t)(n - 1) * n + n - 1];
    e[n - 1] = 0.0;
    if (n >= 2) Wm[(int64_t)(n - 2) * n + n - 2] = 0.0;  // no reflector for k = n-2
  }
}

// ---- B. eigenvalues by bisection on Sturm counts, one thread per
// eigenvalue of every matrix (FP64 instructions of a serial recurrence are
// slow on this part; these threads fill whole warps).  Eigenvalue j is the
// point where the count of eigenvalues below x steps from j to j + 1; the
// LDL^T recurrence q_i = (d_i - x) - e_{i-1}^2 / q_{i-1} counts negative
// pivots, with |q| kept above pivmin = eps |T|.  Results land sorted in ws.
__global__ void eigh_bisect_kernel(const double* __restrict__ de, int n, int64_t batch,
                                   double* ws, int* status) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= batch * n) return;
  const int64_t b = t / n;
  const int j = (int)(t % n);
  const double* d = de + b * 2 * (int64_t)n;
  const double* e = d + n;
  // Gershgorin interval and |T|
  double lo = d[0], hi = d[0], tnorm = 0.0;
  for (int i = 0; i < n; ++i) {
    const double r = (i ? fabs(e[i - 1]) : 0.0) + fabs(e[i]);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    tnorm = fmax(tnorm, fabs(d[i]) + r);
  }
  const double pivmin = DBL_EPSILON * fmax(tnorm, DBL_MIN);
  lo -= 2.0 * pivmin;
  hi += 2.0 * pivmin;
  for (int it = 0; it < 128; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (hi - lo <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + pivmin || mid <= lo ||
        mid >= hi)
      break;
    int cnt = 0;
    double q = d[0] - mid;
    if (fabs(q) < pivmin) q = -pivmin;
    cnt += q < 0.0;
    for (int i = 1; i < n; ++i) {
      q = (d[i] - mid) - e[i - 1] * e[i - 1] * __drcp_rn(q);
      if (fabs(q) < pivmin) q = -pivmin;
      cnt += q < 0.0;
    }
    if (cnt > j)
      hi = mid;
    else
      lo = mid;
  }
  const double lam = 0.5 * (lo + hi);
  if (!isfinite(lam) && status) atomicOr(status, QSX_ERR_NONFINITE);
  ws[b * n + j] = lam;
}

// ---- C. eigenvectors of T by inverse iteration, one thread per eigenvalue
// of every matrix; eigenvalues closer than 1e-3 |T| form a cluster handled
// by its first thread in order, with modified Gram-Schmidt against the
// cluster's earlier vectors.  Z[b] row-major, column j for eigenvalue j.
__global__ void eigh_invit_kernel(const double* __restrict__ de, const double* __restrict__ ws,
                                  int n, int64_t batch, double* Z, double* scratch) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= batch * n) return;
  const int64_t b = t / n;
  const int j = (int)(t % n);
  const double* d = de + b * 2 * (int64_t)n;
  const double* e = d + n;
  const double* w = ws + b * (int64_t)n;
  double* z = Z + b * (int64_t)n * n;
  double tnorm = 0.0;
  for (int i = 0; i < n; ++i)
    tnorm = fmax(tnorm, fabs(d[i]) + fabs(e[i]) + (i ? fabs(e[i - 1]) : 0.0));
  const double ortol = 1e-3 * tnorm;
  const double tiny = DBL_EPSILON * fmax(tnorm, DBL_MIN);
  if (j > 0 && w[j] - w[j - 1] < ortol) return;  // not the first of its cluster
  int jend = j + 1;
  while (jend < n && w[jend] - w[jend - 1] < ortol) ++jend;
  double* sc = scratch + t * 5 * (int64_t)n;
  double* u1 = sc;
  double* u2 = sc + n;
  double* u3 = sc + 2 * n;
  double* lm = sc + 3 * n;
  double* x = sc + 4 * n;
  for (int jj = j; jj < jend; ++jj) {
    // equal eigenvalues of a cluster are pulled apart slightly so that each
    // factorisation differs
    const double lam = w[jj] + (jj - j) * 10.0 * tiny;
    // LU with partial pivoting of T - lam I: u1, u2, u3 the three diagonals
    // of U, lm the multipliers (|l| <= 1; l + 4 where rows i, i+1 swapped)
    double pp = d[0] - lam, qq = n > 1 ? e[0] : 0.0;
    for (int i = 0; i < n - 1; ++i) {
      const double sub = e[i];
      const double an = d[i + 1] - lam, en = (i + 1 < n - 1) ? e[i + 1] : 0.0;
      if (fabs(pp) >= fabs(sub)) {
        if (pp == 0.0) pp = tiny;
        const double l = sub / pp;
        u1[i] = pp;
        u2[i] = qq;
        u3[i] = 0.0;
        lm[i] = l;
        pp = an - l * qq;
        qq = en;
      } else {
        const double l = pp / sub;
        u1[i] = sub;
        u2[i] = an;
        u3[i] = en;
        lm[i] = l + 4.0;
        const double np = qq - l * an;
        qq = -l * en;
        pp = np;
      }
    }
    u1[n - 1] = pp == 0.0 ? tiny : pp;
    for (int i = 0; i < n; ++i) x[i] = 1.0;  // the first solve uses U only
    for (int it = 0; it < 3; ++it) {
      if (it > 0) {
        for (int i = 0; i < n - 1; ++i) {
          const double tt = lm[i];
          if (tt > 2.0) {
            const double l = tt - 4.0;
            const double xi = x[i];
            x[i] = x[i + 1];
            x[i + 1] = xi - l * x[i];
          } else {
            x[i + 1] -= tt * x[i];
          }
        }
      }
      for (int i = n - 1; i >= 0; --i) {
        double vv = x[i];
        if (i + 1 < n) vv -= u2[i] * x[i + 1];
        if (i + 2 < n) vv -= u3[i] * x[i + 2];
        double piv = u1[i];
        if (fabs(piv) < tiny) piv = copysign(tiny, piv);
        x[i] = vv / piv;
      }
      for (int k = j; k < jj; ++k) {
        double dot = 0.0;
        for (int i = 0; i < n; ++i) dot = fma(z[(int64_t)i * n + k], x[i], dot);
        for (int i = 0; i < n; ++i) x[i] -= dot * z[(int64_t)i * n + k];
      }
      double nrm = 0.0;
      for (int i = 0; i < n; ++i) nrm = fma(x[i], x[i], nrm);
      const double inv = nrm > 0.0 ? rsqrt(nrm) : 0.0;
      for (int i = 0; i < n; ++i) x[i] *= inv;
    }
    for (int i = 0; i < n; ++i) z[(int64_t)i * n + jj] = x[i];
  }
}

// ---- D. back-transform U = H_0 H_1 ... H_{n-3} Z (reflector k acts on rows
// k+1 ..), applied from k = n-3 down to 0; writes E and U.
__global__ void __launch_bounds__(TQ_THREADS, 2)
    eigh_backtransform_kernel(const double* __restrict__ W, const double* __restrict__ ws,
                              int n, double* Z, double* __restrict__ E,
                              double* __restrict__ U) {
  extern __shared__ __align__(16) double sm[];
  double* v = sm;  // [n]
  const int tid = threadIdx.x, bd = blockDim.x;
  const int64_t b = blockIdx.x;
  const int64_t nn = (int64_t)n * n;
  const double* Wm = W + b * nn;
  double* z = Z + b * nn;
  for (int k = n - 3; k >= 0; --k) {
    const double tau = Wm[(int64_t)k * n + k];
    if (tau == 0.0) continue;
    const int m = n - k - 1;
    for (int i = tid; i < m; i += bd) v[i] = Wm[(int64_t)k * n + k + 1 + i];
    __syncthreads();
    double* Zb = z + (int64_t)(k + 1) * n;
    for (int c = tid; c < n; c += bd) {
      const double u = tau * col_dot(Zb + c, n, v, m);
      col_rank2(Zb + c, n, v, v, u, 0.0, m);
    }
    __syncthreads();
  }
  for (int i = tid; i < n; i += bd) E[b * n + i] = ws[b * n + i];
  double* u = U + b * nn;
  for (int64_t idx = tid; idx < nn; idx += bd) u[idx] = z[idx];
}

}  // namespace qsx

using namespace qsx;

extern "C" size_t qsx_eigh_large_workspace_bytes(int n, int64_t batch) {
  if (n < 1 || batch < 0) return 0;
  // reduction matrix and eigenvectors (n^2 each), inverse-iteration scratch
  // (5 n per eigenvalue), d/e, their QL copies and the sorted eigenvalues
  return ((size_t)7 * n * n + (size_t)5 * n) * (size_t)batch * sizeof(double);
}

extern "C" int qsx_eigh_large_batched(const double* H, int n, int64_t batch, double* E,
                                      double* U, void* workspace, size_t workspace_bytes,
                                      int32_t* status, void* stream) {
  QSX_CHECK_ARG(n >= 1 && n <= 2048, "qsx_eigh_large_batched: n=%d outside 1..2048", n);
  QSX_CHECK_ARG(batch >= 0 && batch <= 0x7fffffff, "qsx_eigh_large_batched: bad batch");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(H && E && U && status, "qsx_eigh_large_batched: null pointer");
  const size_t need = qsx_eigh_large_workspace_bytes(n, batch);
  QSX_CHECK_ARG(workspace && workspace_bytes >= need,
                "qsx_eigh_large_batched: workspace of %zu bytes needed (got %zu)", need,
                workspace_bytes);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nnb = (size_t)n * n * batch;
  double* W = (double*)workspace;
  double* Z = W + nnb;
  double* scratch = Z + nnb;
  double* de = scratch + 5 * nnb;
  double* ws = de + 4 * (size_t)n * batch;
  const int threads = n >= TQ_THREADS ? TQ_THREADS : ((n + 31) / 32) * 32;
  const size_t smemA = ((size_t)2 * n + 32) * sizeof(double);
  const size_t smemD = (size_t)n * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(eigh_tridiag_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemA);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(eigh_backtransform_kernel,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemD);
  if (e != cudaSuccess) return cuda_status(e, "qsx_eigh_large_batched");
  eigh_tridiag_kernel<<<(unsigned)batch, threads, smemA, s>>>(H, n, W, de);
  const int64_t nt = batch * n;
  eigh_bisect_kernel<<<(unsigned)((nt + 127) / 128), 128, 0, s>>>(de, n, batch, ws, status);
  eigh_invit_kernel<<<(unsigned)((nt + 127) / 128), 128, 0, s>>>(de, ws, n, batch, Z, scratch);
  eigh_backtransform_kernel<<<(unsigned)batch, threads, smemD, s>>>(W, ws, n, Z, E, U);
  QSX_LAUNCH_CHECK("qsx_eigh_large_batched");
  return QSX_OK;
}

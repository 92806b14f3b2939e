// Batched FP64 symmetric eigensolver for matrices too large for the
// register Jacobi kernels (the two-exciton block: 276 states at 24 sites).
// The reference diagonalises each sample's Hamiltonian with scipy.linalg.eigh
// (qspectra/hamiltonian.py:310-328).
//
// One CTA per matrix, three phases over a global-memory workspace:
//   1. Householder reduction to tridiagonal form, A = Q T Q^T: for each
//      column k, v with (I - tau v v^T) x = alpha e_1 and the two-sided
//      update B <- B - v w^T - w v^T, w = p - (tau/2)(v^T p) v, p = tau B v.
//   2. Q = H_0 H_1 ... H_{n-3} accumulated backwards from the identity.
//   3. Implicit QL iterations with Wilkinson-type shifts on T; thread 0 runs
//      each sweep's scalar recurrence and records its Givens rotations, then
//      every thread applies them to its row of Q (Q stored column-major so a
//      rotation touches consecutive addresses across threads).
// Eigenvalues are returned ascending with U[:, k] the k-th eigenvector.
// Every loop is bounded: a QL that does not converge in 60 sweeps per
// eigenvalue stops and reports QSX_ERR_NONFINITE in *status.
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

__global__ void __launch_bounds__(1024)
    eigh_tql_kernel(const double* __restrict__ A, int n, double* W, double* Zw,
                    double* __restrict__ E, double* __restrict__ U, int* status) {
  extern __shared__ __align__(16) double sm[];
  double* d = sm;          // [n] diagonal
  double* e = d + n;       // [n] sub-diagonal
  double* v = e + n;       // [n] Householder vector
  double* w = v + n;       // [n]
  double* rc = w + n;      // [n] rotation cosines
  double* rs = rc + n;     // [n] rotation sines
  double* red = rs + n;    // [32]
  int* ctl = (int*)(red + 32);  // [4] m, nrot, stop
  int* rank = ctl + 4;     // [n]
  const int tid = threadIdx.x, bd = blockDim.x;
  const int64_t b = blockIdx.x;
  const int64_t nn = (int64_t)n * n;
  const double* a = A + b * nn;
  double* Wm = W + b * nn;
  double* Z = Zw + b * nn;
  for (int64_t i = tid; i < nn; i += bd) Wm[i] = a[i];
  __syncthreads();
  // ---- 1. tridiagonalisation (full symmetric trailing block, row k = column k)
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
        double acc = 0.0;
        for (int j = 0; j < m; ++j) acc = fma(B[(int64_t)j * n + r], v[j], acc);
        w[r] = tau * acc;
        vp += v[r] * w[r];
      }
      const double K = 0.5 * tau * block_sum(vp, red);
      for (int r = tid; r < m; r += bd) w[r] -= K * v[r];
      __syncthreads();
      for (int c = tid; c < m; c += bd) {
        const double vc = v[c], wc = w[c];
        for (int i = 0; i < m; ++i) {
          double* x = B + (int64_t)i * n + c;
          *x = fma(-v[i], wc, fma(-w[i], vc, *x));
        }
      }
    } else {
      if (tid == 0) e[k] = x0;
    }
    __syncthreads();
    // keep v (row k, right of the diagonal) and tau (on the diagonal) for phase 2
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
  }
  // ---- 2. Q = H_0 ... H_{n-3}, row-major in Z
  for (int64_t i = tid; i < nn; i += bd) Z[i] = (i / n == i % n) ? 1.0 : 0.0;
  __syncthreads();
  for (int k = n - 3; k >= 0; --k) {
    const double tau = Wm[(int64_t)k * n + k];
    if (tau == 0.0) continue;
    const int m = n - k - 1;
    for (int i = tid; i < m; i += bd) v[i] = Wm[(int64_t)k * n + k + 1 + i];
    __syncthreads();
    double* Zb = Z + (int64_t)(k + 1) * n + k + 1;
    for (int c = tid; c < m; c += bd) {
      double u = 0.0;
      for (int r = 0; r < m; ++r) u = fma(v[r], Zb[(int64_t)r * n + c], u);
      u *= tau;
      for (int r = 0; r < m; ++r) Zb[(int64_t)r * n + c] -= v[r] * u;
    }
    __syncthreads();
  }
  // column-major copy of Q into the (now free) reduction workspace
  for (int64_t i = tid; i < nn; i += bd) Wm[(i % n) * n + i / n] = Z[i];
  __syncthreads();
  double* Q = Wm;  // Q[col * n + row]
  // ---- 3. implicit QL
  if (tid == 0) ctl[2] = 0;
  for (int l = 0; l < n; ++l) {
    for (int iter = 0;; ++iter) {
      __syncthreads();  // every thread has read the previous round's ctl, rc, rs
      if (tid == 0) {
        int m = l;
        for (; m < n - 1; ++m) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= DBL_EPSILON * dd) break;
        }
        int nrot = 0;
        if (m != l && iter < 60) {
          double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
          double r = hypot(g, 1.0);
          g = d[m] - d[l] + e[l] / (g + copysign(r, g));
          double s = 1.0, c = 1.0, p = 0.0;
          bool split = false;
          for (int i = m - 1; i >= l; --i) {
            const double f = s * e[i], bb = c * e[i];
            // Givens rotation from one reciprocal square root (entries are
            // far from the FP64 overflow range, so no hypot scaling)
            const double rr = fma(f, f, g * g);
            if (rr == 0.0) {
              e[i + 1] = 0.0;
              d[i + 1] -= p;
              e[m] = 0.0;
              split = true;
              break;
            }
            const double rinv = rsqrt(rr);
            r = rr * rinv;
            e[i + 1] = r;
            s = f * rinv;
            c = g * rinv;
            g = d[i + 1] - p;
            r = (d[i] - g) * s + 2.0 * c * bb;
            p = s * r;
            d[i + 1] = g + p;
            g = c * r - bb;
            rc[nrot] = c;
            rs[nrot] = s;
            ++nrot;
          }
          if (!split) {
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
          }
        }
        if (m != l && iter >= 60) ctl[2] = 1;
        ctl[0] = m;
        ctl[1] = (m == l || iter >= 60) ? -1 : nrot;
      }
      __syncthreads();
      const int m = ctl[0], nrot = ctl[1];
      if (nrot < 0) break;
      // rotations on columns (i, i+1), i = m-1, m-2, ...: carry column i+1
      for (int r = tid; r < n; r += bd) {
        double x = Q[(int64_t)m * n + r];
        constexpr int PF = 8;  // columns fetched ahead of the carried rotation chain
        for (int j0 = 0; j0 < nrot; j0 += PF) {
          double z[PF];
#pragma unroll
          for (int t = 0; t < PF; ++t)
            z[t] = j0 + t < nrot ? Q[(int64_t)(m - 1 - j0 - t) * n + r] : 0.0;
#pragma unroll
          for (int t = 0; t < PF; ++t) {
            if (j0 + t < nrot) {
              const int i = m - 1 - j0 - t;
              const double c = rc[j0 + t], s = rs[j0 + t];
              Q[(int64_t)(i + 1) * n + r] = s * z[t] + c * x;
              x = c * z[t] - s * x;
            }
          }
        }
        if (nrot > 0) Q[(int64_t)(m - nrot) * n + r] = x;
      }
    }
  }
  __syncthreads();
  if (tid == 0 && ctl[2] && status) atomicOr(status, QSX_ERR_NONFINITE);
  // ---- ascending order: rank of each eigenvalue (ties by index)
  for (int i = tid; i < n; i += bd) {
    int rk = 0;
    const double di = d[i];
    for (int j = 0; j < n; ++j) rk += (d[j] < di) || (d[j] == di && j < i);
    rank[i] = rk;
  }
  __syncthreads();
  for (int i = tid; i < n; i += bd) E[b * n + rank[i]] = d[i];
  double* u = U + b * nn;
  for (int64_t idx = tid; idx < nn; idx += bd) {
    const int col = (int)(idx / n), row = (int)(idx % n);
    u[(int64_t)row * n + rank[col]] = Q[idx];
  }
}

}  // namespace qsx

using namespace qsx;

extern "C" size_t qsx_eigh_large_workspace_bytes(int n, int64_t batch) {
  if (n < 1 || batch < 0) return 0;
  return (size_t)2 * n * n * (size_t)batch * sizeof(double);
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
  const size_t smem = ((size_t)6 * n + 32) * sizeof(double) + ((size_t)4 + n) * sizeof(int);
  cudaError_t e = cudaFuncSetAttribute(eigh_tql_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "qsx_eigh_large_batched");
  double* W = (double*)workspace;
  double* Z = W + (size_t)n * n * batch;
  const int threads = n >= 1024 ? 1024 : ((n + 31) / 32) * 32;
  eigh_tql_kernel<<<(unsigned)batch, threads, smem, (cudaStream_t)stream>>>(H, n, W, Z, E, U,
                                                                            status);
  QSX_LAUNCH_CHECK("qsx_eigh_large_batched");
  return QSX_OK;
}

// Reverse-mode (adjoint) RK4 for ensemble-mean projected signals.
//
// Forward (qsx_rk4_batched, propagator form): per sample s
//   y_{k+1} = P_s y_k,  P_s = I + D_s,  x_n = scale * sum_s c^T y_{s,n}.
// This is the Heisenberg-picture linear response of linear_response /
// absorption_spectra (qspectra/simulate/response.py:15-43) averaged over the
// disorder ensemble (decorators.py:40-64).
//
// Given the cotangents g_n of x_n (PyTorch's convention for complex tensors:
// the gradient of a real loss is dL/dRe + i dL/dIm), the gradient with
// respect to D_s is
//   grad D_s = sum_{k=0}^{N-1} lam_{k+1} y_k^H,
//   lam_N = scale g_N conj(c),  lam_k = P_s^H lam_{k+1} + scale g_k conj(c),
// i.e. the adjoint state runs backward under P^H, the RK4 step of L^H.  The
// forward states are not stored: the caller passes checkpoints every K
// steps and each segment is recomputed into shared memory before its
// backward sweep.  One warp per sample, one lane per row (m <= 32), FP64.
#include "qsx_common.cuh"

namespace qsx {

struct AdjP {
  const double2* D;
  const double2* ck;   // [batch][nck][m]
  const double2* c;    // [m]
  const double2* g;    // [nsteps + 1]
  double2* gradD;      // [batch][m][m]
  double2* grady0;     // [batch][m] or null
  int m, nsteps, K, nck;
  int64_t batch;
  double scale;
};

__global__ void __launch_bounds__(128) rk4_adjoint_kernel(AdjP p) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int m = p.m, K = p.K;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t s = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  const size_t per_warp = (size_t)2 * m * m + (size_t)(K + 1) * m;
  double2* sD = (double2*)smraw + per_warp * warp;  // [m][m]
  double2* sG = sD + m * m;                          // [m][m] gradient rows
  double2* sY = sG + m * m;                          // [K + 1][m] segment states
  if (s >= p.batch) return;  // whole warp leaves together
  const double2* d = p.D + s * m * m;
  for (int e = lane; e < m * m; e += 32) {
    sD[e] = d[e];
    sG[e] = make_double2(0.0, 0.0);
  }
  __syncwarp();
  const bool row = lane < m;
  const double2 cc = row ? cconj(p.c[lane]) : make_double2(0.0, 0.0);
  double2 lam = cscale(cmul(p.g[p.nsteps], cc), p.scale);
  const int N = p.nsteps;
  const int nseg = (N + K - 1) / K;
  for (int seg = nseg - 1; seg >= 0; --seg) {
    const int k0 = seg * K, k1 = min(k0 + K, N);
    // recompute y_{k0} .. y_{k1-1} from the checkpoint at k0
    if (row) sY[lane] = p.ck[(s * p.nck + seg) * m + lane];
    __syncwarp();
    for (int k = k0; k < k1 - 1; ++k) {
      const double2* y = sY + (size_t)(k - k0) * m;
      if (row) {
        double2 acc = y[lane];
        const double2* dr = sD + lane * m;
        for (int j = 0; j < m; ++j) cfma(acc, dr[j], y[j]);
        sY[(size_t)(k + 1 - k0) * m + lane] = acc;
      }
      __syncwarp();
    }
    // backward sweep over the segment
    for (int k = k1 - 1; k >= k0; --k) {
      const double2* y = sY + (size_t)(k - k0) * m;
      if (row) {
        double2* gr = sG + lane * m;
        for (int j = 0; j < m; ++j) cfma(gr[j], lam, cconj(y[j]));
      }
      // lam_k = lam_{k+1} + D^H lam_{k+1} + scale g_k conj(c)
      double2 nl = lam;
      for (int j = 0; j < m; ++j) {
        const double lx = __shfl_sync(0xffffffffu, lam.x, j);
        const double ly = __shfl_sync(0xffffffffu, lam.y, j);
        if (row) cfma(nl, cconj(sD[j * m + lane]), make_double2(lx, ly));
      }
      lam = row ? cadd(nl, cscale(cmul(p.g[k], cc), p.scale)) : make_double2(0.0, 0.0);
    }
    __syncwarp();
  }
  double2* out = p.gradD + s * m * m;
  for (int e = lane; e < m * m; e += 32) out[e] = sG[e];
  if (p.grady0 && row) p.grady0[s * m + lane] = lam;
}

}  // namespace qsx

using namespace qsx;

extern "C" int qsx_rk4_adjoint_batched(const double* D, int m, int64_t batch, int nsteps,
                                       const double* checkpoints, int ck_every, int nck,
                                       const double* c, const double* g, double scale,
                                       double* gradD, double* grady0, void* stream) {
  QSX_CHECK_ARG(m >= 1 && m <= 32, "qsx_rk4_adjoint_batched: m=%d outside 1..32", m);
  QSX_CHECK_ARG(batch >= 0 && nsteps >= 0 && ck_every >= 1 && ck_every <= 1024,
                "qsx_rk4_adjoint_batched: bad batch, step count or checkpoint spacing");
  QSX_CHECK_ARG((int64_t)nck * ck_every >= nsteps && nck >= 1,
                "qsx_rk4_adjoint_batched: %d checkpoints every %d steps do not cover %d steps",
                nck, ck_every, nsteps);
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(D && checkpoints && c && g && gradD, "qsx_rk4_adjoint_batched: null pointer");
  AdjP p;
  p.D = (const double2*)D;
  p.ck = (const double2*)checkpoints;
  p.c = (const double2*)c;
  p.g = (const double2*)g;
  p.gradD = (double2*)gradD;
  p.grady0 = (double2*)grady0;
  p.m = m;
  p.nsteps = nsteps;
  p.K = ck_every;
  p.nck = nck;
  p.batch = batch;
  p.scale = scale;
  const size_t per_warp = ((size_t)2 * m * m + (size_t)(ck_every + 1) * m) * sizeof(double2);
  int warps = 4;
  while (warps > 1 && per_warp * warps > 96 * 1024) warps >>= 1;
  QSX_CHECK_ARG(per_warp <= 227 * 1024,
                "qsx_rk4_adjoint_batched: %zu bytes of segment state exceed shared memory",
                per_warp);
  const size_t smem = per_warp * warps;
  cudaError_t e = cudaFuncSetAttribute(rk4_adjoint_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_adjoint_batched");
  const unsigned grid = (unsigned)((batch + warps - 1) / warps);
  rk4_adjoint_kernel<<<grid, 32 * warps, smem, (cudaStream_t)stream>>>(p);
  QSX_LAUNCH_CHECK("qsx_rk4_adjoint_batched");
  return QSX_OK;
}

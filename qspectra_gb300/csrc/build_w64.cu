// FP64 eigendecomposition refinement and FP64 Redfield operators for
// one-exciton Hilbert spaces ('e' and 'ge', n_sites <= 8), one warp per
// disorder sample.
//
// This is the FP64 build of the precision form: the eigendecomposition of
// the rotating-frame Hamiltonian (hamiltonian.py:310-328) and the Redfield
// tensor in operator form (redfield.py:9-74) in FP64, feeding FP32
// propagation.  GB300 issues FP64 at a small fraction of its FP32 rate, so
// the kernel spends FP64 only where the result needs it:
//
// * Eigenpairs: Jacobi preconditioned in low precision (the mixed-precision
//   Jacobi of Higham, Tisseur, Webb and Zhou, 2024).  The FP32 register
//   Jacobi (eigh_block_kernel<float>) gives an approximate eigenbasis X; in
//   FP64, two Newton-Schulz steps X <- X + X (I - X^T X) / 2 make it
//   orthonormal, S = X^T A X is then diagonal up to the FP32 error, and
//   cyclic FP64 Jacobi sweeps on S (rotating X along) finish the job: one
//   sweep of small rotations, then a sweep that finds nothing to do.  Close
//   and equal eigenvalues need no special case (a rotation zeroes the pair
//   exactly), unlike a perturbative refinement.
// * Operators (site basis, non-secular): with the number-operator couplings
//   of one-exciton states, Kt_i[c][d] = X[i][c] X[i][d], so with
//   Y_i[a][c] = X[a][c] X[i][c] and C[c][d] = C(l_d - l_c)
//   (the closed-form Debye correlation of qsx_bath.cuh),
//     M_i = U (Kt_i o C) U^T = Y_i (C Y_i^T),  G = sum_i diag(occ_i) M_i
//   (row i of G is row i of M_i).  All N sites' products are spread over the
//   warp's lanes together (N n^2 outputs), so few lanes idle.
// Outputs have the layout of qsx_redfield_operators_batched (site basis):
// G [batch][n][n], M [batch][N][n][n] complex128 scaled by unit_convert,
// zero outside the coupled block, and E [batch][n], U [batch][n][n] with the
// eigenvalues ascending inside each block.
#include "qsx_bath.cuh"
#include "qsx_common.cuh"

namespace qsx {

constexpr int BW_WARPS = 4;

template <int NB>
struct BwSmem {
  double A[NB * NB];
  double X[NB * NB];
  double P[NB * NB];
  double S[NB * NB];
  double R[NB * NB];   // scratch
  double lam[NB];
  double2 C[NB * NB];
  double Y[NB * NB * NB];    // [i][a][c]
  double2 T[NB * NB * NB];   // [i][c][b]
};

// Classical Jacobi rotation zeroing a_pq (Golub & Van Loan, Alg. 8.4.1).
__device__ __forceinline__ void jacobi_rotation_f64(double app, double aqq, double apq, double& c,
                                                    double& s, double& t) {
  const double tau = (aqq - app) / (2.0 * apq);
  t = fabs(tau) < 1e100
          ? (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(fma(tau, tau, 1.0)))
          : 0.5 / tau;
  c = rsqrt(fma(t, t, 1.0));
  s = t * c;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int NB>
__global__ void __launch_bounds__(32 * BW_WARPS)
    redfield_build_w64_kernel(const double* __restrict__ H, int n, int off, int64_t batch,
                              const double* __restrict__ Uapprox, DebyeParams bath, double uc,
                              double* __restrict__ E, double* __restrict__ U,
                              double2* __restrict__ G, double2* __restrict__ M) {
  constexpr int NN = NB * NB;
  constexpr int NNN = NB * NB * NB;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  BwSmem<NB>& sm = reinterpret_cast<BwSmem<NB>*>(smraw)[w];
  const int64_t b = (int64_t)blockIdx.x * BW_WARPS + w;
  if (b >= batch) return;   // whole warps leave; no CTA barrier below
  const int nn = n * n;
  const double* h = H + b * nn;
  const double* u0 = Uapprox + b * nn;
  for (int e = lane; e < NN; e += 32) {
    const int r = e / NB, c = e % NB;
    sm.A[e] = h[(off + r) * n + off + c];
    sm.X[e] = u0[(off + r) * n + off + c];
  }
  __syncwarp();
  // ---- FP64 orthonormalisation of the FP32 basis: two Newton-Schulz steps
  // X <- X + X (I - X^T X) / 2 (each squares the orthogonality error)
  for (int it = 0; it < 2; ++it) {
    for (int e = lane; e < NN; e += 32) {   // R = I - X^T X
      const int i = e / NB, j = e % NB;
      double r = 0.0;
#pragma unroll
      for (int k = 0; k < NB; ++k) r = fma(sm.X[k * NB + i], sm.X[k * NB + j], r);
      sm.R[e] = (i == j ? 1.0 : 0.0) - r;
    }
    __syncwarp();
    for (int e = lane; e < NN; e += 32) {   // X + X R / 2, into P
      const int a = e / NB, j = e % NB;
      double acc = 0.0;
#pragma unroll
      for (int k = 0; k < NB; ++k) acc = fma(sm.X[a * NB + k], sm.R[k * NB + j], acc);
      sm.P[e] = fma(0.5, acc, sm.X[e]);
    }
    __syncwarp();
    for (int e = lane; e < NN; e += 32) sm.X[e] = sm.P[e];
    __syncwarp();
  }
  // ---- S = X^T A X (nearly diagonal), symmetrised ------------------------
  for (int e = lane; e < NN; e += 32) {
    const int r = e / NB, c = e % NB;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < NB; ++k) acc = fma(sm.A[r * NB + k], sm.X[k * NB + c], acc);
    sm.P[e] = acc;
  }
  __syncwarp();
  double asum = 0.0;
  for (int e = lane; e < NN; e += 32) {
    const int i = e / NB, j = e % NB;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < NB; ++k) acc = fma(sm.X[k * NB + i], sm.P[k * NB + j], acc);
    sm.R[e] = acc;
    asum = fma(sm.A[e], sm.A[e], asum);
  }
  asum = warp_sum(asum);
  __syncwarp();
  for (int e = lane; e < NN; e += 32) {
    const int i = e / NB, j = e % NB;
    sm.S[e] = 0.5 * (sm.R[e] + sm.R[j * NB + i]);
  }
  __syncwarp();
  // ---- cyclic FP64 Jacobi on S (Golub & Van Loan, Alg. 8.4.3), rotating the
  // columns of X too; one sweep normally zeroes every pair, the next finds
  // nothing above the tolerance.  Lane 0 forms each rotation, lane k < NB
  // updates row/column k of S and row k of X.
  const double tol = 1e-15 * sqrt(asum);
  for (int sweep = 0; sweep < 10; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < NB - 1; ++p)
      for (int q = p + 1; q < NB; ++q) {
        const double apq = sm.S[p * NB + q];
        if (!(fabs(apq) > tol)) continue;   // same value in every lane
        rotated = true;
        const double app = sm.S[p * NB + p], aqq = sm.S[q * NB + q];
        double c = 1.0, sn = 0.0, t = 0.0;
        if (lane == 0) jacobi_rotation_f64(app, aqq, apq, c, sn, t);
        c = __shfl_sync(0xffffffffu, c, 0);
        sn = __shfl_sync(0xffffffffu, sn, 0);
        t = __shfl_sync(0xffffffffu, t, 0);
        __syncwarp();
        if (lane < NB) {
          const int k = lane;
          if (k != p && k != q) {
            const double g = sm.S[k * NB + p], hh = sm.S[k * NB + q];
            const double np_ = c * g - sn * hh, nq = sn * g + c * hh;
            sm.S[k * NB + p] = np_;
            sm.S[p * NB + k] = np_;
            sm.S[k * NB + q] = nq;
            sm.S[q * NB + k] = nq;
          } else if (k == p) {
            sm.S[p * NB + p] = fma(-t, apq, app);
            sm.S[p * NB + q] = 0.0;
            sm.S[q * NB + p] = 0.0;
          } else {
            sm.S[q * NB + q] = fma(t, apq, aqq);
          }
          const double xp = sm.X[k * NB + p], xq = sm.X[k * NB + q];
          sm.X[k * NB + p] = c * xp - sn * xq;
          sm.X[k * NB + q] = sn * xp + c * xq;
        }
        __syncwarp();
      }
    if (!rotated) break;
  }
  if (lane < NB) sm.lam[lane] = sm.S[lane * NB + lane];
  __syncwarp();
  // ---- eigenpairs out, ascending inside the block (stable on ties) -------
  double* Eb = E + b * n;
  double* Ub = U + b * nn;
  for (int e = lane; e < nn; e += 32) {
    const int r = e / n, c = e % n;
    const bool inb = r >= off && r < off + NB && c >= off && c < off + NB;
    if (!inb) Ub[e] = (r == c) ? 1.0 : 0.0;   // the uncoupled 1 x 1 blocks
  }
  for (int i = lane; i < n; i += 32)
    if (i < off || i >= off + NB) Eb[i] = h[i * n + i];
  if (lane < NB) {
    const double li = sm.lam[lane];
    int rank = 0;
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const double lj = sm.lam[j];
      rank += (lj < li || (lj == li && j < lane)) ? 1 : 0;
    }
    Eb[off + rank] = li;
#pragma unroll
    for (int r = 0; r < NB; ++r) Ub[(off + r) * n + off + rank] = sm.X[r * NB + lane];
  }
  // ---- correlation function on the eigenvalue differences ----------------
  for (int e = lane; e < NN; e += 32) {
    const int c = e / NB, d = e % NB;
    if (c > d) continue;
    double2 cp, cn;
    debye_corr_pair(bath, sm.lam[d] - sm.lam[c], cp, cn);
    sm.C[c * NB + d] = cp;
    sm.C[d * NB + c] = cn;
  }
  // Y_i[a][c] = X[a][c] X[i][c]
  for (int e = lane; e < NNN; e += 32) {
    const int i = e / NN, a = (e / NB) % NB, c = e % NB;
    sm.Y[e] = sm.X[a * NB + c] * sm.X[i * NB + c];
  }
  __syncwarp();
  // T_i[c][b] = sum_d C[c][d] Y_i[b][d]
  for (int e = lane; e < NNN; e += 32) {
    const int i = e / NN, c = (e / NB) % NB, bb = e % NB;
    double2 acc = cmk(0.0, 0.0);
    const double* yi = sm.Y + i * NN + bb * NB;
#pragma unroll
    for (int d = 0; d < NB; ++d) {
      const double2 cv = sm.C[c * NB + d];
      const double y = yi[d];
      acc.x = fma(cv.x, y, acc.x);
      acc.y = fma(cv.y, y, acc.y);
    }
    sm.T[e] = acc;
  }
  __syncwarp();
  // M_i[a][b] = uc sum_c Y_i[a][c] T_i[c][b], straight to HBM; G row i = M_i row i
  const int nsites = NB;
  double2* Mb = M + b * (int64_t)nsites * nn;
  double2* Gb = G + b * nn;
  for (int e = lane; e < NNN; e += 32) {
    const int i = e / NN, a = (e / NB) % NB, bb = e % NB;
    double2 acc = cmk(0.0, 0.0);
    const double* yi = sm.Y + i * NN + a * NB;
    const double2* ti = sm.T + i * NN + bb;
#pragma unroll
    for (int c = 0; c < NB; ++c) {
      const double y = yi[c];
      const double2 t = ti[c * NB];
      acc.x = fma(y, t.x, acc.x);
      acc.y = fma(y, t.y, acc.y);
    }
    acc = cmk(acc.x * uc, acc.y * uc);
    Mb[(int64_t)i * nn + (off + a) * n + off + bb] = acc;
    if (a == i) Gb[(off + a) * n + off + bb] = acc;
  }
  // zeros outside the coupled block
  if (off > 0 || n > off + NB) {
    for (int e = lane; e < nn; e += 32) {
      const int r = e / n, c = e % n;
      if (r >= off && r < off + NB && c >= off && c < off + NB) continue;
      Gb[e] = cmk(0.0, 0.0);
      for (int i = 0; i < nsites; ++i) Mb[(int64_t)i * nn + e] = cmk(0.0, 0.0);
    }
  }
}

template <int NB>
static cudaError_t launch_bw(const double* H, int n, int off, int64_t batch, const double* Ua,
                             const DebyeParams& bath, double uc, double* E, double* U, double* G,
                             double* M, cudaStream_t s) {
  const size_t smem = sizeof(BwSmem<NB>) * BW_WARPS;
  cudaError_t e = cudaFuncSetAttribute(redfield_build_w64_kernel<NB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int64_t grid = (batch + BW_WARPS - 1) / BW_WARPS;
  redfield_build_w64_kernel<NB><<<(unsigned)grid, 32 * BW_WARPS, smem, s>>>(
      H, n, off, batch, Ua, bath, uc, E, U, (double2*)G, (double2*)M);
  return cudaGetLastError();
}

}  // namespace qsx

extern "C" int qsx_redfield_build_w64(const double* H, int n, int off, int n_sites,
                                      int64_t batch, const double* U_approx,
                                      double temperature, double reorg_energy,
                                      double cutoff_freq, int matsubara_cutoff,
                                      int discard_imag_corr, double unit_convert, double* E,
                                      double* U, double* G, double* M, void* stream) {
  using namespace qsx;
  QSX_CHECK_ARG(n_sites >= 2 && n_sites <= 8,
                "qsx_redfield_build_w64: n_sites must be 2..8 (got %d)", n_sites);
  QSX_CHECK_ARG(off >= 0 && off + n_sites <= n && n <= 32,
                "qsx_redfield_build_w64: the coupled block [%d, %d) must lie in n = %d <= 32",
                off, off + n_sites, n);
  QSX_CHECK_ARG(batch >= 0, "qsx_redfield_build_w64: negative batch");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(H && U_approx && E && U && G && M, "qsx_redfield_build_w64: null pointer");
  QSX_CHECK_ARG(temperature > 0 && cutoff_freq > 0 && matsubara_cutoff >= 1,
                "qsx_redfield_build_w64: bad bath parameters");
  const DebyeParams bath = make_debye(temperature, reorg_energy, cutoff_freq, matsubara_cutoff,
                                      discard_imag_corr);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaSuccess;
  switch (n_sites) {
    case 2: e = launch_bw<2>(H, n, off, batch, U_approx, bath, unit_convert, E, U, G, M, s); break;
    case 3: e = launch_bw<3>(H, n, off, batch, U_approx, bath, unit_convert, E, U, G, M, s); break;
    case 4: e = launch_bw<4>(H, n, off, batch, U_approx, bath, unit_convert, E, U, G, M, s); break;
    case 5: e = launch_bw<5>(H, n, off, batch, U_approx, bath, unit_convert, E, U, G, M, s); break;
    case 6: e = launch_bw<6>(H, n, off, batch, U_approx, bath, unit_convert, E, U, G, M, s); break;
    case 7: e = launch_bw<7>(H, n, off, batch, U_approx, bath, unit_convert, E, U, G, M, s); break;
    default: e = launch_bw<8>(H, n, off, batch, U_approx, bath, unit_convert, E, U, G, M, s); break;
  }
  if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_build_w64");
  return QSX_OK;
}

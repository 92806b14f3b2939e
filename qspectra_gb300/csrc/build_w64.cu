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
// * Eigenpairs: the FP32 register Jacobi (eigh_block_kernel<float>) gives an
//   approximate eigenbasis X; two steps of the symmetric eigenvalue
//   refinement of Ogita and Aishima (Japan J. Indust. Appl. Math. 35 (2018)
//   1007-1035, Algorithm 1) bring it to FP64 accuracy, each step one
//   quadratic improvement in orthogonality and diagonalisation, all lanes
//   busy:
//     R = I - X^T X,  S = X^T A X,  l_i = S_ii / (1 - R_ii),
//     F_ij = (S_ij + l_j R_ij) / (l_j - l_i)  for well-separated pairs,
//     F_ij = R_ij / 2 otherwise (and on the diagonal),  X <- X + X F.
//   From an FP32 start two steps reach FP64 only for gaps above ~1% of the
//   spectral radius, so closer pairs are treated as clusters (their common
//   subspace is refined, the pair itself is not).  The eigenvalues are the
//   diagonal of the final S = X^T A X; a pair still coupled there (a close
//   pair, a few percent of disorder samples) gets FP64 Jacobi rotations
//   inside its refined subspace (Golub & Van Loan, Alg. 8.4.3) on lane 0.
// * Correlation function: C(x) = lam gamma [(cot(gamma / 2T) - i) /
//   (gamma - i x) + 4 T S(x)] with the Matsubara sum S(x) from a piecewise
//   Chebyshev table (qsx_debye_matsubara_table, FP64 coefficients fitted to
//   the direct finite sum of bath.py:95-102), evaluated by Clenshaw's
//   recurrence in FP64; beyond the table the closed form of qsx_bath.cuh.
// * Operators (site basis, non-secular): with the number-operator couplings
//   of one-exciton states, Kt_i[c][d] = X[i][c] X[i][d], so with
//   Y_i[a][c] = X[a][c] X[i][c] and C[c][d] = C(l_d - l_c)
//   (the closed-form Debye correlation of qsx_bath.cuh),
//     M_i = U (Kt_i o C) U^T = Y_i (C Y_i^T),  G = sum_i diag(occ_i) M_i
//   (row i of G is row i of M_i).  All N sites' products are spread over the
//   warp's lanes together (N n^2 outputs), so few lanes idle.
// The file also holds the FP32 counterpart of the operator stage
// (redfield_operators_w32_kernel, below), for FP32 builds of the same spaces.
// Outputs have the layout of qsx_redfield_operators_batched (site basis):
// G [batch][n][n], M [batch][N][n][n] complex128 scaled by unit_convert,
// zero outside the coupled block, and E [batch][n], U [batch][n][n] with the
// eigenvalues ascending inside each block.
#include "qsx_bath.cuh"
#include "qsx_common.cuh"

namespace qsx {

constexpr int BW_WARPS = 4;
// pairs closer than this fraction of the largest |H| entry are clusters for
// the refinement steps (two steps from an FP32 start resolve wider gaps)
constexpr double BW_CLOSE = 1.5e-2;
constexpr int CHEB_DEG = 18;   // Chebyshev terms per table piece

// Piecewise Chebyshev table of the Matsubara sum S(x), x >= 0: piece j covers
// [j width, (j + 1) width) with CHEB_DEG complex coefficients (NULL: none).
struct ChebTable {
  const double2* coef;
  int pieces;
  double width;
};

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
                              const double* __restrict__ Uapprox, DebyeParams bath,
                              ChebTable ctab, double uc, double* __restrict__ E,
                              double* __restrict__ U, double2* __restrict__ G,
                              double2* __restrict__ M) {
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
  // ---- two refinement steps (Ogita-Aishima), close pairs as clusters ----
  double amax = 0.0;
  for (int e = lane; e < NN; e += 32) amax = fmax(amax, fabs(sm.A[e]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  const double close = BW_CLOSE * amax;
  for (int it = 0; it < 2; ++it) {
    for (int e = lane; e < NN; e += 32) {   // P = A X
      const int r = e / NB, c = e % NB;
      double acc = 0.0;
#pragma unroll
      for (int k = 0; k < NB; ++k) acc = fma(sm.A[r * NB + k], sm.X[k * NB + c], acc);
      sm.P[e] = acc;
    }
    __syncwarp();
    double nA = 0.0, nR = 0.0;
    for (int e = lane; e < NN; e += 32) {   // S = X^T P, R = I - X^T X
      const int i = e / NB, j = e % NB;
      double sv = 0.0, r = 0.0;
#pragma unroll
      for (int k = 0; k < NB; ++k) {
        const double xki = sm.X[k * NB + i];
        sv = fma(xki, sm.P[k * NB + j], sv);
        r = fma(xki, sm.X[k * NB + j], r);
      }
      r = (i == j ? 1.0 : 0.0) - r;
      sm.S[e] = sv;
      sm.R[e] = r;
      nA = fma(sm.A[e], sm.A[e], nA);
      nR = fma(r, r, nR);
    }
    __syncwarp();
    if (lane < NB) sm.lam[lane] = sm.S[lane * NB + lane] / (1.0 - sm.R[lane * NB + lane]);
    __syncwarp();
    double nS = 0.0;
    for (int e = lane; e < NN; e += 32) {
      const int i = e / NB, j = e % NB;
      const double d = sm.S[e] - (i == j ? sm.lam[i] : 0.0);
      nS = fma(d, d, nS);
    }
    nA = warp_sum(nA);
    nR = warp_sum(nR);
    nS = warp_sum(nS);
    const double thr = fmax(2.0 * (sqrt(nS) + sqrt(nA) * sqrt(nR)), close);
    for (int e = lane; e < NN; e += 32) {   // F, into P
      const int i = e / NB, j = e % NB;
      const double gap = sm.lam[j] - sm.lam[i];
      double f;
      if (i != j && fabs(gap) > thr)
        f = (sm.S[e] + sm.lam[j] * sm.R[e]) / gap;
      else
        f = 0.5 * sm.R[e];
      sm.P[e] = f;
    }
    __syncwarp();
    for (int e = lane; e < NN; e += 32) {   // X + X F, into S
      const int a = e / NB, j = e % NB;
      double acc = sm.X[e];
#pragma unroll
      for (int k = 0; k < NB; ++k) acc = fma(sm.X[a * NB + k], sm.P[k * NB + j], acc);
      sm.S[e] = acc;
    }
    __syncwarp();
    for (int e = lane; e < NN; e += 32) sm.X[e] = sm.S[e];
    __syncwarp();
  }
  // ---- final S = X^T A X; close pairs still coupled get Jacobi rotations --
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
  const double tol = 1e-15 * sqrt(asum);
  if (lane == 0) {
    for (int sweep = 0; sweep < 10; ++sweep) {
      bool rotated = false;
      for (int p = 0; p < NB - 1; ++p)
        for (int q = p + 1; q < NB; ++q) {
          const double apq = sm.S[p * NB + q];
          if (!(fabs(apq) > tol)) continue;
          rotated = true;
          double c, sn, t;
          jacobi_rotation_f64(sm.S[p * NB + p], sm.S[q * NB + q], apq, c, sn, t);
          sm.S[p * NB + p] = fma(-t, apq, sm.S[p * NB + p]);
          sm.S[q * NB + q] = fma(t, apq, sm.S[q * NB + q]);
          sm.S[p * NB + q] = sm.S[q * NB + p] = 0.0;
          for (int k = 0; k < NB; ++k) {
            if (k != p && k != q) {
              const double g = sm.S[k * NB + p], hh = sm.S[k * NB + q];
              sm.S[k * NB + p] = sm.S[p * NB + k] = c * g - sn * hh;
              sm.S[k * NB + q] = sm.S[q * NB + k] = sn * g + c * hh;
            }
            const double xp = sm.X[k * NB + p], xq = sm.X[k * NB + q];
            sm.X[k * NB + p] = c * xp - sn * xq;
            sm.X[k * NB + q] = sn * xp + c * xq;
          }
        }
      if (!rotated) break;
    }
  }
  __syncwarp();
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
    const double x = sm.lam[d] - sm.lam[c];
    const double ax = fabs(x);
    const int piece = (int)(ax / ctab.width);
    if (ctab.coef && !bath.real_only && x != 0.0 && piece < ctab.pieces) {
      // Clenshaw on the piece's Chebyshev series of S(|x|); S(-x) = conj S(x)
      const double2* cf = ctab.coef + (size_t)piece * CHEB_DEG;
      const double t = (ax - (piece + 0.5) * ctab.width) * (2.0 / ctab.width);
      const double t2 = 2.0 * t;
      double2 b1 = cmk(0.0, 0.0), b2 = cmk(0.0, 0.0);
      for (int k = CHEB_DEG - 1; k >= 1; --k) {
        const double2 ck = cf[k];
        const double2 b0 = cmk(fma(t2, b1.x, ck.x - b2.x), fma(t2, b1.y, ck.y - b2.y));
        b2 = b1;
        b1 = b0;
      }
      double2 Sx = cmk(fma(t, b1.x, cf[0].x - b2.x), fma(t, b1.y, cf[0].y - b2.y));
      if (x < 0.0) Sx = cconj(Sx);
      cp = debye_from_matsubara(bath, x, Sx);
      cn = debye_from_matsubara(bath, -x, cconj(Sx));
    } else {
      debye_corr_pair(bath, x, cp, cn);
    }
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
                             const DebyeParams& bath, const ChebTable& ctab, double uc, double* E,
                             double* U, double* G, double* M, cudaStream_t s) {
  const size_t smem = sizeof(BwSmem<NB>) * BW_WARPS;
  cudaError_t e = cudaFuncSetAttribute(redfield_build_w64_kernel<NB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int64_t grid = (batch + BW_WARPS - 1) / BW_WARPS;
  redfield_build_w64_kernel<NB><<<(unsigned)grid, 32 * BW_WARPS, smem, s>>>(
      H, n, off, batch, Ua, bath, ctab, uc, E, U, (double2*)G, (double2*)M);
  return cudaGetLastError();
}

// FP32 operator build for the same one-exciton, site-basis case, one warp
// per sample, from the FP32 eigendecomposition (E, U as stored by
// qsx_eigh_batched_prec): the closed-form FP32 correlation function on the
// eigenvalue differences (as redfield_operators_kernel<float>), then
// M_i = Y_i (C Y_i^T) and G row i = M_i row i, all N sites' products over
// the warp's lanes, with no block barrier.  Outputs as qsx_redfield_
// operators_batched (site basis), computed in FP32 and stored as complex128.
template <int NB>
struct Ow32Smem {
  float2 C[NB * NB];
  float2 T[NB * NB * NB];    // [i][c][b]
  float X[NB * NB];
  float lam[NB];
  float Y[NB * NB * NB];     // [i][a][c]
};

// float -> double from the IEEE 754 fields, exact: a normal number keeps
// its sign and fraction (widened by 29 bits) and re-biases its exponent
// (127 -> 1023); zeros, subnormals, infinities and NaNs take the hardware
// conversion.  Integer operations only, so the FP32 kernels that store
// complex128 results leave GB300's narrow FP64 pipe alone.
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const unsigned long long d = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(e + 896u) << 52) |
                               ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)d);
}

// The flat loops below visit e = lane, lane + 32, ... of an [NB][NB][NB]
// array as (i, a, b); 32 = DI NB^2 + DA NB + DB, so each step adds those
// with two carries instead of dividing.
template <int NB>
struct Flat3 {
  static constexpr int DB = 32 % NB, DA = (32 / NB) % NB, DI = 32 / (NB * NB);
  int i, a, b;
  __device__ __forceinline__ explicit Flat3(int e) : i(e / (NB * NB)), a((e / NB) % NB), b(e % NB) {}
  __device__ __forceinline__ void next() {
    b += DB;
    const int ca = b >= NB ? 1 : 0;
    b -= ca * NB;
    a += DA + ca;
    const int ci = a >= NB ? 1 : 0;
    a -= ci * NB;
    i += DI + ci;
  }
};

template <int NB>
__global__ void __launch_bounds__(32 * BW_WARPS)
    redfield_operators_w32_kernel(const double* __restrict__ E, const double* __restrict__ U,
                                  int n, int off, int64_t batch, DebyeF bath, float uc,
                                  double2* __restrict__ G, double2* __restrict__ M) {
  constexpr int NN = NB * NB;
  constexpr int NNN = NB * NB * NB;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Ow32Smem<NB>& sm = reinterpret_cast<Ow32Smem<NB>*>(smraw)[w];
  const int64_t b = (int64_t)blockIdx.x * BW_WARPS + w;
  if (b >= batch) return;   // whole warps leave; no CTA barrier below
  const int nn = n * n;
  const double* u = U + b * nn;
  for (int e = lane; e < NN; e += 32) {
    const int r = e / NB, c = e % NB;
    sm.X[e] = (float)u[(off + r) * n + off + c];
  }
  if (lane < NB) sm.lam[lane] = (float)E[b * n + off + lane];
  __syncwarp();
  // correlation function on the eigenvalue differences; (c, d) and (d, c)
  // share one evaluation
  for (int e = lane; e < NN; e += 32) {
    const int c = e / NB, d = e % NB;
    if (c > d) continue;
    float2 cp, cn;
    debye_corr_pair_f(bath, sm.lam[d] - sm.lam[c], cp, cn);
    sm.C[c * NB + d] = cp;
    sm.C[d * NB + c] = cn;
  }
  // Y_i[a][c] = X[a][c] X[i][c]
  {
    Flat3<NB> ix(lane);
    for (int e = lane; e < NNN; e += 32, ix.next())
      sm.Y[e] = sm.X[ix.a * NB + ix.b] * sm.X[ix.i * NB + ix.b];
  }
  __syncwarp();
  // T_i[c][b] = sum_d C[c][d] Y_i[b][d]
  {
    Flat3<NB> ix(lane);
    for (int e = lane; e < NNN; e += 32, ix.next()) {
      float2 acc = make_float2(0.f, 0.f);
      const float* yi = sm.Y + ix.i * NN + ix.b * NB;
      const float2* cr = sm.C + ix.a * NB;
#pragma unroll
      for (int d = 0; d < NB; ++d) {
        const float2 cv = cr[d];
        const float y = yi[d];
        acc.x = fmaf(cv.x, y, acc.x);
        acc.y = fmaf(cv.y, y, acc.y);
      }
      sm.T[e] = acc;
    }
  }
  __syncwarp();
  // M_i[a][b] = uc sum_c Y_i[a][c] T_i[c][b]; G row i = M_i row i
  double2* Mb = M + b * (int64_t)NB * nn;
  double2* Gb = G + b * nn;
  {
    Flat3<NB> ix(lane);
    for (int e = lane; e < NNN; e += 32, ix.next()) {
      float2 acc = make_float2(0.f, 0.f);
      const float* yi = sm.Y + ix.i * NN + ix.a * NB;
      const float2* ti = sm.T + ix.i * NN + ix.b;
#pragma unroll
      for (int c = 0; c < NB; ++c) {
        const float y = yi[c];
        const float2 t = ti[c * NB];
        acc.x = fmaf(y, t.x, acc.x);
        acc.y = fmaf(y, t.y, acc.y);
      }
      const double2 v = make_double2(f2d_exact(acc.x * uc), f2d_exact(acc.y * uc));
      Mb[(int64_t)ix.i * nn + (off + ix.a) * n + off + ix.b] = v;
      if (ix.a == ix.i) Gb[(off + ix.a) * n + off + ix.b] = v;
    }
  }
  // zeros outside the coupled block
  if (off > 0 || n > off + NB) {
    for (int e = lane; e < nn; e += 32) {
      const int r = e / n, c = e % n;
      if (r >= off && r < off + NB && c >= off && c < off + NB) continue;
      Gb[e] = make_double2(0.0, 0.0);
      for (int i = 0; i < NB; ++i) Mb[(int64_t)i * nn + e] = make_double2(0.0, 0.0);
    }
  }
}

template <int NB>
static cudaError_t launch_ow32(const double* E, const double* U, int n, int off, int64_t batch,
                               const DebyeParams& bath, double uc, double* G, double* M,
                               cudaStream_t s) {
  const size_t smem = sizeof(Ow32Smem<NB>) * BW_WARPS;
  const int64_t grid = (batch + BW_WARPS - 1) / BW_WARPS;
  redfield_operators_w32_kernel<NB><<<(unsigned)grid, 32 * BW_WARPS, smem, s>>>(
      E, U, n, off, batch, debye_f(bath), (float)uc, (double2*)G, (double2*)M);
  return cudaGetLastError();
}

}  // namespace qsx

// Host: Chebyshev coefficients of the Matsubara sum
//   S(x) = sum_{k=1}^{K-1} nu_k / ((nu_k^2 - gamma^2)(nu_k - i x)),
// nu_k = 2 pi k T (bath.py:95-102), on pieces [j w, (j + 1) w), x >= 0:
// CHEB_DEG values at the Chebyshev points of each piece, summed directly in
// FP64, then the discrete cosine transform.
extern "C" int qsx_debye_matsubara_table(double temperature, double cutoff_freq,
                                         int matsubara_cutoff, int pieces, double width,
                                         double* coef) {
  using namespace qsx;
  QSX_CHECK_ARG(temperature > 0 && cutoff_freq > 0 && matsubara_cutoff >= 1 && pieces >= 1 &&
                    width > 0 && coef,
                "qsx_debye_matsubara_table: bad arguments");
  const int D = CHEB_DEG;
  const double pi = 3.14159265358979323846;
  double fr[CHEB_DEG], fi[CHEB_DEG];
  for (int j = 0; j < pieces; ++j) {
    for (int q = 0; q < D; ++q) {
      const double th = pi * (q + 0.5) / D;
      const double x = (j + 0.5) * width + 0.5 * width * cos(th);
      double sr = 0.0, si = 0.0;
      for (int k = 1; k < matsubara_cutoff; ++k) {
        const double nu = 2.0 * pi * k * temperature;
        const double a = nu / (nu * nu - cutoff_freq * cutoff_freq);
        // a / (nu - i x) = a (nu + i x) / (nu^2 + x^2)
        const double den = nu * nu + x * x;
        sr += a * nu / den;
        si += a * x / den;
      }
      fr[q] = sr;
      fi[q] = si;
    }
    for (int m = 0; m < D; ++m) {
      double cr = 0.0, ci = 0.0;
      for (int q = 0; q < D; ++q) {
        const double w = cos(pi * m * (q + 0.5) / D);
        cr += fr[q] * w;
        ci += fi[q] * w;
      }
      const double scale = (m == 0 ? 1.0 : 2.0) / D;
      coef[2 * ((size_t)j * D + m)] = cr * scale;
      coef[2 * ((size_t)j * D + m) + 1] = ci * scale;
    }
  }
  return QSX_OK;
}

extern "C" int qsx_debye_matsubara_table_degree(void) { return qsx::CHEB_DEG; }

extern "C" int qsx_redfield_build_w64(const double* H, int n, int off, int n_sites,
                                      int64_t batch, const double* U_approx,
                                      double temperature, double reorg_energy,
                                      double cutoff_freq, int matsubara_cutoff,
                                      int discard_imag_corr, const double* corr_table,
                                      int corr_pieces, double corr_width, double unit_convert,
                                      double* E, double* U, double* G, double* M, void* stream) {
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
  QSX_CHECK_ARG(corr_table == nullptr || (corr_pieces >= 1 && corr_width > 0),
                "qsx_redfield_build_w64: bad correlation table");
  const DebyeParams bath = make_debye(temperature, reorg_energy, cutoff_freq, matsubara_cutoff,
                                      discard_imag_corr);
  ChebTable ctab;
  ctab.coef = (const double2*)corr_table;
  ctab.pieces = corr_table ? corr_pieces : 0;
  ctab.width = corr_table ? corr_width : 1.0;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaSuccess;
  switch (n_sites) {
    case 2: e = launch_bw<2>(H, n, off, batch, U_approx, bath, ctab, unit_convert, E, U, G, M, s); break;
    case 3: e = launch_bw<3>(H, n, off, batch, U_approx, bath, ctab, unit_convert, E, U, G, M, s); break;
    case 4: e = launch_bw<4>(H, n, off, batch, U_approx, bath, ctab, unit_convert, E, U, G, M, s); break;
    case 5: e = launch_bw<5>(H, n, off, batch, U_approx, bath, ctab, unit_convert, E, U, G, M, s); break;
    case 6: e = launch_bw<6>(H, n, off, batch, U_approx, bath, ctab, unit_convert, E, U, G, M, s); break;
    case 7: e = launch_bw<7>(H, n, off, batch, U_approx, bath, ctab, unit_convert, E, U, G, M, s); break;
    default: e = launch_bw<8>(H, n, off, batch, U_approx, bath, ctab, unit_convert, E, U, G, M, s); break;
  }
  if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_build_w64");
  return QSX_OK;
}

extern "C" int qsx_redfield_operators_w32(const double* E, const double* U, int n, int off,
                                          int n_sites, int64_t batch, double temperature,
                                          double reorg_energy, double cutoff_freq,
                                          int matsubara_cutoff, int discard_imag_corr,
                                          double unit_convert, double* G, double* M,
                                          void* stream) {
  using namespace qsx;
  QSX_CHECK_ARG(n_sites >= 2 && n_sites <= 8,
                "qsx_redfield_operators_w32: n_sites must be 2..8 (got %d)", n_sites);
  QSX_CHECK_ARG(off >= 0 && off + n_sites <= n && n <= 32,
                "qsx_redfield_operators_w32: the coupled block [%d, %d) must lie in n = %d <= 32",
                off, off + n_sites, n);
  QSX_CHECK_ARG(batch >= 0, "qsx_redfield_operators_w32: negative batch");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(E && U && G && M, "qsx_redfield_operators_w32: null pointer");
  QSX_CHECK_ARG(temperature > 0 && cutoff_freq > 0 && matsubara_cutoff >= 1,
                "qsx_redfield_operators_w32: bad bath parameters");
  const DebyeParams bath = make_debye(temperature, reorg_energy, cutoff_freq, matsubara_cutoff,
                                      discard_imag_corr);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaSuccess;
  switch (n_sites) {
    case 2: e = launch_ow32<2>(E, U, n, off, batch, bath, unit_convert, G, M, s); break;
    case 3: e = launch_ow32<3>(E, U, n, off, batch, bath, unit_convert, G, M, s); break;
    case 4: e = launch_ow32<4>(E, U, n, off, batch, bath, unit_convert, G, M, s); break;
    case 5: e = launch_ow32<5>(E, U, n, off, batch, bath, unit_convert, G, M, s); break;
    case 6: e = launch_ow32<6>(E, U, n, off, batch, bath, unit_convert, G, M, s); break;
    case 7: e = launch_ow32<7>(E, U, n, off, batch, bath, unit_convert, G, M, s); break;
    default: e = launch_ow32<8>(E, U, n, off, batch, bath, unit_convert, G, M, s); break;
  }
  if (e != cudaSuccess) return cuda_status(e, "qsx_redfield_operators_w32");
  return QSX_OK;
}

// Third-order response at large site counts: the two-exciton (f) manifold
// in operator form.
//
// The reference builds the dense Redfield tensor of the whole 'gef' space
// (qspectra/dynamics/redfield.py:9-74) and slices Liouville blocks out of it
// (liouville_space.py:316-341); at 24 sites that tensor has 301^4 entries.
// The generator is block-diagonal over manifolds, so the 'fe' block used by
// the excited-state-absorption pathways of third_order_response
// (qspectra/simulate/response.py:297-336) needs only the f-manifold
// operators M_i^f, the e-manifold operators M_i^e and the two Hamiltonians.
//
// Entry points (declared in include/qsx.h):
//   qsx_fblock_tensor        eigenbasis tensor Kt_i o C of the f manifold
//                            (redfield.py:41-69 restricted to one manifold)
//   qsx_fe_generator         Q_b = M_b^f - G^f - i uc H^f, the column
//                            operators of the 'fe' block
//   qsx_fe_heisenberg_rk4    RK4 on the transposed 'fe' block
//   qsx_csr_map_batched      sparse dipole super-operator maps between blocks
#include "qsx_bath.cuh"
#include "qsx_common.cuh"

namespace qsx {

// ------------------------------------------------------------------ f tensor
// Kt_i = U^T diag(occ_i) U over the pair states p = (k, l) (occ_i(p) = 1 when
// i is k or l), and Y_i[c][d] = uc * Kt_i[c][d] * C(E_d - E_c): the operator
// M_i^f = U Y_i U^T in the site basis (the same construction as the dense
// Redfield operators kernel, per manifold).  Output layout, per sample, is
// Y[c][plane][d] with planes 0..N-1 the real parts and N..2N-1 the imaginary
// parts, so that U @ Y and (U Y) @ U^T are two plain batched GEMMs.
constexpr int FT = 16;  // tile edge

template <typename T>
__global__ void __launch_bounds__(256)
    fblock_tensor_kernel(const double* __restrict__ E, const double* __restrict__ U, int P,
                         int N, const int* __restrict__ site_pairs, DebyeParams bath, double uc,
                         T* __restrict__ Y) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double* sUc = (double*)smraw;           // [P][FT]
  double* sUd = sUc + (size_t)P * FT;     // [P][FT]
  T* sMir = (T*)(sUd + (size_t)P * FT);   // [2][FT][FT + 1] mirror staging
  int* sPairs = (int*)(sMir + 2 * FT * (FT + 1));  // [N][N - 1]
  const int64_t s = blockIdx.y;
  // upper-triangular tile pair (tc <= td) from the linear block index
  const int ntile = (P + FT - 1) / FT;
  int t = blockIdx.x, tc = 0;
  while (t >= ntile - tc) {
    t -= ntile - tc;
    ++tc;
  }
  const int td = tc + t;
  const int c0 = tc * FT, d0 = td * FT;
  const double* u = U + s * (int64_t)P * P;
  for (int e = threadIdx.x; e < P * FT; e += blockDim.x) {
    const int p = e / FT, j = e % FT;
    sUc[e] = c0 + j < P ? u[(int64_t)p * P + c0 + j] : 0.0;
    sUd[e] = d0 + j < P ? u[(int64_t)p * P + d0 + j] : 0.0;
  }
  for (int e = threadIdx.x; e < N * (N - 1); e += blockDim.x) sPairs[e] = site_pairs[e];
  __syncthreads();
  const int r = threadIdx.x / FT, q = threadIdx.x % FT;
  const int c = c0 + r, d = d0 + q;
  const bool live = c < P && d < P;
  double2 cp = make_double2(0.0, 0.0), cn = cp;
  if (live) debye_corr_pair(bath, E[s * P + d] - E[s * P + c], cp, cn);
  const bool mirror = tc != td;
  T* y = Y + s * (int64_t)P * 2 * N * P;
  for (int i = 0; i < N; ++i) {
    double acc = 0.0;
    if (live) {
      const int* pi = sPairs + i * (N - 1);
      for (int j = 0; j < N - 1; ++j) {
        const int p = pi[j];
        acc = fma(sUc[p * FT + r], sUd[p * FT + q], acc);
      }
      acc *= uc;
      y[((int64_t)c * 2 * N + i) * P + d] = (T)(acc * cp.x);
      y[((int64_t)c * 2 * N + N + i) * P + d] = (T)(acc * cp.y);
    }
    if (mirror) {
      // Y_i[d][c] = acc * C(E_c - E_d): staged so the stores run along c
      sMir[r * (FT + 1) + q] = (T)(acc * cn.x);
      sMir[FT * (FT + 1) + r * (FT + 1) + q] = (T)(acc * cn.y);
      __syncthreads();
      const int dm = d0 + r, cm = c0 + q;
      if (dm < P && cm < P) {
        y[((int64_t)dm * 2 * N + i) * P + cm] = sMir[q * (FT + 1) + r];
        y[((int64_t)dm * 2 * N + N + i) * P + cm] = sMir[FT * (FT + 1) + q * (FT + 1) + r];
      }
      __syncthreads();
    }
  }
}

// --------------------------------------------------------------- fe generator
// Q[s][q][b][r] = M_b[q][r] - G[q][r] - i uc H[q][r], with M in the plane
// layout above and G = sum_i diag(occ_i) M_i, whose row q (pair (k, l)) is
// M_k[q] + M_l[q].
template <typename T>
__global__ void fe_generator_kernel(const T* __restrict__ M, const double* __restrict__ H,
                                    int P, int N, int64_t batch,
                                    const int* __restrict__ pair_sites, double uc,
                                    typename cplx<T>::type* __restrict__ Q) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= batch * P * P) return;
  const int64_t s = e / ((int64_t)P * P);
  const int q = (int)((e / P) % P), r = (int)(e % P);
  const T* m = M + (s * P + q) * (int64_t)2 * N * P;
  const int k = pair_sites[2 * q], l = pair_sites[2 * q + 1];
  const T gx = m[(int64_t)k * P + r] + m[(int64_t)l * P + r];
  const T gy = m[(int64_t)(N + k) * P + r] + m[(int64_t)(N + l) * P + r];
  const T hy = (T)(uc * H[s * (int64_t)P * P + (int64_t)q * P + r]);
  typename cplx<T>::type* out = Q + (s * P + q) * (int64_t)N * P + r;
  for (int b = 0; b < N; ++b)
    out[(int64_t)b * P] = cmk(m[(int64_t)b * P + r] - gx, m[(int64_t)(N + b) * P + r] - gy - hy);
}

// ------------------------------------------------------------- fe RK4 stage
// The 'fe' block acts on X (P x N: rows pair states, columns e sites; the
// column-stacked vector of the block is X column-major) as
//   (L X)[:, b] = Q_b X[:, b] + row terms,  (L X)[p, :] += X[p, :] R_p^T,
// Q_b = M_b^f - A_f, R_p = conj(M_k^e + M_l^e - A_e) for p = (k, l),
// A = G + i uc H (operator form of the site-basis Redfield generator:
// dX = -A X - X A^+ + sum_i (M_i X K_i + K_i X M_i^+)).  Its plain
// transpose, the Heisenberg-picture generator, is
//   (L^T X)[:, b] = Q_b^T X[:, b] + sum_c X[:, c] R_p[c][b]  (row p),
// so column b reads Q_b[q][r] along r: coalesced in the layout Q[s][q][b][r].
// One CTA per (column b, sample), one thread per row; Q is streamed once per
// stage (the kernel's HBM traffic), X column b and the row operators sit in
// shared memory.
struct FeP {
  int P, N;
  const void* Q;          // [batch][P][N][P] complex (T)
  const void* Ae;         // [batch][N][N] complex (T)
  const void* Me;         // [batch][N][N][N] complex (T): Me[i][c][b]
  const int* pair_sites;  // [P][2]
  double h;
};

constexpr int FE_THREADS = 320;

template <typename T>
__global__ void __launch_bounds__(FE_THREADS, sizeof(T) == 4 ? 4 : 2)
    fe_stage_kernel(FeP p, int stage, const typename cplx<T>::type* in,
                    typename cplx<T>::type* yh, typename cplx<T>::type* yl,
                    typename cplx<T>::type* acc, typename cplx<T>::type* next) {
  using C = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int P = p.P, N = p.N;
  const int b = blockIdx.x;
  const int64_t s = blockIdx.y;
  // shared: column b of X (the column term) and the row operators for
  // column b; each thread reads its own row of X from global memory
  C* sxb = (C*)smraw;          // [P]
  C* sR = sxb + P;             // [N][N]: conj(Me[i][c][b] - Ae[c][b] / 2)
  const int64_t per = (int64_t)P * N;
  const C* x = in + s * per;
  for (int i = threadIdx.x; i < P; i += blockDim.x) sxb[i] = x[(int64_t)b * P + i];
  const C* me = (const C*)p.Me + s * (int64_t)N * N * N;
  const C* ae = (const C*)p.Ae + s * (int64_t)N * N;
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
    const int site = i / N, c = i % N;
    const C m = me[((int64_t)site * N + c) * N + b];
    const C a = ae[(int64_t)c * N + b];
    sR[i] = cmk(m.x - (T)0.5 * a.x, -(m.y - (T)0.5 * a.y));
  }
  __syncthreads();
  for (int row = threadIdx.x; row < P; row += blockDim.x) {
  const C* __restrict__ qcol = (const C*)p.Q + (s * P * N + b) * (int64_t)P + row;
  const int64_t qstride = (int64_t)N * P;
  C k0 = cmk((T)0, (T)0), k1 = k0, k2 = k0, k3 = k0;
  // column term sum_q Q_b[q][row] X[q][b], software-pipelined: the next
  // U rows of Q are in flight while the current U are consumed
  constexpr int U = 4;
  C a[U], nx[U];
  int q = 0;
  if (P >= U) {
#pragma unroll
    for (int t = 0; t < U; ++t) a[t] = __ldg(qcol + (int64_t)t * qstride);
    for (; q + 2 * U <= P; q += U) {
#pragma unroll
      for (int t = 0; t < U; ++t) nx[t] = __ldg(qcol + (int64_t)(q + U + t) * qstride);
#pragma unroll
      for (int t = 0; t < U; t += 4) {
        cfma(k0, a[t], sxb[q + t]);
        cfma(k1, a[t + 1], sxb[q + t + 1]);
        cfma(k2, a[t + 2], sxb[q + t + 2]);
        cfma(k3, a[t + 3], sxb[q + t + 3]);
      }
#pragma unroll
      for (int t = 0; t < U; ++t) a[t] = nx[t];
    }
#pragma unroll
    for (int t = 0; t < U; t += 4) {
      cfma(k0, a[t], sxb[q + t]);
      cfma(k1, a[t + 1], sxb[q + t + 1]);
      cfma(k2, a[t + 2], sxb[q + t + 2]);
      cfma(k3, a[t + 3], sxb[q + t + 3]);
    }
    q += U;
  }
  for (; q < P; ++q) cfma(k0, __ldg(qcol + (int64_t)q * qstride), sxb[q]);
  // row term sum_c X[row][c] (T_k + T_l)[c]
  const int kk = p.pair_sites[2 * row], ll = p.pair_sites[2 * row + 1];
  const C* xr = x + row;
  for (int c = 0; c < N; ++c) {
    const C ra = sR[kk * N + c], rb = sR[ll * N + c];
    cfma(k1, xr[(int64_t)c * P], cmk(ra.x + rb.x, ra.y + rb.y));
  }
  const C k = cmk(k0.x + k1.x + k2.x + k3.x, k0.y + k1.y + k2.y + k3.y);
  const int64_t idx = s * per + (int64_t)b * P + row;
  const T h = (T)p.h;
  if (stage == 0) {
    acc[idx] = k;
    const C y = yh[idx];
    next[idx] = cmk(y.x + (T)0.5 * h * k.x, y.y + (T)0.5 * h * k.y);
  } else if (stage < 3) {
    const C a0 = acc[idx];
    acc[idx] = cmk(a0.x + (T)2 * k.x, a0.y + (T)2 * k.y);
    const C y = yh[idx];
    const T cst = stage == 1 ? (T)0.5 * h : h;
    next[idx] = cmk(y.x + cst * k.x, y.y + cst * k.y);
  } else {
    const C a0 = acc[idx];
    const T s6 = h / (T)6;
    const T ix = s6 * (a0.x + k.x), iy = s6 * (a0.y + k.y);
    const C y = yh[idx];
    if (yl) {
      // split-word state: hi + lo with a TwoSum update
      const C l = yl[idx];
      float hx = (float)y.x, lx = (float)l.x, hy = (float)y.y, ly = (float)l.y;
      dd_add(hx, lx, (float)ix);
      dd_add(hy, ly, (float)iy);
      yh[idx] = cmk((T)hx, (T)hy);
      yl[idx] = cmk((T)lx, (T)ly);
    } else {
      yh[idx] = cmk(y.x + ix, y.y + iy);
    }
  }
  }
}

template <typename T>
__global__ void fe_init_kernel(const double2* __restrict__ y0, int64_t y0_stride, int64_t per,
                               int64_t batch, typename cplx<T>::type* yh,
                               typename cplx<T>::type* yl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per * batch) return;
  const double2 v = y0[(i / per) * y0_stride + i % per];
  yh[i] = cmk((T)v.x, (T)v.y);
  if (yl) yl[i] = cmk((T)(v.x - (double)(T)v.x), (T)(v.y - (double)(T)v.y));
}

template <typename T>
__global__ void fe_save_kernel(const typename cplx<T>::type* __restrict__ yh,
                               const typename cplx<T>::type* __restrict__ yl, int64_t per,
                               int64_t batch, int k, int nsave, double2* __restrict__ out,
                               int* status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per * batch) return;
  const int64_t s = i / per, e = i % per;
  double vx = (double)yh[i].x, vy = (double)yh[i].y;
  if (yl) {
    vx += (double)yl[i].x;
    vy += (double)yl[i].y;
  }
  if (status && !(isfinite(vx) && isfinite(vy))) atomicOr(status, QSX_ERR_NONFINITE);
  out[(s * nsave + k) * per + e] = make_double2(vx, vy);
}

// ------------------------------------------------------------------ CSR map
// out[b][r] = sum_k vals[k] in[b][cols[k]] over rowptr[r] <= k < rowptr[r+1].
__global__ void csr_map_kernel(const double2* __restrict__ in, int64_t n_in, int64_t batch,
                               const int* __restrict__ rowptr, const int* __restrict__ cols,
                               const double2* __restrict__ vals, int n_out,
                               double2* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= batch * n_out) return;
  const int64_t b = e / n_out;
  const int r = (int)(e % n_out);
  const double2* x = in + b * n_in;
  double2 acc = make_double2(0.0, 0.0);
  for (int k = rowptr[r]; k < rowptr[r + 1]; ++k) {
    const double2 v = vals[k], xv = x[cols[k]];
    acc.x = fma(v.x, xv.x, fma(-v.y, xv.y, acc.x));
    acc.y = fma(v.x, xv.y, fma(v.y, xv.x, acc.y));
  }
  out[e] = acc;
}

}  // namespace qsx

using namespace qsx;

extern "C" int qsx_fblock_tensor(const double* E, const double* U, int P, int N,
                                 const int* site_pairs, int64_t batch, double temperature,
                                 double reorg_energy, double cutoff_freq, int matsubara_cutoff,
                                 int discard_imag_corr, double unit_convert, int precision,
                                 void* Y, void* stream) {
  QSX_CHECK_ARG(N >= 2 && N <= 64 && P == N * (N - 1) / 2,
                "qsx_fblock_tensor: P=%d must be N(N-1)/2 for N=%d sites", P, N);
  QSX_CHECK_ARG(batch >= 0 && batch <= 65535, "qsx_fblock_tensor: batch out of range");
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_fblock_tensor: bad precision");
  QSX_CHECK_ARG(temperature > 0 && cutoff_freq > 0 && matsubara_cutoff >= 1,
                "qsx_fblock_tensor: bad bath parameters");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(E && U && site_pairs && Y, "qsx_fblock_tensor: null pointer");
  const DebyeParams bath = make_debye(temperature, reorg_energy, cutoff_freq, matsubara_cutoff,
                                      discard_imag_corr != 0);
  const int ntile = (P + FT - 1) / FT;
  const dim3 grid((unsigned)(ntile * (ntile + 1) / 2), (unsigned)batch);
  cudaStream_t s = (cudaStream_t)stream;
  auto run = [&](auto tag) -> int {
    using T = decltype(tag);
    const size_t smem = 2 * (size_t)P * FT * sizeof(double) + 2 * FT * (FT + 1) * sizeof(T) +
                        (size_t)N * (N - 1) * sizeof(int);
    QSX_CHECK_ARG(smem <= 227 * 1024, "qsx_fblock_tensor: %d pair states exceed shared memory",
                  P);
    cudaError_t e = cudaFuncSetAttribute(fblock_tensor_kernel<T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_fblock_tensor");
    fblock_tensor_kernel<T><<<grid, FT * FT, smem, s>>>(E, U, P, N, site_pairs, bath,
                                                        unit_convert, (T*)Y);
    QSX_LAUNCH_CHECK("qsx_fblock_tensor");
    return QSX_OK;
  };
  return precision == QSX_FP32 ? run(0.0f) : run(0.0);
}

extern "C" int qsx_fe_generator(const void* M, const double* H, int P, int N, int64_t batch,
                                const int* pair_sites, double unit_convert, int precision,
                                void* Q, void* stream) {
  QSX_CHECK_ARG(N >= 2 && N <= 64 && P == N * (N - 1) / 2,
                "qsx_fe_generator: P=%d must be N(N-1)/2 for N=%d sites", P, N);
  QSX_CHECK_ARG(batch >= 0, "qsx_fe_generator: negative batch");
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_fe_generator: bad precision");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(M && H && pair_sites && Q, "qsx_fe_generator: null pointer");
  const int64_t n = batch * P * P;
  const unsigned grid = (unsigned)((n + 255) / 256);
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == QSX_FP32)
    fe_generator_kernel<float><<<grid, 256, 0, s>>>((const float*)M, H, P, N, batch, pair_sites,
                                                    unit_convert, (float2*)Q);
  else
    fe_generator_kernel<double><<<grid, 256, 0, s>>>((const double*)M, H, P, N, batch,
                                                     pair_sites, unit_convert, (double2*)Q);
  QSX_LAUNCH_CHECK("qsx_fe_generator");
  return QSX_OK;
}

extern "C" size_t qsx_fe_heisenberg_workspace_bytes(int P, int N, int64_t batch, int precision) {
  if (P < 1 || N < 1 || batch < 0) return 0;
  const size_t cs = precision == QSX_FP32 ? sizeof(float2) : sizeof(double2);
  const size_t n = (size_t)P * N * (size_t)batch;
  return (precision == QSX_FP32 ? 5 : 4) * n * cs;
}

extern "C" int qsx_fe_heisenberg_rk4(const void* Q, const void* Ae, const void* Me,
                                     const int* pair_sites, int P, int N, int64_t batch,
                                     int precision, const double* y0, int64_t y0_stride,
                                     int nsteps, double h, double* out, void* workspace,
                                     size_t workspace_bytes, int32_t* status, void* stream) {
  QSX_CHECK_ARG(N >= 2 && N <= 64 && P == N * (N - 1) / 2,
                "qsx_fe_heisenberg_rk4: P=%d must be N(N-1)/2 for N=%d sites", P, N);
  QSX_CHECK_ARG(batch >= 0 && batch <= 65535 && nsteps >= 0,
                "qsx_fe_heisenberg_rk4: batch or step count out of range");
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_fe_heisenberg_rk4: bad precision");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(Q && Ae && Me && pair_sites && y0 && out && status,
                "qsx_fe_heisenberg_rk4: null pointer");
  const size_t need = qsx_fe_heisenberg_workspace_bytes(P, N, batch, precision);
  QSX_CHECK_ARG(workspace && workspace_bytes >= need,
                "qsx_fe_heisenberg_rk4: workspace of %zu bytes needed (got %zu)", need,
                workspace_bytes);
  cudaStream_t s = (cudaStream_t)stream;
  FeP p;
  p.P = P;
  p.N = N;
  p.Q = Q;
  p.Ae = Ae;
  p.Me = Me;
  p.pair_sites = pair_sites;
  p.h = h;
  const int64_t per = (int64_t)P * N;
  const int64_t n = per * batch;
  const dim3 grid((unsigned)N, (unsigned)batch);
  const int threads = P >= FE_THREADS ? FE_THREADS : ((P + 31) / 32) * 32;
  const unsigned eg = (unsigned)((n + 255) / 256);
  auto run = [&](auto tag) -> int {
    using T = decltype(tag);
    using C = typename cplx<T>::type;
    C* yh = (C*)workspace;
    C* yl = sizeof(T) == 4 ? yh + n : nullptr;
    C* acc = yh + (sizeof(T) == 4 ? 2 : 1) * n;
    C* s0 = acc + n;
    C* s1 = s0 + n;
    const size_t smem = ((size_t)P + (size_t)N * N) * sizeof(C);
    QSX_CHECK_ARG(smem <= 227 * 1024,
                  "qsx_fe_heisenberg_rk4: %zu bytes of column state exceed shared memory", smem);
    cudaError_t e = cudaFuncSetAttribute(fe_stage_kernel<T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_fe_heisenberg_rk4");
    fe_init_kernel<T><<<eg, 256, 0, s>>>((const double2*)y0, y0_stride, per, batch, yh, yl);
    fe_save_kernel<T><<<eg, 256, 0, s>>>(yh, yl, per, batch, 0, nsteps + 1, (double2*)out,
                                        status);
    for (int step = 1; step <= nsteps; ++step) {
      fe_stage_kernel<T><<<grid, threads, smem, s>>>(p, 0, yh, yh, yl, acc, s0);
      fe_stage_kernel<T><<<grid, threads, smem, s>>>(p, 1, s0, yh, yl, acc, s1);
      fe_stage_kernel<T><<<grid, threads, smem, s>>>(p, 2, s1, yh, yl, acc, s0);
      fe_stage_kernel<T><<<grid, threads, smem, s>>>(p, 3, s0, yh, yl, acc, nullptr);
      fe_save_kernel<T><<<eg, 256, 0, s>>>(yh, yl, per, batch, step, nsteps + 1,
                                          (double2*)out, status);
    }
    QSX_LAUNCH_CHECK("qsx_fe_heisenberg_rk4");
    return QSX_OK;
  };
  return precision == QSX_FP32 ? run(0.0f) : run(0.0);
}

extern "C" int qsx_csr_map_batched(const double* in, int64_t n_in, int64_t batch,
                                   const int* rowptr, const int* cols, const double* vals,
                                   int n_out, double* out, void* stream) {
  QSX_CHECK_ARG(n_in >= 1 && n_out >= 1 && batch >= 0, "qsx_csr_map_batched: bad sizes");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(in && rowptr && cols && vals && out, "qsx_csr_map_batched: null pointer");
  const int64_t n = batch * n_out;
  csr_map_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      (const double2*)in, n_in, batch, rowptr, cols, (const double2*)vals, n_out,
      (double2*)out);
  QSX_LAUNCH_CHECK("qsx_csr_map_batched");
  return QSX_OK;
}

// Direct DFT of uniformly sampled signals at arbitrary frequencies (FP64),
// replacing fourier_transform (qspectra/simulate/utils.py:154-219).
//
// The reference zero-pads to a symmetric time grid and runs an FFT; padded
// zeros contribute nothing, so on the FFT frequency grid the result equals
//   X(f) = dt * sum_n x_n exp(i * sign * (f - rw) * uc * t_n)
// which this kernel evaluates directly (any grid, e.g. 1024 points in a
// window).  The twiddle e^{i n Δ} advances by complex rotation and is
// re-seeded from sincos every 32 samples to bound drift.
#include "qsx_common.cuh"

namespace qsx {

// grid (ceil(nf / 8), batch), 256 threads: 8 frequencies per CTA, the time
// samples split into 32 slices, partial sums meet in shared memory (fixed
// order).
__global__ void __launch_bounds__(256)
    dft_kernel(const double2* __restrict__ x, int nt, double t0, double dt,
               const double* __restrict__ freqs, int nf, double rw, double uc, int sign,
               double2* __restrict__ X) {
  // 8 frequencies per CTA, each summed over 32 time slices (lane / 8 and the
  // warp pick the slice), so a spectrum of ~1000 points spreads over ~128
  // SMs; the slices are added in a fixed order
  __shared__ double2 part[32][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int kl = lane & 7, slice = w * 4 + (lane >> 3);
  const int64_t b = blockIdx.y;
  const int k = blockIdx.x * 8 + kl;
  const double wk = k < nf ? (double)sign * (freqs[k] - rw) * uc : 0.0;
  double sd, cd;
  sincos(wk * dt, &sd, &cd);
  const int chunk = (nt + 31) / 32;
  const int n0 = slice * chunk, n1 = min(nt, n0 + chunk);
  const double2* xb = x + b * nt;
  double2 acc = make_double2(0.0, 0.0);
  double2 ph = make_double2(1.0, 0.0);
  for (int n = n0; n < n1; ++n) {
    if (((n - n0) & 31) == 0) {   // re-anchor the rotation every 32 steps
      double s, c;
      sincos(wk * (t0 + (double)n * dt), &s, &c);
      ph = make_double2(c, s);
    }
    cfma(acc, __ldg(&xb[n]), ph);
    ph = make_double2(ph.x * cd - ph.y * sd, ph.x * sd + ph.y * cd);
  }
  part[slice][kl] = acc;
  __syncthreads();
  if (threadIdx.x < 8 && k < nf) {
    double2 t = part[0][kl];
#pragma unroll
    for (int i = 1; i < 32; ++i) t = cadd(t, part[i][kl]);
    X[b * nf + k] = cscale(t, dt);
  }
}

// The same sum for signals that come from FP32 propagation: the phase is
// anchored in FP64 at the start of each time slice (one sincos a thread),
// then rotated and accumulated in FP32 over the slice (at most 128 samples,
// a relative drift of order 1e-5 at worst), with the slices added in FP64.
// The signal is read once per CTA and converted to FP32 in shared memory, so
// the inner loop issues no FP64 work.
__global__ void __launch_bounds__(256)
    dft_f32_kernel(const double2* __restrict__ x, int nt, double t0, double dt,
                   const double* __restrict__ freqs, int nf, double rw, double uc, int sign,
                   double2* __restrict__ X) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* sx = reinterpret_cast<float2*>(smraw);   // [nt]
  __shared__ double2 part[32][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int kl = lane & 7, slice = w * 4 + (lane >> 3);
  const int64_t b = blockIdx.y;
  const int k = blockIdx.x * 8 + kl;
  const double2* xb = x + b * nt;
  for (int n = threadIdx.x; n < nt; n += blockDim.x) {
    const double2 v = xb[n];
    sx[n] = make_float2((float)v.x, (float)v.y);
  }
  __syncthreads();
  const double wk = k < nf ? (double)sign * (freqs[k] - rw) * uc : 0.0;
  double sd, cd;
  sincos(wk * dt, &sd, &cd);
  const float sdf = (float)sd, cdf = (float)cd;
  const int chunk = (nt + 31) / 32;
  const int n0 = slice * chunk, n1 = min(nt, n0 + chunk);
  double2 acc = make_double2(0.0, 0.0);
  float2 ph = make_float2(1.f, 0.f), a32 = make_float2(0.f, 0.f);
  for (int n = n0; n < n1; ++n) {
    if (((n - n0) & 127) == 0) {   // FP64 anchor (at most every 128 samples)
      acc.x += (double)a32.x;
      acc.y += (double)a32.y;
      a32 = make_float2(0.f, 0.f);
      double s, c;
      sincos(wk * (t0 + (double)n * dt), &s, &c);
      ph = make_float2((float)c, (float)s);
    }
    const float2 v = sx[n];
    a32.x = fmaf(v.x, ph.x, fmaf(-v.y, ph.y, a32.x));
    a32.y = fmaf(v.x, ph.y, fmaf(v.y, ph.x, a32.y));
    ph = make_float2(ph.x * cdf - ph.y * sdf, ph.x * sdf + ph.y * cdf);
  }
  acc.x += (double)a32.x;
  acc.y += (double)a32.y;
  part[slice][kl] = acc;
  __syncthreads();
  if (threadIdx.x < 8 && k < nf) {
    double2 t = part[0][kl];
#pragma unroll
    for (int i = 1; i < 32; ++i) t = cadd(t, part[i][kl]);
    X[b * nf + k] = cscale(t, dt);
  }
}

// Two-dimensional transform of a third-order signal x[n1][b][n3] (t1, t2,
// t3; any strides) over t1 and t3 in one launch (FP64):
//   X[k1][b][k3] = dt1 dt3 sum_{n1, n3} x[n1][b][n3]
//                  exp(i s1 (f1_k1 - rw) uc t1_n1) exp(i s3 (f3_k3 - rw) uc t3_n3),
// t_n = t0 + n dt on each axis.  CTA (chunk of 8 t3 frequencies, b): first the
// t3 transform of every t1 row for those frequencies, into shared memory
// (Y[n1][8]); then the t1 transform of Y for every t1 frequency.  Each sum
// advances its twiddle by complex rotation, re-seeded from sincos every 32
// samples, as dft_kernel does.
constexpr int DFT2_F3 = 8;

__global__ void __launch_bounds__(256)
    dft2_kernel(const double2* __restrict__ x, int n1, int n3, int64_t s1, int64_t sb,
                int64_t s3, double t01, double dt1, const double* __restrict__ f1, int nf1,
                int sign1, double t03, double dt3, const double* __restrict__ f3, int nf3,
                int sign3, double rw, double uc, double2* __restrict__ X) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double2* Y = reinterpret_cast<double2*>(smraw);   // [n1][DFT2_F3]
  const int k3base = blockIdx.x * DFT2_F3;
  const int64_t b = blockIdx.y;
  const int64_t nb = gridDim.y;
  const double2* xb = x + b * sb;
  // t3 transform: one (n1, k3) sum a thread
  for (int o = threadIdx.x; o < n1 * DFT2_F3; o += blockDim.x) {
    const int r = o / DFT2_F3, kl = o % DFT2_F3, k = k3base + kl;
    double2 acc = make_double2(0.0, 0.0);
    if (k < nf3) {
      const double wk = (double)sign3 * (f3[k] - rw) * uc;
      double sd, cd;
      sincos(wk * dt3, &sd, &cd);
      const double2* xr = xb + (int64_t)r * s1;
      double2 ph = make_double2(1.0, 0.0);
      for (int n = 0; n < n3; ++n) {
        if ((n & 31) == 0) {
          double sn, cn;
          sincos(wk * (t03 + (double)n * dt3), &sn, &cn);
          ph = make_double2(cn, sn);
        }
        cfma(acc, xr[(int64_t)n * s3], ph);
        ph = make_double2(ph.x * cd - ph.y * sd, ph.x * sd + ph.y * cd);
      }
    }
    Y[r * DFT2_F3 + kl] = cscale(acc, dt3);
  }
  __syncthreads();
  // t1 transform: one (k1, k3) sum a thread
  for (int o = threadIdx.x; o < nf1 * DFT2_F3; o += blockDim.x) {
    const int k1 = o / DFT2_F3, kl = o % DFT2_F3, k = k3base + kl;
    if (k >= nf3) continue;
    const double wk = (double)sign1 * (f1[k1] - rw) * uc;
    double sd, cd;
    sincos(wk * dt1, &sd, &cd);
    double2 acc = make_double2(0.0, 0.0), ph = make_double2(1.0, 0.0);
    for (int n = 0; n < n1; ++n) {
      if ((n & 31) == 0) {
        double sn, cn;
        sincos(wk * (t01 + (double)n * dt1), &sn, &cn);
        ph = make_double2(cn, sn);
      }
      cfma(acc, Y[n * DFT2_F3 + kl], ph);
      ph = make_double2(ph.x * cd - ph.y * sd, ph.x * sd + ph.y * cd);
    }
    X[((int64_t)k1 * nb + b) * nf3 + k] = cscale(acc, dt1);
  }
}

}  // namespace qsx

extern "C" int qsx_dft_batched_f32(const double* x, int nt, int64_t batch, double t0, double dt,
                                   const double* freqs, int nf, double rw_freq,
                                   double unit_convert, int sign, double* X, void* stream) {
  QSX_CHECK_ARG(nt >= 1 && nt <= 24576 && nf >= 1 && batch >= 0 && batch <= 65535,
                "qsx_dft_batched_f32: bad sizes nt=%d nf=%d (nt <= 24576)", nt, nf);
  QSX_CHECK_ARG(sign == 1 || sign == -1, "qsx_dft_batched_f32: sign must be +1 or -1");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(x && freqs && X, "qsx_dft_batched_f32: null pointer");
  const size_t smem = (size_t)nt * sizeof(float2);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(qsx::dft_f32_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return qsx::cuda_status(e, "qsx_dft_batched_f32");
  }
  dim3 grid((unsigned)((nf + 7) / 8), (unsigned)batch);
  qsx::dft_f32_kernel<<<grid, 256, smem, (cudaStream_t)stream>>>(
      (const double2*)x, nt, t0, dt, freqs, nf, rw_freq, unit_convert, sign, (double2*)X);
  QSX_LAUNCH_CHECK("qsx_dft_batched_f32");
  return QSX_OK;
}

extern "C" int qsx_dft_batched(const double* x, int nt, int64_t batch, double t0, double dt,
                               const double* freqs, int nf, double rw_freq,
                               double unit_convert, int sign, double* X, void* stream) {
  QSX_CHECK_ARG(nt >= 1 && nf >= 1 && batch >= 0 && batch <= 65535,
                "qsx_dft_batched: bad sizes nt=%d nf=%d", nt, nf);
  QSX_CHECK_ARG(sign == 1 || sign == -1, "qsx_dft_batched: sign must be +1 or -1");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(x && freqs && X, "qsx_dft_batched: null pointer");
  dim3 grid((unsigned)((nf + 7) / 8), (unsigned)batch);
  qsx::dft_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(
      (const double2*)x, nt, t0, dt, freqs, nf, rw_freq, unit_convert, sign, (double2*)X);
  QSX_LAUNCH_CHECK("qsx_dft_batched");
  return QSX_OK;
}

extern "C" int qsx_dft2_batched(const double* x, int n1, int64_t batch, int n3, int64_t s1,
                                int64_t sb, int64_t s3, double t01, double dt1,
                                const double* f1, int nf1, int sign1, double t03, double dt3,
                                const double* f3, int nf3, int sign3, double rw_freq,
                                double unit_convert, double* X, void* stream) {
  QSX_CHECK_ARG(n1 >= 1 && n3 >= 1 && nf1 >= 1 && nf3 >= 1 && batch >= 0 && batch <= 65535,
                "qsx_dft2_batched: bad sizes n1=%d n3=%d nf1=%d nf3=%d", n1, n3, nf1, nf3);
  QSX_CHECK_ARG((sign1 == 1 || sign1 == -1) && (sign3 == 1 || sign3 == -1),
                "qsx_dft2_batched: signs must be +1 or -1");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(x && f1 && f3 && X, "qsx_dft2_batched: null pointer");
  const size_t smem = (size_t)n1 * qsx::DFT2_F3 * sizeof(double2);
  QSX_CHECK_ARG(smem <= 200 * 1024, "qsx_dft2_batched: n1 = %d too long (at most %d)", n1,
                (int)(200 * 1024 / (qsx::DFT2_F3 * sizeof(double2))));
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(qsx::dft2_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return qsx::cuda_status(e, "qsx_dft2_batched");
  }
  dim3 grid((unsigned)((nf3 + qsx::DFT2_F3 - 1) / qsx::DFT2_F3), (unsigned)batch);
  qsx::dft2_kernel<<<grid, 256, smem, (cudaStream_t)stream>>>(
      (const double2*)x, n1, n3, s1, sb, s3, t01, dt1, f1, nf1, sign1, t03, dt3, f3, nf3, sign3,
      rw_freq, unit_convert, (double2*)X);
  QSX_LAUNCH_CHECK("qsx_dft2_batched");
  return QSX_OK;
}

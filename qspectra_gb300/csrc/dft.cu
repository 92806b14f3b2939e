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

}  // namespace qsx

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

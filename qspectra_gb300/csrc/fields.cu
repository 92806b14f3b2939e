// RK4 under applied fields: the time loop of simulate_with_fields /
// simulate_pump (qspectra/simulate/eom.py:77-227).  The reference integrates
//   dy/dt = L y + sum_p (-i E_p(t)^(*)) [V_p, y]
// with zvode, calling each pulse at every right-hand-side evaluation.  Here
// the host tabulates the field coefficients a_p(t) = -i E_p(t) (conjugated
// for '+' transitions) at every RK4 stage time (t_n, t_n + h/2, t_n + h) and
// one CTA per disorder sample runs the classical RK4 stages
//   k = (L + sum_p a_p(t) C_p) x,   C_p = the commutator map of V_p,
// with L and the C_p transposed in shared memory (thread r reads column r of
// the transposed matrices: conflict-free), one thread per state row.  FP32
// keeps a split-word (hi + lo) state.
#include "qsx_common.cuh"

namespace qsx {

struct FieldP {
  int m, nsteps, np, save_every, nsave;
  int64_t batch;
  const void* L;     // [batch][m][m] complex (T), stride L_stride elements (0 = shared)
  int64_t L_stride;
  const void* C;     // [np][m][m] complex (T), stride C_stride elements (0 = shared)
  int64_t C_stride;
  const void* coef;  // [nsteps][3][np] complex (T)
  double h;
  const double2* y0;
  int64_t y0_stride;
  double2* out;      // [batch][nsave][m]
  int* status;
};

template <typename T>
__global__ void __launch_bounds__(1024) rk4_field_kernel(FieldP p) {
  using Cx = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int m = p.m, np = p.np;
  Cx* sx = (Cx*)smraw;                   // [m] stage input
  Cx* sLT = sx + m;                      // [m][m] L transposed
  Cx* sCT = sLT + (size_t)m * m;         // [np][m][m] C_p transposed
  Cx* sa = sCT + (size_t)np * m * m;     // [np] stage coefficients
  const int64_t s = blockIdx.x;
  const Cx* L = (const Cx*)p.L + s * p.L_stride;
  const Cx* C = (const Cx*)p.C + s * p.C_stride;
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int r = e / m, c = e % m;
    sLT[c * m + r] = L[e];
  }
  for (int e = threadIdx.x; e < np * m * m; e += blockDim.x) {
    const int q = e / (m * m), rc = e % (m * m);
    const int r = rc / m, c = rc % m;
    sCT[(size_t)q * m * m + c * m + r] = C[e];
  }
  const int r = threadIdx.x;
  const bool row = r < m;
  const T h = (T)p.h;
  Cx yh = cmk((T)0, (T)0), yl = yh;
  if (row) {
    const double2 v = p.y0[s * p.y0_stride + r];
    yh = cmk((T)v.x, (T)v.y);
    if (sizeof(T) == 4) yl = cmk((T)(v.x - (double)yh.x), (T)(v.y - (double)yh.y));
  }
  auto save = [&](int k) {
    if (row) {
      double vx = (double)yh.x, vy = (double)yh.y;
      if (sizeof(T) == 4) {
        vx += (double)yl.x;
        vy += (double)yl.y;
      }
      p.out[(s * p.nsave + k) * m + r] = make_double2(vx, vy);
    }
  };
  save(0);
  const Cx* coef = (const Cx*)p.coef;
  const T cst[4] = {(T)0, (T)0.5, (T)0.5, (T)1};
  const T wgt[4] = {(T)1, (T)2, (T)2, (T)1};
  for (int step = 0; step < p.nsteps; ++step) {
    Cx kprev = cmk((T)0, (T)0), acc = kprev;
    for (int stage = 0; stage < 4; ++stage) {
      __syncthreads();  // everyone is done with the previous stage's sx, sa
      if (row) {
        const T c = cst[stage] * h;
        sx[r] = cmk(yh.x + c * kprev.x, yh.y + c * kprev.y);
      }
      const int ci = stage == 0 ? 0 : (stage == 3 ? 2 : 1);
      for (int q = threadIdx.x; q < np; q += blockDim.x)
        sa[q] = coef[((int64_t)step * 3 + ci) * np + q];
      __syncthreads();
      if (row) {
        Cx k0 = cmk((T)0, (T)0), k1 = k0;
        for (int j = 0; j < m; j += 2) {
          cfma(k0, sLT[j * m + r], sx[j]);
          if (j + 1 < m) cfma(k1, sLT[(j + 1) * m + r], sx[j + 1]);
        }
        Cx k = cmk(k0.x + k1.x, k0.y + k1.y);
        for (int q = 0; q < np; ++q) {
          const Cx* cq = sCT + (size_t)q * m * m;
          Cx f = cmk((T)0, (T)0);
          for (int j = 0; j < m; ++j) cfma(f, cq[j * m + r], sx[j]);
          cfma(k, sa[q], f);
        }
        acc = cmk(acc.x + wgt[stage] * k.x, acc.y + wgt[stage] * k.y);
        kprev = k;
      }
    }
    if (row) {
      const T s6 = h / (T)6;
      if (sizeof(T) == 4) {
        float hx = (float)yh.x, lx = (float)yl.x, hy = (float)yh.y, ly = (float)yl.y;
        dd_add(hx, lx, (float)(s6 * acc.x));
        dd_add(hy, ly, (float)(s6 * acc.y));
        yh = cmk((T)hx, (T)hy);
        yl = cmk((T)lx, (T)ly);
      } else {
        yh = cmk(yh.x + s6 * acc.x, yh.y + s6 * acc.y);
      }
    }
    if ((step + 1) % p.save_every == 0) save((step + 1) / p.save_every);
  }
  if (row && p.status && !(isfinite((double)yh.x) && isfinite((double)yh.y)))
    atomicOr(p.status, QSX_ERR_NONFINITE);
}

}  // namespace qsx

using namespace qsx;

extern "C" int qsx_rk4_field_batched(const void* L, int64_t L_stride, const void* C,
                                     int64_t C_stride, int npulses, const void* coef,
                                     int m, int64_t batch,
                                     int nsteps, double h, const double* y0,
                                     int64_t y0_stride, int save_every, int precision,
                                     double* out_state, int32_t* status, void* stream) {
  QSX_CHECK_ARG(m >= 1 && m <= 1024 && npulses >= 0 && batch >= 0 && nsteps >= 0 &&
                    save_every >= 1 && nsteps % save_every == 0,
                "qsx_rk4_field_batched: bad sizes (m=%d, pulses=%d, steps=%d, save_every=%d)",
                m, npulses, nsteps, save_every);
  QSX_CHECK_ARG(precision == QSX_FP32 || precision == QSX_FP64,
                "qsx_rk4_field_batched: bad precision");
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(L && y0 && out_state && (npulses == 0 || (C && coef)),
                "qsx_rk4_field_batched: null pointer");
  const size_t cs = precision == QSX_FP32 ? sizeof(float2) : sizeof(double2);
  const size_t smem = ((size_t)m + (size_t)(1 + npulses) * m * m + npulses) * cs;
  QSX_CHECK_ARG(smem <= 227 * 1024,
                "qsx_rk4_field_batched: %zu bytes of generator and field maps exceed "
                "shared memory",
                smem);
  FieldP p;
  p.m = m;
  p.nsteps = nsteps;
  p.np = npulses;
  p.save_every = save_every;
  p.nsave = nsteps / save_every + 1;
  p.batch = batch;
  p.L = L;
  p.L_stride = L_stride;
  p.C = C;
  p.C_stride = npulses ? C_stride : 0;
  p.coef = coef;
  p.h = h;
  p.y0 = (const double2*)y0;
  p.y0_stride = y0_stride;
  p.out = (double2*)out_state;
  p.status = status;
  const int threads = ((m + 31) / 32) * 32;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (precision == QSX_FP32) {
    e = cudaFuncSetAttribute(rk4_field_kernel<float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_field_batched");
    rk4_field_kernel<float><<<(unsigned)batch, threads, smem, s>>>(p);
  } else {
    e = cudaFuncSetAttribute(rk4_field_kernel<double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_field_batched");
    rk4_field_kernel<double><<<(unsigned)batch, threads, smem, s>>>(p);
  }
  QSX_LAUNCH_CHECK("qsx_rk4_field_batched");
  return QSX_OK;
}

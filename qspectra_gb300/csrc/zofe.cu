// ZOFE master equation (qspectra/dynamics/zofe.py:121-229): the time loop of
// a ZOFEModel, optionally under applied fields (simulate/eom.py:77-105).
//
// State: rho (n x n) and the auxiliary operators O[pm][s] (n x n) for every
// pseudomode pm and site s, laid out as the reference's state vector
// (rho column-major, then O column-major over (pm, s, k, l)).  The right-hand
// side is quadratic in the state:
//   S_s   = sum_pm O[pm][s]
//   a     = sum_s L_s^H S_s,   b = -i H - a
//   rho'  = b rho + sum_s L_s rho S_s^H + rho (i H - a^H) + sum_s S_s rho L_s^H
//   O'    = Gamma[pm][s] L_s - w[pm][s] O + b O - O b,
// all times unit_convert, with L_s the (diagonal) system-bath coupling of
// site s (already carrying the ZOFE sign).  A pulse p adds a_p(t) [V_p, .] to
// both rho and every O (not scaled by unit_convert), which folds into the
// small operators: the left operator becomes b + sum_p a_p V_p / unit_convert
// and the right one (i H - a^H) - sum_p a_p V_p / unit_convert.  The
// rho_hermit forms (zofe.py:179-192) take rho^H in the last rho term and, with
// ham_hermit, in the third one too (the field part still multiplies rho).
//
// GB300 layout: one thread-block cluster per sample.  The pseudomodes are
// split over the cluster's CTAs; each CTA keeps its share of O (plus a
// replica of rho) in shared memory as the stage input and its own elements
// in registers.  Per RK4 stage the only exchange is the pseudomode sum S:
// each CTA writes its partial sum, the cluster barrier publishes it, and
// every CTA adds the peers' partials through distributed shared memory
// (double-buffered, so one cluster barrier per stage suffices).  The small
// operators a, b are then rebuilt redundantly in every CTA.
#include <cooperative_groups.h>

#include "qsx_common.cuh"

namespace cg = cooperative_groups;

namespace qsx {

struct ZofeP {
  int n, N, npm, pmc, csize;  // states, sites, pseudomodes, pseudomodes per CTA, cluster
  int nsteps, save_every, nsave, np, nproj, mode, rho_only;
  int herm_big, herm_right;   // rho^H in sum_s S_s rho L_s^H / in rho (i H - a^H)
  int64_t batch, H_stride, V_stride, y0_stride;
  int64_t M;                  // n^2 + npm N n^2
  const double* H;            // real [n][n], rotating frame
  const double* Ld;           // [N][n] diagonal of L_s
  const double2* G;           // [npm][N] Gamma = Omega^2 huang
  const double2* W;           // [npm][N] w = i Omega + gamma
  const double2* V;           // [np][n][n] row-major
  const double2* coef;        // [nsteps][3][np]
  const double2* proj;        // [nproj][n*n] over rho (column-major)
  double uc, inv_uc, h;
  const double2* y0;          // [batch][M]
  double2* out_state;         // [batch][nsave][M] or NULL
  double2* out_proj;          // [batch][nsave][nproj] or NULL
  int* status;
};

// Write the state (rank 0 owns rho, every rank its pseudomodes) and, on
// rank 0, the projections of rho, for output k.
template <typename T, int EPT>
__device__ __forceinline__ void zofe_save(const ZofeP& p, int k, int64_t smp, int rank,
                                          const int64_t (&gidx)[EPT],
                                          const typename cplx<T>::type (&yh)[EPT],
                                          const typename cplx<T>::type (&yl)[EPT],
                                          typename cplx<T>::type* sx) {
  const int n2 = p.n * p.n, tid = threadIdx.x, bd = blockDim.x;
  if (p.out_state) {
    const int64_t row = p.rho_only ? (int64_t)n2 : p.M;
#pragma unroll
    for (int u = 0; u < EPT; ++u) {
      const int e = tid + u * bd;
      if (gidx[u] < 0 || (e < n2 && rank != 0) || (p.rho_only && e >= n2)) continue;
      double vx = (double)yh[u].x, vy = (double)yh[u].y;
      if (sizeof(T) == 4) {
        vx += (double)yl[u].x;
        vy += (double)yl[u].y;
      }
      p.out_state[(smp * p.nsave + k) * row + gidx[u]] = make_double2(vx, vy);
    }
  }
  if (p.out_proj && rank == 0) {
    __syncthreads();
#pragma unroll
    for (int u = 0; u < EPT; ++u) {
      const int e = tid + u * bd;
      if (e < n2) sx[e] = yh[u];
    }
    __syncthreads();
    for (int r = tid; r < p.nproj; r += bd) {
      double ax = 0.0, ay = 0.0;
      const double2* pr = p.proj + (int64_t)r * n2;
      for (int e = 0; e < n2; ++e) {
        const double2 a = pr[e];
        const double bx = (double)sx[e].x, by = (double)sx[e].y;
        ax += a.x * bx - a.y * by;
        ay += a.x * by + a.y * bx;
      }
      p.out_proj[(smp * p.nsave + k) * p.nproj + r] = make_double2(ax, ay);
    }
  }
}

template <typename T, int EPT>
__global__ void __launch_bounds__(EPT >= 4 ? 512 : 1024, 1)
    zofe_rk4_kernel(ZofeP p) {
  using Cx = typename cplx<T>::type;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int C = p.csize;
  const int64_t smp = blockIdx.x / C;
  const int n = p.n, N = p.N, n2 = n * n, Q = N * n2, np = p.np;
  const int pm0 = rank * p.pmc;
  const int P = max(0, min(p.npm, pm0 + p.pmc) - pm0);
  const int Mloc = n2 + P * Q;
  const int tid = threadIdx.x, bd = blockDim.x;

  extern __shared__ __align__(16) unsigned char smraw[];
  Cx* sx = (Cx*)smraw;                        // [n2 + pmc Q] stage input
  Cx* sS = sx + n2 + (size_t)p.pmc * Q;       // [Q] pseudomode sum
  Cx* sPart = sS + Q;                         // [2][Q] partial sums (read by peers)
  Cx* sB = sPart + 2 * (size_t)Q;             // [n2] left operator, row-major
  Cx* sR = sB + n2;                           // [n2] right operator (rho), row-major
  Cx* sF = sR + n2;                           // [n2] field part of the right operator
  Cx* sG = sF + n2;                           // [pmc][N]
  Cx* sW = sG + (size_t)p.pmc * N;            // [pmc][N]
  Cx* sV = sW + (size_t)p.pmc * N;            // [np][n2]
  Cx* sa = sV + (size_t)np * n2;              // [np]
  T* sH = (T*)(sa + np + (np & 1));           // [n2]
  T* sLd = sH + n2;                           // [N][n]

  const double* Hs = p.H + smp * p.H_stride;
  for (int e = tid; e < n2; e += bd) sH[e] = (T)Hs[e];
  for (int e = tid; e < N * n; e += bd) sLd[e] = (T)p.Ld[e];
  for (int e = tid; e < P * N; e += bd) {
    const int pmL = e / N, s = e % N;
    const double2 g = p.G[(pm0 + pmL) * N + s], w = p.W[(pm0 + pmL) * N + s];
    sG[e] = cmk((T)g.x, (T)g.y);
    sW[e] = cmk((T)w.x, (T)w.y);
  }
  const double2* Vs = p.V + smp * p.V_stride;
  for (int e = tid; e < np * n2; e += bd) sV[e] = cmk((T)Vs[e].x, (T)Vs[e].y);

  // this thread's elements: local index -> global index of the state vector
  int64_t gidx[EPT];
  Cx yh[EPT], yl[EPT], acc[EPT], dk[EPT];
#pragma unroll
  for (int u = 0; u < EPT; ++u) {
    const int e = tid + u * bd;
    gidx[u] = -1;
    yh[u] = yl[u] = acc[u] = dk[u] = cmk((T)0, (T)0);
    if (e < Mloc) {
      if (e < n2) {
        gidx[u] = e;
      } else {
        const int qq = e - n2, pmL = qq % P, q = qq / P;
        gidx[u] = n2 + (int64_t)(pm0 + pmL) + (int64_t)p.npm * q;
      }
      const double2 v = p.y0[smp * p.y0_stride + gidx[u]];
      yh[u] = cmk((T)v.x, (T)v.y);
      if (sizeof(T) == 4) yl[u] = cmk((T)(v.x - (double)yh[u].x), (T)(v.y - (double)yh[u].y));
    }
  }

  const T h = (T)p.h, uc = (T)p.uc, inv_uc = (T)p.inv_uc;
  const int nsteps = p.mode == 1 ? 1 : p.nsteps;
  const int nstages = p.mode == 1 ? 1 : 4;
  if (p.mode == 0) zofe_save<T, EPT>(p, 0, smp, rank, gidx, yh, yl, sx);
  for (int step = 0; step < nsteps; ++step) {
    for (int stage = 0; stage < nstages; ++stage) {
      const int buf = (step * 4 + stage) & 1;
      __syncthreads();  // everyone is done with the previous stage's sx and operators
      const T c = (stage == 0 ? (T)0 : (stage == 3 ? (T)1 : (T)0.5)) * h;
      const T wg = (stage == 0 || stage == 3) ? (T)1 : (T)2;
#pragma unroll
      for (int u = 0; u < EPT; ++u) {
        const int e = tid + u * bd;
        if (e < Mloc) sx[e] = cmk(yh[u].x + c * dk[u].x, yh[u].y + c * dk[u].y);
      }
      const int ci = stage == 0 ? 0 : (stage == 3 ? 2 : 1);
      for (int q = tid; q < np; q += bd) {
        const double2 v = p.coef[((int64_t)step * 3 + ci) * np + q];
        sa[q] = cmk((T)v.x, (T)v.y);
      }
      __syncthreads();
      // partial pseudomode sums of this CTA's share of O
      Cx* part = sPart + (size_t)buf * Q;
      for (int q = tid; q < Q; q += bd) {
        Cx z = cmk((T)0, (T)0);
        for (int pmL = 0; pmL < P; ++pmL) z = cadd2(z, sx[n2 + pmL + (size_t)P * q]);
        part[q] = z;
      }
      cluster.sync();  // partials published cluster-wide
      for (int q = tid; q < Q; q += bd) {
        // issue every peer's load before adding (they are independent)
        Cx v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r)
          v[r] = r < C ? cluster.map_shared_rank(part, r)[q] : cmk((T)0, (T)0);
        Cx z = v[0];
#pragma unroll
        for (int r = 1; r < 8; ++r) z = cadd2(z, v[r]);
        sS[q] = z;
      }
      __syncthreads();
      // small operators: B = -iH - a + sum_p a_p V_p, R = iH - a^H - sum_p a_p V_p
      for (int e = tid; e < n2; e += bd) {
        const int i = e / n, k = e % n;
        Cx aik = cmk((T)0, (T)0), aki = aik, fv = aik;
        for (int s = 0; s < N; ++s) {
          const T li = sLd[s * n + i], lk = sLd[s * n + k];
          if (li != (T)0) {
            const Cx Sik = sS[s + N * (i + n * k)];
            aik = cmk(aik.x + li * Sik.x, aik.y + li * Sik.y);
          }
          if (lk != (T)0) {
            const Cx Ski = sS[s + N * (k + n * i)];
            aki = cmk(aki.x + lk * Ski.x, aki.y + lk * Ski.y);
          }
        }
        for (int q = 0; q < np; ++q) cfma(fv, sa[q], sV[(size_t)q * n2 + e]);
        // the field term is not scaled by unit_convert: fold it in divided by it
        fv = cmk(fv.x * inv_uc, fv.y * inv_uc);
        const T Hik = sH[e];
        sB[e] = cmk(-aik.x + fv.x, -Hik - aik.y + fv.y);
        sR[e] = cmk(-aki.x - fv.x, Hik + aki.y - fv.y);
        sF[e] = fv;
      }
      __syncthreads();
      // derivatives of this thread's elements
#pragma unroll
      for (int u = 0; u < EPT; ++u) {
        const int e = tid + u * bd;
        if (e >= Mloc) continue;
        Cx d = cmk((T)0, (T)0);
        if (e < n2) {
          const int i = e % n, m = e / n;  // rho[i][m], column-major
          for (int j = 0; j < n; ++j) cfma(d, sB[i * n + j], sx[j + n * m]);
          if (!p.herm_right) {
            for (int j = 0; j < n; ++j) cfma(d, sx[i + n * j], sR[j * n + m]);
          } else {
            // rho^H (R + F) - rho F: the field still acts on rho itself
            for (int j = 0; j < n; ++j) {
              const Cx rh = sx[j + n * i], r = sx[i + n * j], f = sF[j * n + m];
              cfma(d, cmk(rh.x, -rh.y), sR[j * n + m]);
              cfma(d, cmk(rh.x - r.x, -rh.y - r.y), f);
            }
          }
          // the couplings are site number operators: most L_s[i] vanish
          for (int s = 0; s < N; ++s) {
            const T li = sLd[s * n + i], lm = sLd[s * n + m];
            if (li != (T)0) {
              Cx cs = cmk((T)0, (T)0);
              for (int k = 0; k < n; ++k) {
                const Cx Smk = sS[s + N * (m + n * k)];
                cfma(cs, sx[i + n * k], cmk(Smk.x, -Smk.y));
              }
              d = cmk(d.x + li * cs.x, d.y + li * cs.y);
            }
            if (lm != (T)0) {
              Cx bs = cmk((T)0, (T)0);
              if (!p.herm_big) {
                for (int k = 0; k < n; ++k) cfma(bs, sS[s + N * (i + n * k)], sx[k + n * m]);
              } else {
                for (int k = 0; k < n; ++k) {
                  const Cx r = sx[m + n * k];
                  cfma(bs, sS[s + N * (i + n * k)], cmk(r.x, -r.y));
                }
              }
              d = cmk(d.x + lm * bs.x, d.y + lm * bs.y);
            }
          }
        } else {
          const int qq = e - n2, pmL = qq % P, q = qq / P;
          const int s = q % N, k = (q / N) % n, l = q / (N * n);
          const Cx* Ob = sx + n2 + pmL + (size_t)P * s;  // O[pmL][s][j][l] = Ob[P N (j + n l)]
          const size_t js = (size_t)P * N;
          for (int j = 0; j < n; ++j) {
            cfma(d, sB[k * n + j], Ob[js * (j + n * l)]);
            const Cx okj = Ob[js * (k + n * j)];
            const Cx bjl = sB[j * n + l];
            cfma(d, cmk(-okj.x, -okj.y), bjl);
          }
          const Cx w = sW[pmL * N + s];
          cfma(d, cmk(-w.x, -w.y), sx[e]);
          if (k == l) {
            const Cx g = sG[pmL * N + s];
            const T lk = sLd[s * n + k];
            d = cmk(d.x + g.x * lk, d.y + g.y * lk);
          }
        }
        d = cmk(d.x * uc, d.y * uc);
        acc[u] = cmk(acc[u].x + wg * d.x, acc[u].y + wg * d.y);
        dk[u] = d;
      }
    }
    if (p.mode == 1) break;
    const T s6 = h / (T)6;
#pragma unroll
    for (int u = 0; u < EPT; ++u) {
      if (sizeof(T) == 4) {
        float hx = (float)yh[u].x, lx = (float)yl[u].x, hy = (float)yh[u].y, ly = (float)yl[u].y;
        dd_add(hx, lx, (float)(s6 * acc[u].x));
        dd_add(hy, ly, (float)(s6 * acc[u].y));
        yh[u] = cmk((T)hx, (T)hy);
        yl[u] = cmk((T)lx, (T)ly);
      } else {
        yh[u] = cmk(yh[u].x + s6 * acc[u].x, yh[u].y + s6 * acc[u].y);
      }
      acc[u] = dk[u] = cmk((T)0, (T)0);
    }
    if ((step + 1) % p.save_every == 0)
      zofe_save<T, EPT>(p, (step + 1) / p.save_every, smp, rank, gidx, yh, yl, sx);
  }
  if (p.mode == 1 && p.out_state) {
    // the right-hand side at y0 (stage 0 derivative)
#pragma unroll
    for (int u = 0; u < EPT; ++u) {
      const int e = tid + u * bd;
      if (gidx[u] < 0 || (e < n2 && rank != 0)) continue;
      p.out_state[smp * p.M + gidx[u]] = make_double2((double)dk[u].x, (double)dk[u].y);
    }
  }
  bool bad = false;
#pragma unroll
  for (int u = 0; u < EPT; ++u)
    if (gidx[u] >= 0 && !(isfinite((double)yh[u].x) && isfinite((double)yh[u].y))) bad = true;
  if (bad && p.status) atomicOr(p.status, QSX_ERR_NONFINITE);
  cluster.sync();  // peers may still read this CTA's partial sums
}

template <typename T, int EPT>
static cudaError_t launch_zofe(const ZofeP& p, int threads, size_t smem, cudaStream_t s) {
  auto kern = zofe_rk4_kernel<T, EPT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(p.batch * p.csize));
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)p.csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, p);
}

}  // namespace qsx

using namespace qsx;

extern "C" size_t qsx_zofe_args_bytes(void) { return sizeof(qsx_zofe_args); }

extern "C" int qsx_zofe_rk4(const qsx_zofe_args* a, void* stream) {
  QSX_CHECK_ARG(a != nullptr, "qsx_zofe_rk4: null args");
  QSX_CHECK_ARG(a->precision == QSX_FP32 || a->precision == QSX_FP64,
                "qsx_zofe_rk4: bad precision");
  QSX_CHECK_ARG(a->n >= 1 && a->n <= 32 && a->n_sites >= 1 && a->npm >= 1 &&
                    a->npulses >= 0 && a->nproj >= 0 && a->batch >= 0 && a->nsteps >= 0 &&
                    a->save_every >= 1 && a->nsteps % a->save_every == 0 &&
                    (a->mode == 0 || a->mode == 1) && a->cluster >= 0 && a->cluster <= 8 &&
                    (a->hermit == 0 || a->hermit == QSX_ZOFE_RHO_HERMIT ||
                     a->hermit == (QSX_ZOFE_RHO_HERMIT | QSX_ZOFE_HAM_HERMIT)) &&
                    (a->save_rho_only == 0 || a->save_rho_only == 1),
                "qsx_zofe_rk4: bad sizes (n=%d, sites=%d, pseudomodes=%d, steps=%d)", a->n,
                a->n_sites, a->npm, a->nsteps);
  if (a->batch == 0) return QSX_OK;
  QSX_CHECK_ARG(a->H && a->Ld && a->Gamma && a->w && a->y0 &&
                    (a->npulses == 0 || (a->V && a->coef)) &&
                    (a->nproj == 0 || (a->proj && a->out_proj)) &&
                    (a->out_state || a->out_proj),
                "qsx_zofe_rk4: null pointer");
  QSX_CHECK_ARG(a->mode == 0 || a->out_state, "qsx_zofe_rk4: mode 1 writes out_state");
  QSX_CHECK_ARG(a->npulses == 0 || a->unit_convert != 0.0,
                "qsx_zofe_rk4: pulses need a nonzero unit_convert");
  const int n = a->n, N = a->n_sites, n2 = n * n, Q = N * n2;
  // cluster size: enough CTAs to fill the GPU, each owning at least one pseudomode
  int C = a->cluster;
  if (C == 0) {
    C = 1;
    while (C < 8 && C * 2 <= a->npm && a->batch * C < 2 * 152) C *= 2;
  }
  auto per_cta = [&](int c) { return n2 + ((a->npm + c - 1) / c) * Q; };
  while (per_cta(C) > 4096 && C < 8 && C * 2 <= a->npm) C *= 2;
  const int pmc = (a->npm + C - 1) / C;
  const int Mloc = per_cta(C);
  if (Mloc > 4096) {
    set_error("qsx_zofe_rk4: %d state elements per CTA exceed 4096 (n=%d, sites=%d, "
              "pseudomodes=%d, cluster %d)",
              Mloc, n, N, a->npm, C);
    return QSX_ERR_UNSUPPORTED;
  }
  const bool f32 = a->precision == QSX_FP32;
  // elements per thread: FP64 keeps 128 registers a thread above one element
  const int ept = Mloc <= 1024 ? 1 : (Mloc <= 2048 ? (f32 ? 2 : 4) : 8);
  const int maxthr = ept >= 4 ? 512 : 1024;
  int threads = (Mloc + ept - 1) / ept;
  threads = ((threads + 31) / 32) * 32;
  if (threads < 64) threads = 64;
  if (threads > maxthr) threads = maxthr;
  const size_t cs = a->precision == QSX_FP32 ? sizeof(float2) : sizeof(double2);
  const size_t rs = a->precision == QSX_FP32 ? sizeof(float) : sizeof(double);
  const int np = a->npulses;
  const size_t smem = ((size_t)n2 + (size_t)pmc * Q + 3 * (size_t)Q + 3 * (size_t)n2 +
                       2 * (size_t)pmc * N + (size_t)np * n2 + np + (np & 1)) * cs +
                      ((size_t)n2 + (size_t)N * n) * rs;
  QSX_CHECK_ARG(smem <= 227 * 1024, "qsx_zofe_rk4: %zu bytes of shared memory needed", smem);
  ZofeP p;
  p.n = n;
  p.N = N;
  p.npm = a->npm;
  p.pmc = pmc;
  p.csize = C;
  p.nsteps = a->mode == 1 ? 0 : a->nsteps;
  p.save_every = a->save_every;
  p.nsave = a->mode == 1 ? 1 : a->nsteps / a->save_every + 1;
  p.np = np;
  p.nproj = a->nproj;
  p.mode = a->mode;
  p.rho_only = a->save_rho_only;
  p.herm_big = (a->hermit & QSX_ZOFE_RHO_HERMIT) != 0;
  p.herm_right = a->hermit == (QSX_ZOFE_RHO_HERMIT | QSX_ZOFE_HAM_HERMIT);
  p.batch = a->batch;
  p.H_stride = a->H_stride;
  p.V_stride = np ? a->V_stride : 0;
  p.y0_stride = a->y0_stride;
  p.M = (int64_t)n2 + (int64_t)a->npm * Q;
  p.H = a->H;
  p.Ld = a->Ld;
  p.G = (const double2*)a->Gamma;
  p.W = (const double2*)a->w;
  p.V = (const double2*)a->V;
  p.coef = (const double2*)a->coef;
  p.proj = (const double2*)a->proj;
  p.uc = a->unit_convert;
  p.inv_uc = np ? 1.0 / a->unit_convert : 0.0;
  p.h = a->h;
  p.y0 = (const double2*)a->y0;
  p.out_state = (double2*)a->out_state;
  p.out_proj = a->mode == 1 ? nullptr : (double2*)a->out_proj;
  p.status = a->status;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (ept == 1)
    e = f32 ? launch_zofe<float, 1>(p, threads, smem, s) : launch_zofe<double, 1>(p, threads, smem, s);
  else if (ept == 2)
    e = launch_zofe<float, 2>(p, threads, smem, s);
  else if (ept == 4)
    e = launch_zofe<double, 4>(p, threads, smem, s);
  else
    e = f32 ? launch_zofe<float, 8>(p, threads, smem, s) : launch_zofe<double, 8>(p, threads, smem, s);
  if (e != cudaSuccess) return cuda_status(e, "qsx_zofe_rk4");
  QSX_LAUNCH_CHECK("qsx_zofe_rk4");
  return QSX_OK;
}

// Hierarchical equations of motion (HEOM) on the GPU: the generator of
// HEOMModel (qspectra/dynamics/heom.py:298-443) applied in structured form,
// and the fixed-step RK4 time loop over it.
//
// The state is one Liouville block XY (nx x ny density matrices, column
// stacked, vec index a + nx b) per hierarchy node.  For node n,
//   d rho_n / dt = uc * { -i (Hx rho_n - rho_n Hy) - shift_n rho_n
//                         - tc * W o rho_n
//                         + sum_t (alpha_t occ_j(a) + beta_t occ_j(b)) rho_{nbr_t} }
// where j = site of term t, W[a][b] = sum_j (o_j(a) + o_j(b) - 2 o_j(a) o_j(b))
// is the low-temperature double commutator sum_j [K_j, [K_j, .]] for number
// operators, and the term table holds the up couplings (alpha, beta) =
// (-i m, +i m) and the down couplings (-i m c_k, +i m conj(c_k)).  The
// transposed generator (Heisenberg picture) has the same form with the term
// table transposed, which the host builds.
#include <algorithm>

#include "qsx_common.cuh"

namespace qsx {

struct HeomP {
  int nx, ny, E, nnodes, nterms, n_sites, nsteps, save_every, nsave;
  int64_t batch;
  const double* Hx;  // [batch][nx][nx] (stride Hx_stride)
  const double* Hy;
  int64_t Hx_stride, Hy_stride;
  const double* occx;  // [n_sites][nx]
  const double* occy;  // [n_sites][ny]
  const double* W;     // [E] low-temperature weights (already times tc), or null
  const double* shift;  // [nnodes]
  const int* nbr;       // [nnodes][nterms], -1 = none
  const int* site;      // [nnodes][nterms]
  const double2* alpha;  // [nnodes][nterms]
  const double2* beta;   // [nnodes][nterms]
  double uc, h;
};

// k = RHS(x) for nodes [n0, n0 + nodes_per_cta) of sample b, one thread per
// element.  Shared: Hx, Hy of the sample and the CTA's node blocks of x.
template <typename C>
__device__ __forceinline__ void heom_rhs_elem(const HeomP& p, const C* x, int64_t b,
                                              int node, int e, const C* sx, const double* sHx,
                                              const double* sHy, C& out) {
  using T = decltype(out.x);
  const int a = e % p.nx, bb = e / p.nx;
  // commutator: -i (Hx x - x Hy)[a][bb]
  T cr = 0, ci = 0;
  for (int c = 0; c < p.nx; ++c) {
    const T hv = (T)sHx[a * p.nx + c];
    const C v = sx[c + p.nx * bb];
    cr = fma(hv, v.x, cr);
    ci = fma(hv, v.y, ci);
  }
  for (int c = 0; c < p.ny; ++c) {
    const T hv = (T)sHy[c * p.ny + bb];
    const C v = sx[a + p.nx * c];
    cr = fma(-hv, v.x, cr);
    ci = fma(-hv, v.y, ci);
  }
  // -i (cr + i ci) = ci - i cr
  const C self = sx[e];
  T orr = ci, oi = -cr;
  const T sh = (T)p.shift[node] + (p.W ? (T)p.W[e] : (T)0);
  orr = fma(-sh, self.x, orr);
  oi = fma(-sh, self.y, oi);
  const int base = node * p.nterms;
  const size_t nodesz = (size_t)p.E;
  const C* xb = x + b * (int64_t)p.nnodes * p.E;
  for (int t = 0; t < p.nterms; ++t) {
    const int nb = p.nbr[base + t];
    if (nb < 0) continue;
    const int j = p.site[base + t];
    const double2 al = p.alpha[base + t], be = p.beta[base + t];
    const double oa = p.occx[j * p.nx + a], ob = p.occy[j * p.ny + bb];
    const T fr = (T)(al.x * oa + be.x * ob), fi = (T)(al.y * oa + be.y * ob);
    const C v = xb[nb * nodesz + e];
    orr = fma(fr, v.x, fma(-fi, v.y, orr));
    oi = fma(fr, v.y, fma(fi, v.x, oi));
  }
  out.x = (T)p.uc * orr;
  out.y = (T)p.uc * oi;
}

// Shared staging of H and the CTA's node blocks; returns false if this CTA
// has no nodes.  blockDim = nodes_per_cta * E (rounded up to a warp).
template <typename C>
__device__ __forceinline__ void heom_stage_smem(const HeomP& p, const C* x, int64_t b,
                                                int n0, int npc, C* sx, double* sHx, double* sHy) {
  for (int i = threadIdx.x; i < p.nx * p.nx; i += blockDim.x) sHx[i] = p.Hx[b * p.Hx_stride + i];
  for (int i = threadIdx.x; i < p.ny * p.ny; i += blockDim.x) sHy[i] = p.Hy[b * p.Hy_stride + i];
  const C* xb = x + (b * p.nnodes + n0) * (int64_t)p.E;
  const int cnt = (npc < p.nnodes - n0 ? npc : p.nnodes - n0) * p.E;
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) sx[i] = xb[i];
  __syncthreads();
}

// One RK4 stage (see qsx_heom_rk4): k = RHS(in); stage 0..2 write the next
// stage input, stage 3 adds h/6 (acc + k) to the state (split-word in FP32).
template <typename T>
__global__ void __launch_bounds__(256)
    heom_stage_kernel(HeomP p, int stage, const typename cplx<T>::type* in,
                      typename cplx<T>::type* yh, typename cplx<T>::type* __restrict__ yl,
                      typename cplx<T>::type* __restrict__ acc,
                      typename cplx<T>::type* __restrict__ next, int npc) {
  using C = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  double* sHx = (double*)smraw;
  double* sHy = sHx + p.nx * p.nx;
  C* sx = (C*)(sHy + p.ny * p.ny + ((p.nx * p.nx + p.ny * p.ny) & 1));
  const int64_t b = blockIdx.y;
  const int n0 = blockIdx.x * npc;
  heom_stage_smem(p, in, b, n0, npc, sx, sHx, sHy);
  const int local = threadIdx.x / p.E, e = threadIdx.x % p.E;
  const int node = n0 + local;
  if (local >= npc || node >= p.nnodes) return;
  C k;
  heom_rhs_elem(p, in, b, node, e, sx + local * p.E, sHx, sHy, k);
  const int64_t idx = (b * p.nnodes + node) * (int64_t)p.E + e;
  const T h = (T)p.h;
  if (stage == 0) {
    acc[idx] = k;
    const C y = yh[idx];
    next[idx] = cmk(y.x + (T)0.5 * h * k.x, y.y + (T)0.5 * h * k.y);
  } else if (stage < 3) {
    C a = acc[idx];
    acc[idx] = cmk(a.x + (T)2 * k.x, a.y + (T)2 * k.y);
    const C y = yh[idx];
    const T c = stage == 1 ? (T)0.5 * h : h;
    next[idx] = cmk(y.x + c * k.x, y.y + c * k.y);
  } else {
    const C a = acc[idx];
    const T sx6 = h / (T)6;
    const T ix = sx6 * (a.x + k.x), iy = sx6 * (a.y + k.y);
    C y = yh[idx];
    if (sizeof(T) == 4) {
      C l = yl[idx];
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

// out = RHS(x) in FP64 (the equation of motion as a callable).
__global__ void __launch_bounds__(256)
    heom_rhs_kernel(HeomP p, const double2* __restrict__ x, double2* __restrict__ out, int npc) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double* sHx = (double*)smraw;
  double* sHy = sHx + p.nx * p.nx;
  double2* sx = (double2*)(sHy + p.ny * p.ny + ((p.nx * p.nx + p.ny * p.ny) & 1));
  const int64_t b = blockIdx.y;
  const int n0 = blockIdx.x * npc;
  heom_stage_smem(p, x, b, n0, npc, sx, sHx, sHy);
  const int local = threadIdx.x / p.E, e = threadIdx.x % p.E;
  const int node = n0 + local;
  if (local >= npc || node >= p.nnodes) return;
  double2 k;
  heom_rhs_elem(p, x, b, node, e, sx + local * p.E, sHx, sHy, k);
  out[(b * p.nnodes + node) * (int64_t)p.E + e] = k;
}

// initial state: y0 [batch or shared][nnodes][E] complex128 -> (yh, yl)
template <typename T>
__global__ void heom_init_kernel(const double2* __restrict__ y0, int64_t y0_stride, int64_t per,
                                 int64_t batch, typename cplx<T>::type* yh,
                                 typename cplx<T>::type* yl) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= per * batch) return;
  const int64_t b = i / per, r = i % per;
  const double2 v = y0[b * y0_stride + r];
  yh[i] = cmk((T)v.x, (T)v.y);
  if (yl) yl[i] = cmk((T)(v.x - (double)(T)v.x), (T)(v.y - (double)(T)v.y));
}

// the first `keep` node blocks of every sample into out[b][k][keep * E]
template <typename T>
__global__ void heom_save_kernel(const typename cplx<T>::type* __restrict__ yh,
                                 const typename cplx<T>::type* __restrict__ yl, int nnodes, int E,
                                 int keep, int64_t batch, int k, int nsave, double2* out,
                                 int* status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t ke = (int64_t)keep * E;
  if (i >= batch * ke) return;
  const int64_t b = i / ke;
  const int64_t e = i % ke;
  const int64_t src = b * nnodes * (int64_t)E + e;
  double vx = (double)yh[src].x, vy = (double)yh[src].y;
  if (yl) {
    vx += (double)yl[src].x;
    vy += (double)yl[src].y;
  }
  if (status && !(isfinite(vx) && isfinite(vy))) atomicOr(status, QSX_ERR_NONFINITE);
  out[(b * nsave + k) * ke + e] = make_double2(vx, vy);
}

__global__ void heom_mean_kernel(const double2* __restrict__ per, int64_t batch, int64_t n,
                                 double scale, double2* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double2 acc = make_double2(0.0, 0.0);
  for (int64_t b = 0; b < batch; ++b) acc = cadd(acc, per[b * n + i]);
  out[i] = cscale(acc, scale);
}

static int heom_validate(const qsx_heom_args* a) {
  QSX_CHECK_ARG(a != nullptr, "qsx_heom: null args");
  QSX_CHECK_ARG(a->precision == QSX_FP32 || a->precision == QSX_FP64, "qsx_heom: bad precision");
  QSX_CHECK_ARG(a->nx >= 1 && a->ny >= 1 && a->nx <= 32 && a->ny <= 32 && a->nx * a->ny <= 256,
                "qsx_heom: need nx, ny <= 32 and nx * ny <= 256");
  QSX_CHECK_ARG(a->nnodes >= 1 && a->nterms >= 0 && a->n_sites >= 1, "qsx_heom: bad sizes");
  QSX_CHECK_ARG(a->batch >= 0 && a->batch <= 65535, "qsx_heom: batch must be in [0, 65535]");
  QSX_CHECK_ARG(a->nsteps >= 0 && a->save_every >= 1 && a->nsteps % a->save_every == 0,
                "qsx_heom: nsteps must be a non-negative multiple of save_every");
  QSX_CHECK_ARG(a->save_nodes >= 1 && a->save_nodes <= a->nnodes,
                "qsx_heom: save_nodes must be in [1, nnodes]");
  QSX_CHECK_ARG(a->batch == 0 || (a->Hx && a->Hy && a->occx && a->occy && a->shift &&
                                  (a->nterms == 0 || (a->nbr && a->site && a->alpha && a->beta))),
                "qsx_heom: null table pointer");
  return QSX_OK;
}

static HeomP heom_params(const qsx_heom_args* a) {
  HeomP p;
  p.nx = a->nx;
  p.ny = a->ny;
  p.E = a->nx * a->ny;
  p.nnodes = a->nnodes;
  p.nterms = a->nterms;
  p.n_sites = a->n_sites;
  p.nsteps = a->nsteps;
  p.save_every = a->save_every;
  p.nsave = a->nsteps / a->save_every + 1;
  p.batch = a->batch;
  p.Hx = a->Hx;
  p.Hy = a->Hy;
  p.Hx_stride = a->H_stride ? (int64_t)a->nx * a->nx : 0;
  p.Hy_stride = a->H_stride ? (int64_t)a->ny * a->ny : 0;
  p.occx = a->occx;
  p.occy = a->occy;
  p.W = a->W;
  p.shift = a->shift;
  p.nbr = a->nbr;
  p.site = a->site;
  p.alpha = (const double2*)a->alpha;
  p.beta = (const double2*)a->beta;
  p.uc = a->unit_convert;
  p.h = a->h;
  return p;
}

static size_t heom_state_elems(const qsx_heom_args* a) {
  return (size_t)a->batch * a->nnodes * a->nx * a->ny;
}

}  // namespace qsx

using namespace qsx;

extern "C" {

size_t qsx_heom_args_bytes(void) { return sizeof(qsx_heom_args); }

int qsx_heom_workspace_bytes(const qsx_heom_args* a, size_t* bytes) {
  int st = heom_validate(a);
  if (st) return st;
  QSX_CHECK_ARG(bytes != nullptr, "qsx_heom_workspace_bytes: null output");
  const size_t n = heom_state_elems(a);
  const size_t cs = a->precision == QSX_FP32 ? sizeof(float2) : sizeof(double2);
  const int nsave = a->nsteps / a->save_every + 1;
  // yh, yl (FP32 only), acc, two stage buffers, per-sample node-0 outputs
  const size_t states = (a->precision == QSX_FP32 ? 5 : 4) * n * cs;
  const size_t saves =
      a->out_mean ? (size_t)a->batch * nsave * a->save_nodes * a->nx * a->ny * sizeof(double2) : 0;
  *bytes = states + saves + 256;
  return QSX_OK;
}

int qsx_heom_rhs(const qsx_heom_args* a, const double* x, double* out, void* stream) {
  int st = heom_validate(a);
  if (st) return st;
  if (a->batch == 0) return QSX_OK;
  QSX_CHECK_ARG(x && out, "qsx_heom_rhs: null state");
  HeomP p = heom_params(a);
  const int npc = std::max(1, 256 / p.E);
  const int threads = ((npc * p.E + 31) / 32) * 32;
  const size_t smem = (p.nx * p.nx + p.ny * p.ny + 1) * sizeof(double) + npc * p.E * sizeof(double2);
  dim3 grid((unsigned)((p.nnodes + npc - 1) / npc), (unsigned)p.batch);
  heom_rhs_kernel<<<grid, threads, smem, (cudaStream_t)stream>>>(p, (const double2*)x,
                                                                 (double2*)out, npc);
  QSX_LAUNCH_CHECK("qsx_heom_rhs");
  return QSX_OK;
}

int qsx_heom_rk4(const qsx_heom_args* a, void* stream) {
  int st = heom_validate(a);
  if (st) return st;
  if (a->batch == 0) return QSX_OK;
  QSX_CHECK_ARG(a->y0 != nullptr, "qsx_heom_rk4: null y0");
  QSX_CHECK_ARG(a->out_state || a->out_mean, "qsx_heom_rk4: no output requested");
  size_t need = 0;
  st = qsx_heom_workspace_bytes(a, &need);
  if (st) return st;
  QSX_CHECK_ARG(a->workspace && a->workspace_bytes >= need,
                "qsx_heom_rk4: workspace of %zu bytes needed (got %zu)", need, a->workspace_bytes);
  HeomP p = heom_params(a);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t n = heom_state_elems(a);
  const int npc = std::max(1, 256 / p.E);
  const int threads = ((npc * p.E + 31) / 32) * 32;
  dim3 grid((unsigned)((p.nnodes + npc - 1) / npc), (unsigned)p.batch);
  const int64_t per = (int64_t)p.nnodes * p.E;
  double2* node0 = a->out_state ? (double2*)a->out_state : nullptr;
  const int keep = a->save_nodes;
  unsigned char* ws = (unsigned char*)a->workspace;
  auto run = [&](auto tag) -> int {
    using T = decltype(tag);
    using C = typename cplx<T>::type;
    C* yh = (C*)ws;
    C* yl = sizeof(T) == 4 ? yh + n : nullptr;
    C* acc = (sizeof(T) == 4 ? yl : yh) + n;
    C* s0 = acc + n;
    C* s1 = s0 + n;
    double2* saves = (double2*)(((size_t)(s1 + n) + 255) & ~(size_t)255);
    if (!node0) node0 = saves;
    const size_t smem = (p.nx * p.nx + p.ny * p.ny + 1) * sizeof(double) + npc * p.E * sizeof(C);
    heom_init_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        (const double2*)a->y0, a->y0_stride ? per : 0, per, p.batch, yh, yl);
    QSX_LAUNCH_CHECK("qsx_heom_rk4 init");
    const unsigned sg = (unsigned)((p.batch * keep * p.E + 255) / 256);
    heom_save_kernel<T><<<sg, 256, 0, s>>>(yh, yl, p.nnodes, p.E, keep, p.batch, 0, p.nsave,
                                          node0, a->status);
    for (int step = 1; step <= p.nsteps; ++step) {
      heom_stage_kernel<T><<<grid, threads, smem, s>>>(p, 0, yh, yh, yl, acc, s0, npc);
      heom_stage_kernel<T><<<grid, threads, smem, s>>>(p, 1, s0, yh, yl, acc, s1, npc);
      heom_stage_kernel<T><<<grid, threads, smem, s>>>(p, 2, s1, yh, yl, acc, s0, npc);
      heom_stage_kernel<T><<<grid, threads, smem, s>>>(p, 3, s0, yh, yl, acc, nullptr, npc);
      if (step % p.save_every == 0)
        heom_save_kernel<T><<<sg, 256, 0, s>>>(yh, yl, p.nnodes, p.E, keep, p.batch,
                                              step / p.save_every, p.nsave, node0, a->status);
    }
    QSX_LAUNCH_CHECK("qsx_heom_rk4 steps");
    if (a->out_mean) {
      const int64_t m = (int64_t)p.nsave * keep * p.E;
      heom_mean_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(node0, p.batch, m,
                                                                   1.0 / (double)p.batch,
                                                                   (double2*)a->out_mean);
      QSX_LAUNCH_CHECK("qsx_heom_rk4 mean");
    }
    return QSX_OK;
  };
  return a->precision == QSX_FP32 ? run(0.0f) : run(0.0);
}

}  // extern "C"

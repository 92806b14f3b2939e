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
// (-i m, +i m) and the down couplings (-i m c_k, +i m conj(c_k)).  With
// aki_temp_corr (heom.py:385-442) a down term also carries
// gamma_t Wd[a][b] (occ_j(a) - occ_j(b)) rho_nbr with the raw (unscaled)
// double-commutator weights Wd.  The
// transposed generator (Heisenberg picture) has the same form with the term
// table transposed, which the host builds.
#include <cooperative_groups.h>

#include <algorithm>

#include "qsx_common.cuh"
#include "qsx_tc.cuh"

namespace cg = cooperative_groups;

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
  const double2* gamma;  // [nnodes][nterms] or null (aki_temp_corr terms)
  const double* Wraw;    // [E] or null
  double uc, h;
};

// Per-CTA tables in the working precision T (staged once so the element
// loop issues no FP64 work in the FP32 form): H blocks, occupations, the
// low-temperature weights and the term tables of the CTA's nodes.
template <typename T>
struct HeomSmem {
  using C = typename cplx<T>::type;
  T* Hx;      // nx * nx
  T* Hy;      // ny * ny
  T* ox;      // n_sites * nx
  T* oy;      // n_sites * ny
  T* W;       // E
  T* shift;   // npc
  C* al;      // npc * nterms
  C* be;      // npc * nterms
  C* ga;      // npc * nterms (zero without aki_temp_corr)
  T* Wr;      // E
  int* nbr;   // npc * nterms
  int* site;  // npc * nterms
  C* x;       // npc * E, this CTA's node blocks of the input
};

template <typename T>
__host__ __device__ inline size_t heom_smem_bytes(int nx, int ny, int n_sites, int E, int npc,
                                                  int nterms) {
  using C = typename cplx<T>::type;
  size_t b = (size_t)npc * E * sizeof(C) + 3 * (size_t)npc * nterms * sizeof(C);
  b += ((size_t)nx * nx + ny * ny + (size_t)n_sites * (nx + ny) + 2 * E + npc) * sizeof(T);
  b += 2 * (size_t)npc * nterms * sizeof(int);
  return b + 64;
}

template <typename T>
__device__ __forceinline__ HeomSmem<T> heom_carve(unsigned char* raw, const HeomP& p, int npc) {
  using C = typename cplx<T>::type;
  HeomSmem<T> s;
  s.x = (C*)raw;
  s.al = s.x + npc * p.E;
  s.be = s.al + npc * p.nterms;
  s.ga = s.be + npc * p.nterms;
  s.Hx = (T*)(s.ga + npc * p.nterms);
  s.Hy = s.Hx + p.nx * p.nx;
  s.ox = s.Hy + p.ny * p.ny;
  s.oy = s.ox + p.n_sites * p.nx;
  s.W = s.oy + p.n_sites * p.ny;
  s.Wr = s.W + p.E;
  s.shift = s.Wr + p.E;
  s.nbr = (int*)(s.shift + npc);
  s.site = s.nbr + npc * p.nterms;
  return s;
}

template <typename T>
__device__ __forceinline__ void heom_stage_smem(const HeomP& p, const typename cplx<T>::type* x,
                                                int64_t b, int n0, int npc, HeomSmem<T>& s) {
  using C = typename cplx<T>::type;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nn = (npc < p.nnodes - n0 ? npc : p.nnodes - n0);
    for (int i = tid; i < p.nx * p.nx; i += nt) s.Hx[i] = p.Hx[b * p.Hx_stride + i];
    for (int i = tid; i < p.ny * p.ny; i += nt) s.Hy[i] = p.Hy[b * p.Hy_stride + i];
    for (int i = tid; i < p.n_sites * p.nx; i += nt) s.ox[i] = p.occx[i];
    for (int i = tid; i < p.n_sites * p.ny; i += nt) s.oy[i] = p.occy[i];
    for (int i = tid; i < p.E; i += nt) s.W[i] = p.W ? p.W[i] : 0.0;
    for (int i = tid; i < p.E; i += nt) s.Wr[i] = p.Wraw ? p.Wraw[i] : 0.0;
    for (int i = tid; i < npc; i += nt) s.shift[i] = i < nn ? p.shift[n0 + i] : 0.0;
  for (int i = tid; i < npc * p.nterms; i += nt) {
    const bool ok = i < nn * p.nterms;
    const int g = n0 * p.nterms + i;
    s.nbr[i] = ok ? p.nbr[g] : -1;
    s.site[i] = ok ? p.site[g] : 0;
    s.al[i] = ok ? p.alpha[g] : make_double2(0.0, 0.0);
    s.be[i] = ok ? p.beta[g] : make_double2(0.0, 0.0);
    s.ga[i] = (ok && p.gamma) ? p.gamma[g] : make_double2(0.0, 0.0);
  }
  const C* xb = x + (b * p.nnodes + n0) * (int64_t)p.E;
  for (int i = tid; i < nn * p.E; i += nt) s.x[i] = xb[i];
  __syncthreads();
}

// k = RHS(x) for element e of local node `local` (global `node`) of sample b.
template <typename T>
__device__ __forceinline__ void heom_rhs_elem(const HeomP& p, const typename cplx<T>::type* x,
                                              int64_t b, int local, int e, const HeomSmem<T>& s,
                                              typename cplx<T>::type& out) {
  using C = typename cplx<T>::type;
  const int a = e % p.nx, bb = e / p.nx;
  const C* xs = s.x + local * p.E;
  // commutator: -i (Hx x - x Hy)[a][bb]
  T cr = 0, ci = 0;
  for (int c = 0; c < p.nx; ++c) {
    const T hv = s.Hx[a * p.nx + c];
    const C v = xs[c + p.nx * bb];
    cr = fma(hv, v.x, cr);
    ci = fma(hv, v.y, ci);
  }
  for (int c = 0; c < p.ny; ++c) {
    const T hv = s.Hy[c * p.ny + bb];
    const C v = xs[a + p.nx * c];
    cr = fma(-hv, v.x, cr);
    ci = fma(-hv, v.y, ci);
  }
  // -i (cr + i ci) = ci - i cr
  const C self = xs[e];
  T orr = ci, oi = -cr;
  const T sh = s.shift[local] + s.W[e];
  orr = fma(-sh, self.x, orr);
  oi = fma(-sh, self.y, oi);
  const C* xb = x + b * (int64_t)p.nnodes * p.E;
  const int base = local * p.nterms;
  // every term of the node, the same sequence in every lane of a warp (the
  // lanes serve one node), so each neighbour load is one coalesced access;
  // a term of site j weighs occ_j(a) alpha + occ_j(b) beta
  for (int t = 0; t < p.nterms; ++t) {
    const int nb = s.nbr[base + t];
    if (nb < 0) break;
    const int j = s.site[base + t];
    const C al = s.al[base + t], be = s.be[base + t], ga = s.ga[base + t];
    const T oa = s.ox[j * p.nx + a], ob = s.oy[j * p.ny + bb];
    const T gw = s.Wr[e] * (oa - ob);
    const T fr = al.x * oa + be.x * ob + ga.x * gw, fi = al.y * oa + be.y * ob + ga.y * gw;
    const C v = xb[(int64_t)nb * p.E + e];
    orr = fma(fr, v.x, fma(-fi, v.y, orr));
    oi = fma(fr, v.y, fma(fi, v.x, oi));
  }
  const T uc = (T)p.uc;
  out.x = uc * orr;
  out.y = uc * oi;
}

// ------------------------------------------- per-stage form, warp per node
// One warp per node block and stage, no block-wide staging: the lanes own
// the elements e = lane + 32 i of the block, the Hamiltonians, occupations
// and weights are read through the L1 (a few hundred bytes shared by every
// warp), the node's own block goes through a warp-private slice of shared
// memory for the commutator, and the term table is read one packed record at
// a time (the same address in every lane: one broadcast).  Each warp walks a
// contiguous range of (sample, node) blocks, so the warps of a CTA touch
// neighbouring nodes and their neighbour reads share the L1.
template <typename T>
struct __align__(16) HTerm;
template <>
struct __align__(16) HTerm<float> {
  int nbr, site;
  float2 al, be, ga;
};
template <>
struct __align__(16) HTerm<double> {
  int nbr, site, pad0, pad1;
  double2 al, be, ga;
};

template <typename T>
__global__ void heom_pack_terms_kernel(const int* __restrict__ nbr, const int* __restrict__ site,
                                       const double2* __restrict__ alpha,
                                       const double2* __restrict__ beta,
                                       const double2* __restrict__ gamma, int64_t n,
                                       HTerm<T>* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  HTerm<T> r;
  r.nbr = nbr[i];
  r.site = site[i];
  const double2 a = alpha[i], b = beta[i];
  const double2 g = gamma ? gamma[i] : make_double2(0.0, 0.0);
  r.al = cmk((T)a.x, (T)a.y);
  r.be = cmk((T)b.x, (T)b.y);
  r.ga = cmk((T)g.x, (T)g.y);
  if constexpr (sizeof(T) == 8) r.pad0 = r.pad1 = 0;
  out[i] = r;
}

struct HeomWP {
  int nx, ny, E, nnodes, nterms, n_sites, per_warp;
  int64_t items;              // batch * nnodes
  int64_t Hx_stride, Hy_stride;
  const void* Hx;             // T tables (FP32 copies in the FP32 form)
  const void* Hy;
  const void* occx;
  const void* occy;
  const void* W;              // or null
  const void* Wraw;           // or null
  const void* shift;
  const void* terms;          // HTerm<T> [nnodes][nterms]
  const void* site_terms;     // HTerm<T> [nnodes][n_sites][site_slots], grouped by site, or null
  int site_slots;             // max(nterms, 2)
  int has_gamma;
  double uc, h;
};

template <typename T>
__device__ __forceinline__ void load_term(const HTerm<T>* r, int& nbr, int& site,
                                          typename cplx<T>::type& al,
                                          typename cplx<T>::type& be,
                                          typename cplx<T>::type& ga) {
  if constexpr (sizeof(T) == 4) {
    const int4 a = __ldg(reinterpret_cast<const int4*>(r));
    const float4 b = __ldg(reinterpret_cast<const float4*>(r) + 1);
    nbr = a.x;
    site = a.y;
    al = make_float2(__int_as_float(a.z), __int_as_float(a.w));
    be = make_float2(b.x, b.y);
    ga = make_float2(b.z, b.w);
  } else {
    const int4 a = __ldg(reinterpret_cast<const int4*>(r));
    nbr = a.x;
    site = a.y;
    al = __ldg(reinterpret_cast<const double2*>(r) + 1);
    be = __ldg(reinterpret_cast<const double2*>(r) + 2);
    ga = __ldg(reinterpret_cast<const double2*>(r) + 3);
  }
}

// RK4 bookkeeping of one element after its stage derivative k: stages 0..2
// accumulate k and write the next stage input, stage 3 adds h/6 (acc + k) to
// the state (split-word in FP32).
template <typename T>
__device__ __forceinline__ void heom_rk4_update(int stage, int64_t idx,
                                                typename cplx<T>::type k, T h,
                                                typename cplx<T>::type* yh,
                                                typename cplx<T>::type* yl,
                                                typename cplx<T>::type* acc,
                                                typename cplx<T>::type* next) {
  using Cx = typename cplx<T>::type;
  if (stage == 0) {
    acc[idx] = k;
    const Cx y = yh[idx];
    next[idx] = cmk(y.x + (T)0.5 * h * k.x, y.y + (T)0.5 * h * k.y);
  } else if (stage < 3) {
    const Cx a = acc[idx];
    acc[idx] = cmk(a.x + (T)2 * k.x, a.y + (T)2 * k.y);
    const Cx y = yh[idx];
    const T c = stage == 1 ? (T)0.5 * h : h;
    next[idx] = cmk(y.x + c * k.x, y.y + c * k.y);
  } else {
    const Cx a = acc[idx];
    const T s6 = h / (T)6;
    const T ix = s6 * (a.x + k.x), iy = s6 * (a.y + k.y);
    const Cx y = yh[idx];
    if constexpr (sizeof(T) == 4) {
      const Cx l = yl[idx];
      float hx = y.x, lx = l.x, hy = y.y, ly = l.y;
      dd_add(hx, lx, ix);
      dd_add(hy, ly, iy);
      yh[idx] = cmk(hx, hy);
      yl[idx] = cmk(lx, ly);
    } else {
      yh[idx] = cmk(y.x + ix, y.y + iy);
    }
  }
}

// Any block shape (nx * ny <= 256): EPL elements per lane.
template <typename T, int EPL>
__global__ void __launch_bounds__(256)
    heom_warp_stage_kernel(HeomWP p, int stage, const typename cplx<T>::type* __restrict__ in,
                           typename cplx<T>::type* yh, typename cplx<T>::type* __restrict__ yl,
                           typename cplx<T>::type* __restrict__ acc,
                           typename cplx<T>::type* __restrict__ next) {
  using Cx = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  Cx* xs = reinterpret_cast<Cx*>(smraw) + (size_t)wib * 32 * EPL;
  const int64_t warp = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
  const int64_t i0 = warp * p.per_warp;
  const int64_t i1 = min(p.items, i0 + p.per_warp);
  const int E = p.E, nx = p.nx, ny = p.ny, nt = p.nterms;
  const T* Hx0 = (const T*)p.Hx;
  const T* Hy0 = (const T*)p.Hy;
  const T* ox = (const T*)p.occx;
  const T* oy = (const T*)p.occy;
  const T* shift = (const T*)p.shift;
  const HTerm<T>* terms = (const HTerm<T>*)p.terms;
  const T uc = (T)p.uc, h = (T)p.h;
  // the lane's elements: indices and the per-element weights
  int ea[EPL], eb[EPL];
  T w[EPL], wr[EPL];
#pragma unroll
  for (int u = 0; u < EPL; ++u) {
    const int e = lane + 32 * u;
    const int ec = e < E ? e : 0;
    ea[u] = ec % nx;
    eb[u] = ec / nx;
    w[u] = p.W ? __ldg((const T*)p.W + ec) : (T)0;
    wr[u] = p.Wraw ? __ldg((const T*)p.Wraw + ec) : (T)0;
  }
  for (int64_t it = i0; it < i1; ++it) {
    const int64_t b = it / p.nnodes;
    const int n = (int)(it - b * p.nnodes);
    const Cx* xb = in + b * (int64_t)p.nnodes * E;
    const T* Hx = Hx0 + b * p.Hx_stride;
    const T* Hy = Hy0 + b * p.Hy_stride;
    Cx self[EPL];
#pragma unroll
    for (int u = 0; u < EPL; ++u) {
      const int e = lane + 32 * u;
      self[u] = cmk((T)0, (T)0);
      if (e < E) {
        self[u] = xb[(int64_t)n * E + e];
        xs[e] = self[u];
      }
    }
    __syncwarp();
    const T sh = __ldg(shift + n);
    T orr[EPL], oi[EPL];
#pragma unroll
    for (int u = 0; u < EPL; ++u) {
      const int a = ea[u], bb = eb[u];
      // -i (Hx x - x Hy)[a][bb]
      T cr = 0, ci = 0;
      for (int c = 0; c < nx; ++c) {
        const T hv = __ldg(Hx + a * nx + c);
        const Cx v = xs[c + nx * bb];
        cr = fma(hv, v.x, cr);
        ci = fma(hv, v.y, ci);
      }
      for (int c = 0; c < ny; ++c) {
        const T hv = __ldg(Hy + c * ny + bb);
        const Cx v = xs[a + nx * c];
        cr = fma(-hv, v.x, cr);
        ci = fma(-hv, v.y, ci);
      }
      const T d = sh + w[u];
      orr[u] = fma(-d, self[u].x, ci);
      oi[u] = fma(-d, self[u].y, -cr);
    }
    // couplings: every term of the node in the same order in all lanes
    const HTerm<T>* tr = terms + (int64_t)n * nt;
    for (int t = 0; t < nt; ++t) {
      int m, j;
      Cx al, be, ga;
      load_term<T>(tr + t, m, j, al, be, ga);
      if (m < 0) continue;
      const Cx* xm = xb + (int64_t)m * E;
#pragma unroll
      for (int u = 0; u < EPL; ++u) {
        const int e = lane + 32 * u;
        if (e >= E) continue;
        const Cx v = xm[e];
        const T oa = __ldg(ox + j * nx + ea[u]), ob = __ldg(oy + j * ny + eb[u]);
        T fr = al.x * oa + be.x * ob, fi = al.y * oa + be.y * ob;
        if (p.has_gamma) {
          const T gw = wr[u] * (oa - ob);
          fr = fma(ga.x, gw, fr);
          fi = fma(ga.y, gw, fi);
        }
        orr[u] = fma(fr, v.x, fma(-fi, v.y, orr[u]));
        oi[u] = fma(fr, v.y, fma(fi, v.x, oi[u]));
      }
    }
#pragma unroll
    for (int u = 0; u < EPL; ++u) {
      const int e = lane + 32 * u;
      if (e >= E) continue;
      heom_rk4_update<T>(stage, (b * p.nnodes + n) * (int64_t)E + e,
                         cmk(uc * orr[u], uc * oi[u]), h, yh, yl, acc, next);
    }
    __syncwarp();   // the block slice is rewritten by the next node
  }
}

// Blocks of at most 8 x 8 (every one-exciton hierarchy up to 8 sites): two
// elements per lane, the lane's rows of Hx and columns of Hy in registers
// (reloaded when the sample changes), the term loop four terms at a time so
// eight neighbour loads per lane are in flight, and independent accumulator
// chains in the commutator.  NB = 8 fixes the block at 8 x 8 at compile time;
// NB = 0 takes nx, ny <= 8 at run time.
template <typename T, int NB, int G, int MINB>
__global__ void __launch_bounds__(256, MINB)
    heom_warp_small_kernel(HeomWP p, int stage, const typename cplx<T>::type* __restrict__ in,
                           typename cplx<T>::type* yh, typename cplx<T>::type* __restrict__ yl,
                           typename cplx<T>::type* __restrict__ acc,
                           typename cplx<T>::type* __restrict__ next) {
  using Cx = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nx = NB ? NB : p.nx, ny = NB ? NB : p.ny, E = NB ? NB * NB : p.E;
  const int nt = p.nterms, N = p.n_sites, nnodes = p.nnodes;
  Cx* xs = reinterpret_cast<Cx*>(smraw) + (size_t)wib * 64;
  T* sox = reinterpret_cast<T*>(reinterpret_cast<Cx*>(smraw) + (size_t)(blockDim.x >> 5) * 64);
  T* soy = sox + N * nx;
  for (int i = threadIdx.x; i < N * nx; i += blockDim.x) sox[i] = ((const T*)p.occx)[i];
  for (int i = threadIdx.x; i < N * ny; i += blockDim.x) soy[i] = ((const T*)p.occy)[i];
  __syncthreads();
  const int64_t warp = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
  const int64_t i0 = warp * p.per_warp;
  const int64_t i1 = min(p.items, i0 + p.per_warp);
  if (i0 >= i1) return;
  const T* shift = (const T*)p.shift;
  const HTerm<T>* terms = (const HTerm<T>*)p.terms;
  const T uc = (T)p.uc, h = (T)p.h;
  int ea[2], eb[2];
  bool ev[2];
  T w[2], wr[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int e = lane + 32 * u;
    ev[u] = e < E;
    const int ec = ev[u] ? e : 0;
    ea[u] = ec % nx;
    eb[u] = ec / nx;
    w[u] = p.W ? __ldg((const T*)p.W + ec) : (T)0;
    wr[u] = p.Wraw ? __ldg((const T*)p.Wraw + ec) : (T)0;
  }
  // (sample, node) of the first item; later items step through them
  int64_t b = i0 / nnodes;
  int n = (int)(i0 - b * nnodes);
  T hx[2][8], hy[2][8];
  const Cx* xb = nullptr;
  bool fresh = true;
  for (int64_t it = i0; it < i1; ++it) {
    if (fresh) {
      fresh = false;
      xb = in + b * (int64_t)nnodes * E;
      const T* Hx = (const T*)p.Hx + b * p.Hx_stride;
      const T* Hy = (const T*)p.Hy + b * p.Hy_stride;
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          // at 8 x 8 both elements of a lane share the row a (e and e + 32)
          hx[u][c] = c < nx ? __ldg(Hx + ea[NB == 8 ? 0 : u] * nx + c) : (T)0;
          hy[u][c] = c < ny ? __ldg(Hy + c * ny + eb[u]) : (T)0;
        }
    }
    const int64_t base = it * E;
    const Cx* xn = xb + n * E + lane;
    Cx self[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      self[u] = cmk((T)0, (T)0);
      if (ev[u]) {
        self[u] = xn[32 * u];
        xs[lane + 32 * u] = self[u];
      }
    }
    const HTerm<T>* tr = terms + n * nt;
    int gm[G], gj[G];
    Cx gal[G], gbe[G], gga[G], gv[G][2];
    auto load_group = [&](int t0) {
#pragma unroll
      for (int q = 0; q < G; ++q) {
        gm[q] = -1;
        gj[q] = 0;
        if (t0 + q < nt) load_term<T>(tr + t0 + q, gm[q], gj[q], gal[q], gbe[q], gga[q]);
      }
#pragma unroll
      for (int q = 0; q < G; ++q) {
        const Cx* xm = xb + (gm[q] < 0 ? 0 : gm[q]) * E + lane;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          gv[q][u] = cmk((T)0, (T)0);
          if (gm[q] >= 0 && ev[u]) gv[q][u] = xm[32 * u];
        }
      }
    };
    T orr[2], oi[2];
    auto use_group = [&]() {
#pragma unroll
      for (int q = 0; q < G; ++q) {
        if (gm[q] < 0) continue;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const T oa = sox[gj[q] * nx + ea[u]], ob = soy[gj[q] * ny + eb[u]];
          T fr = gal[q].x * oa + gbe[q].x * ob, fi = gal[q].y * oa + gbe[q].y * ob;
          if (p.has_gamma) {
            const T gw = wr[u] * (oa - ob);
            fr = fma(gga[q].x, gw, fr);
            fi = fma(gga[q].y, gw, fi);
          }
          orr[u] = fma(fr, gv[q][u].x, fma(-fi, gv[q][u].y, orr[u]));
          oi[u] = fma(fr, gv[q][u].y, fma(fi, gv[q][u].x, oi[u]));
        }
      }
    };
    load_group(0);
    // RK4 operands, then the commutator while the neighbour loads fly
    Cx yv[2], av[2], lv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      yv[u] = av[u] = lv[u] = cmk((T)0, (T)0);
      if (ev[u]) {
        yv[u] = yh[base + lane + 32 * u];
        if (stage > 0) av[u] = acc[base + lane + 32 * u];
        if constexpr (sizeof(T) == 4) {
          if (stage == 3) lv[u] = yl[base + lane + 32 * u];
        }
      }
    }
    __syncwarp();
    const T sh = __ldg(shift + n);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      // -i (Hx x - x Hy)[a][bb] in four independent chains
      T c0 = 0, s0 = 0, c1 = 0, s1 = 0;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        if (c < nx) {
          const Cx xv = xs[c + nx * eb[u]];
          c0 = fma(hx[u][c], xv.x, c0);
          s0 = fma(hx[u][c], xv.y, s0);
        }
        if (c < ny) {
          const Cx xv = xs[ea[u] + nx * c];
          c1 = fma(hy[u][c], xv.x, c1);
          s1 = fma(hy[u][c], xv.y, s1);
        }
      }
      const T d = sh + w[u];
      orr[u] = fma(-d, self[u].x, s0 - s1);
      oi[u] = fma(-d, self[u].y, c1 - c0);
    }
    use_group();
    for (int t0 = G; t0 < nt; t0 += G) {
      load_group(t0);
      use_group();
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (!ev[u]) continue;
      const Cx k = cmk(uc * orr[u], uc * oi[u]);
      const int64_t idx = base + lane + 32 * u;
      if (stage == 0) {
        acc[idx] = k;
        next[idx] = cmk(yv[u].x + (T)0.5 * h * k.x, yv[u].y + (T)0.5 * h * k.y);
      } else if (stage < 3) {
        acc[idx] = cmk(av[u].x + (T)2 * k.x, av[u].y + (T)2 * k.y);
        const T c = stage == 1 ? (T)0.5 * h : h;
        next[idx] = cmk(yv[u].x + c * k.x, yv[u].y + c * k.y);
      } else {
        const T s6 = h / (T)6;
        const T ix = s6 * (av[u].x + k.x), iy = s6 * (av[u].y + k.y);
        if constexpr (sizeof(T) == 4) {
          float hx_ = yv[u].x, lx = lv[u].x, hy_ = yv[u].y, ly = lv[u].y;
          dd_add(hx_, lx, ix);
          dd_add(hy_, ly, iy);
          yh[idx] = cmk(hx_, hy_);
          yl[idx] = cmk(lx, ly);
        } else {
          yh[idx] = cmk(yv[u].x + ix, yv[u].y + iy);
        }
      }
    }
    if (++n == nnodes) {
      n = 0;
      ++b;
      fresh = true;
    }
    __syncwarp();   // the block slice is rewritten by the next node
  }
}

// ------------------------------ per-stage form, coupling terms by site
// The coupling of element (a, b) of node n is
//   sum_t (alpha_t occx[j_t][a] + beta_t occy[j_t][b]
//          + gamma_t Wraw[a][b] (occx[j_t][a] - occy[j_t][b])) rho_{nbr_t}[a][b],
// so only the terms whose site j_t couples to row a or to column b
// contribute.  With the site number operators of one-exciton states that is
// one site each: the terms of a node are packed once per call, grouped by
// site ([node][slot][site] records, at least two slots, padded with nbr = -1;
// each record's `site` field holds the number of records of its (node,
// site), since the kernel knows the site).  A warp copies a node's first two
// slots of every site (contiguous) into its shared-memory slice with
// coalesced 16-byte loads, and each
// lane visits only its own sites' terms instead of every term of the node,
// with the neighbour loads of both its elements in flight together.  A lane
// whose row or column couples to more than one site takes the full term
// loop.
template <typename T>
__global__ void heom_pack_site_terms_kernel(const HTerm<T>* __restrict__ terms, int nnodes,
                                            int nterms, int n_sites, int slots,
                                            HTerm<T>* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;   // (node, site)
  if (i >= (int64_t)nnodes * n_sites) return;
  const int n = (int)(i / n_sites), j = (int)(i - (int64_t)n * n_sites);
  const HTerm<T>* tr = terms + (int64_t)n * nterms;
  HTerm<T>* o = out + (int64_t)n * slots * n_sites + j;   // slot k at o[k * n_sites]
  int c = 0;
  for (int t = 0; t < nterms; ++t)
    if (tr[t].nbr >= 0 && tr[t].site == j) ++c;
  int k = 0;
  for (int t = 0; t < nterms; ++t) {
    HTerm<T> r = tr[t];
    if (r.nbr >= 0 && r.site == j) {
      r.site = c;
      o[(int64_t)(k++) * n_sites] = r;
    }
  }
  for (; k < slots; ++k) {
    HTerm<T> r = {};
    r.nbr = -1;
    r.site = c;
    o[(int64_t)k * n_sites] = r;
  }
}

// two-wide multiply-add a * b + c per component: one packed FFMA2 in FP32
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ double2 pfma(double2 a, double2 b, double2 c) {
  return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ double2 pmul(double2 a, double2 b) {
  return make_double2(a.x * b.x, a.y * b.y);
}

template <typename T, int NB, int MINB>
__global__ void __launch_bounds__(256, MINB)
    heom_warp_site_kernel(HeomWP p, int stage, const typename cplx<T>::type* __restrict__ in,
                          typename cplx<T>::type* yh, typename cplx<T>::type* __restrict__ yl,
                          typename cplx<T>::type* __restrict__ acc,
                          typename cplx<T>::type* __restrict__ next) {
  using Cx = typename cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nx = NB ? NB : p.nx, ny = NB ? NB : p.ny, E = NB ? NB * NB : p.E;
  const int nt = p.nterms, N = p.n_sites, nnodes = p.nnodes;
  // per warp, twice (the node in work and the next one, copied in by
  // cp.async while this one computes): the node's first two coupling slots
  // of every site (2 N records) and its node block (64 complex); then the
  // occupations
  const int nw = blockDim.x >> 5;
  HTerm<T>* hrec2 = reinterpret_cast<HTerm<T>*>(smraw) + (size_t)wib * 4 * N;
  Cx* xs2 = reinterpret_cast<Cx*>(reinterpret_cast<HTerm<T>*>(smraw) + (size_t)nw * 4 * N) +
            (size_t)wib * 128;
  T* sox = reinterpret_cast<T*>(reinterpret_cast<Cx*>(reinterpret_cast<HTerm<T>*>(smraw) +
                                                      (size_t)nw * 4 * N) +
                                (size_t)nw * 128);
  T* soy = sox + N * nx;
  for (int i = threadIdx.x; i < N * nx; i += blockDim.x) sox[i] = ((const T*)p.occx)[i];
  for (int i = threadIdx.x; i < N * ny; i += blockDim.x) soy[i] = ((const T*)p.occy)[i];
  __syncthreads();
  const int64_t warp = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
  const int64_t i0 = warp * p.per_warp;
  const int64_t i1 = min(p.items, i0 + p.per_warp);
  if (i0 >= i1) return;
  const T* shift = (const T*)p.shift;
  const HTerm<T>* terms = (const HTerm<T>*)p.terms;
  const HTerm<T>* sterms = (const HTerm<T>*)p.site_terms;
  const int slots = p.site_slots;
  const int hchunks = 2 * N * (int)sizeof(HTerm<T>) / 16;   // 16-byte pieces of the head
  const T uc = (T)p.uc, h = (T)p.h;
  int ea[2], eb[2];
  bool ev[2];
  T w[2], wr[2];
  // the site of row a and, when it differs, the site of column b for each of
  // this lane's elements; `full` when a row or column couples to more than
  // one site (those lanes take every term)
  int js[2][2];
  bool full[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int e = lane + 32 * u;
    ev[u] = e < E;
    const int ec = ev[u] ? e : 0;
    ea[u] = ec % nx;
    eb[u] = ec / nx;
    w[u] = p.W ? __ldg((const T*)p.W + ec) : (T)0;
    wr[u] = p.Wraw ? __ldg((const T*)p.Wraw + ec) : (T)0;
    int na = 0, nb = 0, ja = -1, jb = -1;
    for (int j = 0; j < N; ++j) {
      if (sox[j * nx + ea[u]] != (T)0) {
        ja = j;
        ++na;
      }
      if (soy[j * ny + eb[u]] != (T)0) {
        jb = j;
        ++nb;
      }
    }
    full[u] = na > 1 || nb > 1;
    js[u][0] = ja;
    js[u][1] = jb != ja ? jb : -1;
  }
  const bool any_full = __any_sync(0xffffffffu, full[0] || full[1]);
  int64_t b = i0 / nnodes;
  int n = (int)(i0 - b * nnodes);
  // node (bb, nn): its head records and block into buffer `buf`
  auto prefetch = [&](int64_t bb, int nn, int buf) {
    const char* src = reinterpret_cast<const char*>(sterms + (int64_t)nn * slots * N);
    const uint32_t dh = (uint32_t)__cvta_generic_to_shared(hrec2 + buf * 2 * N);
    for (int c = lane; c < hchunks; c += 32)
      asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dh + 16u * c),
                   "l"(src + 16 * c)
                   : "memory");
    const Cx* xsrc = in + (bb * nnodes + nn) * (int64_t)E + lane;
    const uint32_t dx = (uint32_t)__cvta_generic_to_shared(xs2 + buf * 64 + lane);
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (ev[u]) {
        if constexpr (sizeof(Cx) == 8)
          asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dx + 8u * 32 * u),
                       "l"(xsrc + 32 * u)
                       : "memory");
        else
          asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(dx + 16u * 32 * u),
                       "l"(xsrc + 32 * u)
                       : "memory");
      }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  prefetch(b, n, 0);
  int buf = 0;
  T hx[2][8], hy[2][8];
  const Cx* xb = nullptr;
  bool fresh = true;
  for (int64_t it = i0; it < i1; ++it, buf ^= 1) {
    // this node's copies have landed (every lane's), then the next node's
    // are issued into the other buffer
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncwarp();
    if (it + 1 < i1) {
      const bool wrap = n + 1 == nnodes;
      prefetch(wrap ? b + 1 : b, wrap ? 0 : n + 1, buf ^ 1);
    }
    const HTerm<T>* hrec = hrec2 + buf * 2 * N;
    const Cx* xs = xs2 + buf * 64;
    if (fresh) {
      fresh = false;
      xb = in + b * (int64_t)nnodes * E;
      const T* Hx = (const T*)p.Hx + b * p.Hx_stride;
      const T* Hy = (const T*)p.Hy + b * p.Hy_stride;
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          hx[u][c] = c < nx ? __ldg(Hx + ea[NB == 8 ? 0 : u] * nx + c) : (T)0;
          // negated: the commutator sums Hx x - x Hy in one accumulator
          hy[u][c] = c < ny ? -__ldg(Hy + c * ny + eb[u]) : (T)0;
        }
    }
    const int64_t base = it * E;
    Cx self[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) self[u] = ev[u] ? xs[lane + 32 * u] : cmk((T)0, (T)0);
    Cx yv[2], av[2], lv[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      yv[u] = av[u] = lv[u] = cmk((T)0, (T)0);
      if (ev[u]) {
        yv[u] = yh[base + lane + 32 * u];
        if (stage > 0) av[u] = acc[base + lane + 32 * u];
        if constexpr (sizeof(T) == 4) {
          if (stage == 3) lv[u] = yl[base + lane + 32 * u];
        }
      }
    }
    // the coupling terms of this lane's sites: the first two terms of each
    // site (coefficient and neighbour node) for both elements, then every
    // neighbour load in flight together.  Complex sums in packed two-wide
    // multiply-adds: o += f v as o += f.x (v.x, v.y) + (-f.y, f.y) (v.y, v.x)
    Cx o[2] = {cmk((T)0, (T)0), cmk((T)0, (T)0)};
    auto coef = [&](int u, int j, const HTerm<T>& r) -> Cx {
      const T oa = sox[j * nx + ea[u]], ob = soy[j * ny + eb[u]];
      Cx f = pfma(r.be, cmk(ob, ob), pmul(r.al, cmk(oa, oa)));
      if (p.has_gamma) {
        const T gw = wr[u] * (oa - ob);
        f = pfma(r.ga, cmk(gw, gw), f);
      }
      return f;
    };
    auto cmac = [](Cx& acc_, Cx f, Cx v) {
      acc_ = pfma(cmk(f.x, f.x), v, acc_);
      acc_ = pfma(cmk(-f.y, f.y), cmk(v.y, v.x), acc_);
    };
    int cnt[2][2], nbi[2][2][2];
    Cx cf[2][2][2];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const bool on = ev[u] && !full[u] && js[u][q] >= 0;
        cnt[u][q] = 0;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          nbi[u][q][r] = -1;
          cf[u][q][r] = cmk((T)0, (T)0);
          if (on) {
            // the first two slots always exist (padding: nbr = -1)
            const HTerm<T> rec = hrec[r * N + js[u][q]];
            cnt[u][q] = rec.site;
            nbi[u][q][r] = rec.nbr;
            if (rec.nbr >= 0) cf[u][q][r] = coef(u, js[u][q], rec);
          }
        }
      }
    Cx nv[2][2][2];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int r = 0; r < 2; ++r)
          nv[u][q][r] = nbi[u][q][r] >= 0 ? xb[(int64_t)nbi[u][q][r] * E + lane + 32 * u]
                                          : cmk((T)0, (T)0);
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int q = 0; q < 2; ++q)
#pragma unroll
        for (int r = 0; r < 2; ++r) cmac(o[u], cf[u][q][r], nv[u][q][r]);
    // sites with more than two terms (several exponents per bath)
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
      for (int q = 0; q < 2; ++q)
        for (int r = 2; r < cnt[u][q]; ++r) {
          HTerm<T> rq;
          load_term<T>(sterms + ((int64_t)n * slots + r) * N + js[u][q], rq.nbr, rq.site, rq.al,
                       rq.be, rq.ga);
          cmac(o[u], coef(u, js[u][q], rq), xb[(int64_t)rq.nbr * E + lane + 32 * u]);
        }
    if (any_full) {
      // lanes whose row or column couples to more than one site: every term
      const HTerm<T>* tr = terms + (int64_t)n * nt;
      for (int t = 0; t < nt; ++t) {
        HTerm<T> rq;
        load_term<T>(tr + t, rq.nbr, rq.site, rq.al, rq.be, rq.ga);
        if (rq.nbr < 0) continue;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          if (!(ev[u] && full[u])) continue;
          cmac(o[u], coef(u, rq.site, rq), xb[(int64_t)rq.nbr * E + lane + 32 * u]);
        }
      }
    }
    __syncwarp();
    const T sh = __ldg(shift + n);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      // g = (Hx x - x Hy)[a][bb] in two packed chains (hy holds -Hy); the
      // step adds -i g - d x
      Cx g0 = cmk((T)0, (T)0), g1 = cmk((T)0, (T)0);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        if (c < nx) g0 = pfma(cmk(hx[u][c], hx[u][c]), xs[c + nx * eb[u]], g0);
        if (c < ny) g1 = pfma(cmk(hy[u][c], hy[u][c]), xs[ea[u] + nx * c], g1);
      }
      const T d = sh + w[u];
      o[u].x += fma(-d, self[u].x, g0.y + g1.y);
      o[u].y += fma(-d, self[u].y, -(g0.x + g1.x));
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (!ev[u]) continue;
      const Cx k = cmk(uc * o[u].x, uc * o[u].y);
      const int64_t idx = base + lane + 32 * u;
      if (stage == 0) {
        acc[idx] = k;
        next[idx] = cmk(yv[u].x + (T)0.5 * h * k.x, yv[u].y + (T)0.5 * h * k.y);
      } else if (stage < 3) {
        acc[idx] = cmk(av[u].x + (T)2 * k.x, av[u].y + (T)2 * k.y);
        const T c = stage == 1 ? (T)0.5 * h : h;
        next[idx] = cmk(yv[u].x + c * k.x, yv[u].y + c * k.y);
      } else {
        const T s6 = h / (T)6;
        const T ix = s6 * (av[u].x + k.x), iy = s6 * (av[u].y + k.y);
        if constexpr (sizeof(T) == 4) {
          float hx_ = yv[u].x, lx = lv[u].x, hy_ = yv[u].y, ly = lv[u].y;
          dd_add(hx_, lx, ix);
          dd_add(hy_, ly, iy);
          yh[idx] = cmk(hx_, hy_);
          yl[idx] = cmk(lx, ly);
        } else {
          yh[idx] = cmk(yv[u].x + ix, yv[u].y + iy);
        }
      }
    }
    if (++n == nnodes) {
      n = 0;
      ++b;
      fresh = true;
    }
    __syncwarp();   // this buffer is rewritten by the node after next
  }
}

// ------------------------- per-stage form, node commutators on the tensor cores
// FP32, blocks up to 8 x 8.  For a tile of up to 64 node blocks of one sample,
// the commutators vec(Hx rho - rho Hy) = L vec(rho),
//   L[(a,b),(c,d)] = Hx[a][c] d_bd - d_ac Hy[d][b]   (vec index a + nx b),
// are one tcgen05 product: A = the tile's blocks, one row per node and part
// (row 2k the real part of node k, row 2k + 1 its imaginary part; K = E
// padded to 8), B^T = L (N = E padded to 16), 3xTF32 (hi/lo TF32 split of
// both operands; lo is stored raw, the tensor core reads its leading TF32
// bits), FP32 accumulation in tensor memory.  L depends on the sample only
// and is rebuilt when a CTA's tile moves to another sample.  The accumulator
// rows go to shared memory as complex node blocks, and then, one warp per node
// block as in heom_warp_small_kernel, the lanes add -i uc (commutator),
// -(shift + W) rho and the coupling terms, and do the RK4 bookkeeping.
// Persistent CTAs, two per SM, stride over the tiles (measured against 32-node
// tiles with one tile per CTA: 643 against 720 ms for 64 samples x 1999
// steps); the completion wait is bounded (a timeout sets QSX_ERR_CUDA in
// *status and the CTA stops).
constexpr int HTC_NODES = 64;   // node blocks per tile: A rows 0 .. 2 HTC_NODES - 1

__device__ __forceinline__ void htc_split4(unsigned char* hi, unsigned char* lo, uint32_t off,
                                           float a, float b, float c, float d) {
  const float4 h = make_float4(tc::tf32_round(a), tc::tf32_round(b), tc::tf32_round(c),
                               tc::tf32_round(d));
  *reinterpret_cast<float4*>(hi + off) = h;
  *reinterpret_cast<float4*>(lo + off) = make_float4(a - h.x, b - h.y, c - h.z, d - h.w);
}

// shared-memory bytes: A hi/lo (128 x KP), B^T hi/lo (NP x KP), occupations,
// then the mbarrier and the tensor-memory address
__host__ __device__ inline size_t heom_tc_smem_bytes(int E, int n_sites, int nx, int ny) {
  const size_t kp = (E + 7) & ~7, np = (E + 15) & ~15;
  const size_t planes = 2 * (size_t)tc::ROWS * kp * 4 + 2 * np * kp * 4;
  return ((planes + (size_t)n_sites * (nx + ny) * 4 + 15) & ~(size_t)15) + 16;
}

__global__ void __launch_bounds__(256, 2)
    heom_tc_stage_kernel(HeomWP p, int stage, const float2* __restrict__ in, float2* yh,
                         float2* __restrict__ yl, float2* __restrict__ acc,
                         float2* __restrict__ next, int* status) {
  using namespace tc;
  using Cx = float2;
  constexpr int G = 4;
  extern __shared__ __align__(16) unsigned char smraw[];   // tcgen05 planes: 16-byte aligned
  const int nx = p.nx, ny = p.ny, E = p.E, N = p.n_sites, nnodes = p.nnodes, nt = p.nterms;
  const int kp = (E + 7) & ~7, np = (E + 15) & ~15, kq = kp / 4;
  const uint32_t sbo = (uint32_t)kp * 32u;
  const uint32_t PA = ROWS * kp * 4, PB = np * kp * 4;
  unsigned char* a_hi = smraw;
  unsigned char* a_lo = a_hi + PA;
  unsigned char* b_hi = a_lo + PA;
  unsigned char* b_lo = b_hi + PB;
  Cx* S = reinterpret_cast<Cx*>(a_hi);   // [HTC_NODES][E] commutators, once the MMA is done
  float* sox = reinterpret_cast<float*>(b_lo + PB);
  float* soy = sox + N * nx;
  const size_t off_mbar = ((size_t)(2 * PA + 2 * PB) + (size_t)N * (nx + ny) * 4 + 15) & ~(size_t)15;
  uint64_t* mbar_p = reinterpret_cast<uint64_t*>(smraw + off_mbar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar_p + 1);
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mbar = (uint32_t)__cvta_generic_to_shared(mbar_p);

  for (int i = tid; i < N * nx; i += blockDim.x) sox[i] = ((const float*)p.occx)[i];
  for (int i = tid; i < N * ny; i += blockDim.x) soy[i] = ((const float*)p.occy)[i];
  for (uint32_t i = tid; i < 2 * PA / 16; i += blockDim.x)
    reinterpret_cast<uint4*>(a_hi)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    s_abort = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint64_t da_hi = smem_desc((uint32_t)__cvta_generic_to_shared(a_hi), sbo);
  const uint64_t da_lo = smem_desc((uint32_t)__cvta_generic_to_shared(a_lo), sbo);
  const uint64_t db_hi = smem_desc((uint32_t)__cvta_generic_to_shared(b_hi), sbo);
  const uint64_t db_lo = smem_desc((uint32_t)__cvta_generic_to_shared(b_lo), sbo);
  const uint32_t idesc = make_idesc(np);
  const int lg = warp & 3, c0 = 32 * (warp >> 2);
  const uint32_t taddr = tmem + ((uint32_t)(32 * lg) << 16) + (uint32_t)c0;

  // this lane's two elements of a node block
  int ea[2], eb[2];
  bool ev[2];
  float w[2], wr[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int e = lane + 32 * u;
    ev[u] = e < E;
    const int ec = ev[u] ? e : 0;
    ea[u] = ec % nx;
    eb[u] = ec / nx;
    w[u] = p.W ? __ldg((const float*)p.W + ec) : 0.f;
    wr[u] = p.Wraw ? __ldg((const float*)p.Wraw + ec) : 0.f;
  }
  const float* shift = (const float*)p.shift;
  const HTerm<float>* terms = (const HTerm<float>*)p.terms;
  const float uc = (float)p.uc, h = (float)p.h;

  const int tiles_per = (nnodes + HTC_NODES - 1) / HTC_NODES;
  const int64_t ntiles = (p.items / nnodes) * tiles_per;
  int64_t cur_b = -1;
  uint32_t parity = 0;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t b = t / tiles_per;
    const int n0 = (int)(t - b * tiles_per) * HTC_NODES;
    const int nn = min(HTC_NODES, nnodes - n0);
    const Cx* xb = in + b * (int64_t)nnodes * E;   // the sample's stage input
    __syncthreads();   // the previous tile's warps are done with the staging
    // A: node k's real part in row 2k, imaginary part in row 2k + 1
    for (int g = tid; g < HTC_NODES * kq; g += blockDim.x) {
      const int k = g / kq, e0 = 4 * (g - k * kq);
      float re[4], im[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int e = e0 + q;
        const Cx v = (k < nn && e < E) ? xb[(int64_t)(n0 + k) * E + e] : make_float2(0.f, 0.f);
        re[q] = v.x;
        im[q] = v.y;
      }
      htc_split4(a_hi, a_lo, op_offset(2 * k, e0, sbo), re[0], re[1], re[2], re[3]);
      htc_split4(a_hi, a_lo, op_offset(2 * k + 1, e0, sbo), im[0], im[1], im[2], im[3]);
    }
    if (b != cur_b) {
      // B^T = L of sample b: row n = output element, column k = input element
      cur_b = b;
      const float* Hx = (const float*)p.Hx + b * p.Hx_stride;
      const float* Hy = (const float*)p.Hy + b * p.Hy_stride;
      for (int g = tid; g < np * kq; g += blockDim.x) {
        const int n = g / kq, k0 = 4 * (g - n * kq);
        float v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int k = k0 + q;
          float x = 0.f;
          if (n < E && k < E) {
            const int a = n % nx, bb = n / nx, c = k % nx, d = k / nx;
            if (bb == d) x = __ldg(Hx + a * nx + c);
            if (a == c) x -= __ldg(Hy + d * ny + bb);
          }
          v[q] = x;
        }
        htc_split4(b_hi, b_lo, op_offset(n, k0, sbo), v[0], v[1], v[2], v[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      issue_product(tmem, da_hi, da_lo, db_hi, db_lo, kp / 8, idesc, mbar);
      if (!wait_parity(mbar, parity)) {
        if (status) atomicOr(status, QSX_ERR_CUDA);
        s_abort = 1;
      }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (s_abort) break;
    parity ^= 1;
    {
      // accumulator lane 2k + part, columns c0 .. c0 + 31 -> S[k][e].part
      float v[32];
      tmem_load(taddr, v);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      const int L = 32 * lg + lane, k = L >> 1, part = L & 1;
      if (k < nn) {
        float* sk = reinterpret_cast<float*>(S + k * E) + part;
#pragma unroll
        for (int c = 0; c < 32; ++c)
          if (c0 + c < E) sk[2 * (c0 + c)] = v[c];
      }
    }
    __syncthreads();
    // one warp per node block: the rest of the generator and the RK4 step
    for (int k = warp; k < nn; k += blockDim.x >> 5) {
      const int n = n0 + k;
      const int64_t base = (b * (int64_t)nnodes + n) * E;
      const HTerm<float>* tr = terms + (int64_t)n * nt;
      int gm[G], gj[G];
      Cx gal[G], gbe[G], gga[G], gv[G][2];
      auto load_group = [&](int t0) {
#pragma unroll
        for (int q = 0; q < G; ++q) {
          gm[q] = -1;
          gj[q] = 0;
          if (t0 + q < nt) load_term<float>(tr + t0 + q, gm[q], gj[q], gal[q], gbe[q], gga[q]);
        }
#pragma unroll
        for (int q = 0; q < G; ++q) {
          const Cx* xm = xb + (int64_t)(gm[q] < 0 ? 0 : gm[q]) * E + lane;
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            gv[q][u] = make_float2(0.f, 0.f);
            if (gm[q] >= 0 && ev[u]) gv[q][u] = xm[32 * u];
          }
        }
      };
      float orr[2], oi[2];
      auto use_group = [&]() {
#pragma unroll
        for (int q = 0; q < G; ++q) {
          if (gm[q] < 0) continue;
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const float oa = sox[gj[q] * nx + ea[u]], ob = soy[gj[q] * ny + eb[u]];
            float fr = gal[q].x * oa + gbe[q].x * ob, fi = gal[q].y * oa + gbe[q].y * ob;
            if (p.has_gamma) {
              const float gw = wr[u] * (oa - ob);
              fr = fmaf(gga[q].x, gw, fr);
              fi = fmaf(gga[q].y, gw, fi);
            }
            orr[u] = fmaf(fr, gv[q][u].x, fmaf(-fi, gv[q][u].y, orr[u]));
            oi[u] = fmaf(fr, gv[q][u].y, fmaf(fi, gv[q][u].x, oi[u]));
          }
        }
      };
      load_group(0);
      const float sh = __ldg(shift + n);
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        orr[u] = oi[u] = 0.f;
        if (ev[u]) {
          const int e = lane + 32 * u;
          const Cx self = xb[(int64_t)n * E + e];
          const Cx cm = S[k * E + e];   // (Hx rho - rho Hy)[e]
          const float d = sh + w[u];
          orr[u] = fmaf(-d, self.x, cm.y);
          oi[u] = fmaf(-d, self.y, -cm.x);
        }
      }
      use_group();
      for (int t0 = G; t0 < nt; t0 += G) {
        load_group(t0);
        use_group();
      }
#pragma unroll
      for (int u = 0; u < 2; ++u)
        if (ev[u])
          heom_rk4_update<float>(stage, base + lane + 32 * u, make_float2(uc * orr[u], uc * oi[u]),
                                 h, yh, yl, acc, next);
    }
  }
  if (s_abort && tid == 0) wait_parity(mbar, parity);   // let an unfinished product drain
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
}

// ------------------------------------------------ persistent cluster form
// The whole RK4 loop in one launch: one thread-block cluster per disorder
// sample, the hierarchy nodes split into contiguous ranges over its C CTAs.
// Each CTA keeps the stage input of its nodes in shared memory, double
// buffered, and its elements' state (split-word in FP32) and RK4
// accumulator in registers; a node's commutator reads its own CTA's block,
// the coupling terms read the neighbour nodes' blocks through distributed
// shared memory.  One cluster barrier per stage publishes the stage input:
// a CTA writes the next stage's input into the other buffer, which no peer
// reads until after the next barrier.
struct HeomCP {
  int nx, ny, E, nnodes, nterms, n_sites, nsave, save_every, nsteps, keep;
  int csize, npcta;
  int64_t batch, Hx_stride, Hy_stride, y0_stride;
  const double* Hx;
  const double* Hy;
  const double* occx;
  const double* occy;
  const double* W;
  const double* shift;
  const int* nbr;
  const int* site;
  const double2* alpha;
  const double2* beta;
  const double2* gamma;
  const double* Wraw;
  double uc, h;
  const double2* y0;
  double2* saves;   // [batch][nsave][keep * E]
  int* status;
};

template <typename T>
__host__ __device__ inline size_t heom_cluster_smem_bytes(int nx, int ny, int n_sites, int E,
                                                          int npcta, int nterms) {
  using C = typename cplx<T>::type;
  size_t b = 2 * (size_t)npcta * E * sizeof(C);                        // stage inputs
  b += 3 * (size_t)npcta * nterms * sizeof(C);                         // alpha, beta, gamma
  b += ((size_t)nx * nx + ny * ny + (size_t)n_sites * (nx + ny) + 2 * E + npcta) * sizeof(T);
  b += 2 * (size_t)npcta * nterms * sizeof(int);                       // nbr, site
  return b + 64;
}

template <typename T, int EPT>
__global__ void __launch_bounds__(512, 1) heom_cluster_kernel(HeomCP p) {
  using Cx = typename cplx<T>::type;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int64_t smp = blockIdx.x / p.csize;
  const int E = p.E, nx = p.nx, ny = p.ny, N = p.n_sites, nt = p.nterms;
  const int node0 = rank * p.npcta;
  const int nloc = max(0, min(p.nnodes, node0 + p.npcta) - node0);
  const int Mloc = nloc * E;
  const int tid = threadIdx.x, bd = blockDim.x;

  extern __shared__ __align__(16) unsigned char smraw[];
  Cx* sx = (Cx*)smraw;                                  // [2][npcta E]
  Cx* sal = sx + 2 * (size_t)p.npcta * E;               // [npcta nterms]
  Cx* sbe = sal + (size_t)p.npcta * nt;
  Cx* sga = sbe + (size_t)p.npcta * nt;
  T* sHx = (T*)(sga + (size_t)p.npcta * nt);
  T* sHy = sHx + nx * nx;
  T* sox = sHy + ny * ny;
  T* soy = sox + N * nx;
  T* sW = soy + N * ny;
  T* sWr = sW + E;
  T* ssh = sWr + E;
  int* snb = (int*)(ssh + p.npcta);
  int* sst = snb + p.npcta * nt;

  const double* hx = p.Hx + smp * p.Hx_stride;
  const double* hy = p.Hy + smp * p.Hy_stride;
  for (int i = tid; i < nx * nx; i += bd) sHx[i] = (T)hx[i];
  for (int i = tid; i < ny * ny; i += bd) sHy[i] = (T)hy[i];
  for (int i = tid; i < N * nx; i += bd) sox[i] = (T)p.occx[i];
  for (int i = tid; i < N * ny; i += bd) soy[i] = (T)p.occy[i];
  for (int i = tid; i < E; i += bd) sW[i] = p.W ? (T)p.W[i] : (T)0;
  for (int i = tid; i < E; i += bd) sWr[i] = p.Wraw ? (T)p.Wraw[i] : (T)0;
  for (int i = tid; i < p.npcta; i += bd) ssh[i] = i < nloc ? (T)p.shift[node0 + i] : (T)0;
  for (int i = tid; i < p.npcta * nt; i += bd) {
    const bool ok = i < nloc * nt;
    const int g = node0 * nt + i;
    snb[i] = ok ? p.nbr[g] : -1;
    sst[i] = ok ? p.site[g] : 0;
    const double2 a = ok ? p.alpha[g] : make_double2(0.0, 0.0);
    const double2 b = ok ? p.beta[g] : make_double2(0.0, 0.0);
    const double2 c = (ok && p.gamma) ? p.gamma[g] : make_double2(0.0, 0.0);
    sal[i] = cmk((T)a.x, (T)a.y);
    sbe[i] = cmk((T)b.x, (T)b.y);
    sga[i] = cmk((T)c.x, (T)c.y);
  }
  __syncthreads();
  // this thread's elements: state (split-word in FP32) and RK4 accumulator
  Cx yh[EPT], yl[EPT], acc[EPT];
  const double2* y0 = p.y0 + smp * p.y0_stride;
#pragma unroll
  for (int u = 0; u < EPT; ++u) {
    const int el = tid + u * bd;
    yh[u] = yl[u] = acc[u] = cmk((T)0, (T)0);
    if (el < Mloc) {
      const double2 v = y0[(int64_t)node0 * E + el];
      yh[u] = cmk((T)v.x, (T)v.y);
      if (sizeof(T) == 4) yl[u] = cmk((T)(v.x - (double)yh[u].x), (T)(v.y - (double)yh[u].y));
      sx[el] = yh[u];   // stage 0 input of step 0, buffer 0
    }
  }
  const T h = (T)p.h, uc = (T)p.uc;
  auto save = [&](int k) {
#pragma unroll
    for (int u = 0; u < EPT; ++u) {
      const int el = tid + u * bd;
      const int node = node0 + el / E;
      if (el >= Mloc || node >= p.keep) continue;
      double vx = (double)yh[u].x, vy = (double)yh[u].y;
      if (sizeof(T) == 4) {
        vx += (double)yl[u].x;
        vy += (double)yl[u].y;
      }
      if (p.status && !(isfinite(vx) && isfinite(vy))) atomicOr(p.status, QSX_ERR_NONFINITE);
      p.saves[(smp * p.nsave + k) * (int64_t)p.keep * E + (int64_t)node * E + el % E] =
          make_double2(vx, vy);
    }
  };
  save(0);
  for (int step = 0; step < p.nsteps; ++step) {
    for (int stage = 0; stage < 4; ++stage) {
      const int buf = stage & 1;   // 4 stages per step: the parity pattern repeats
      cluster.sync();              // this stage's input is complete cluster-wide
      const Cx* xin = sx + (size_t)buf * p.npcta * E;
      Cx* xout = sx + (size_t)(buf ^ 1) * p.npcta * E;
      const T cnext = stage == 2 ? h : (T)0.5 * h;
      const T wg = (stage == 0 || stage == 3) ? (T)1 : (T)2;
      // commutator and diagonal terms of every element of this thread
      T orr[EPT], oi[EPT];
#pragma unroll
      for (int u = 0; u < EPT; ++u) {
        const int el = tid + u * bd;
        orr[u] = oi[u] = (T)0;
        if (el >= Mloc) continue;
        const int l = el / E, e = el % E;
        const int a = e % nx, bb = e / nx;
        const Cx* xs = xin + l * E;
        // -i (Hx x - x Hy)[a][bb]
        T cr = 0, ci = 0;
        for (int c = 0; c < nx; ++c) {
          const T hv = sHx[a * nx + c];
          const Cx v = xs[c + nx * bb];
          cr = fma(hv, v.x, cr);
          ci = fma(hv, v.y, ci);
        }
        for (int c = 0; c < ny; ++c) {
          const T hv = sHy[c * ny + bb];
          const Cx v = xs[a + nx * c];
          cr = fma(-hv, v.x, cr);
          ci = fma(-hv, v.y, ci);
        }
        const Cx self = xs[e];
        const T sh = ssh[l] + sW[e];
        orr[u] = fma(-sh, self.x, ci);
        oi[u] = fma(-sh, self.y, -cr);
      }
      // couplings, term by term across all of the thread's elements, so the
      // neighbour loads of different elements (local or through distributed
      // shared memory) are in flight together; the lanes serving one node
      // read its terms in the same order (one coalesced access per warp when
      // E is a multiple of 32)
      for (int t = 0; t < nt; ++t) {
        Cx v[EPT];
        int tt[EPT];
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
          const int el = tid + u * bd;
          tt[u] = -1;
          v[u] = cmk((T)0, (T)0);
          if (el >= Mloc) continue;
          const int l = el / E;
          const int m = snb[l * nt + t];
          if (m < 0) continue;
          tt[u] = l * nt + t;
          const int r = m / p.npcta, ml = m - r * p.npcta;
          const Cx* src = r == rank ? xin : cluster.map_shared_rank(xin, r);
          v[u] = src[ml * E + el % E];
        }
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
          if (tt[u] < 0) continue;
          const int e = (tid + u * bd) % E;
          const int a = e % nx, bb = e / nx;
          const int j = sst[tt[u]];
          const Cx al = sal[tt[u]], be = sbe[tt[u]], ga = sga[tt[u]];
          const T oa = sox[j * nx + a], ob = soy[j * ny + bb];
          const T gw = sWr[e] * (oa - ob);
          const T fr = al.x * oa + be.x * ob + ga.x * gw, fi = al.y * oa + be.y * ob + ga.y * gw;
          orr[u] = fma(fr, v[u].x, fma(-fi, v[u].y, orr[u]));
          oi[u] = fma(fr, v[u].y, fma(fi, v[u].x, oi[u]));
        }
      }
#pragma unroll
      for (int u = 0; u < EPT; ++u) {
        const int el = tid + u * bd;
        if (el >= Mloc) continue;
        const Cx d = cmk(uc * orr[u], uc * oi[u]);
        acc[u] = stage == 0 ? d : cmk(acc[u].x + wg * d.x, acc[u].y + wg * d.y);
        if (stage < 3) {
          xout[el] = cmk(yh[u].x + cnext * d.x, yh[u].y + cnext * d.y);
        } else {
          const T s6 = h / (T)6;
          if (sizeof(T) == 4) {
            float hxv = (float)yh[u].x, lxv = (float)yl[u].x, hyv = (float)yh[u].y,
                  lyv = (float)yl[u].y;
            dd_add(hxv, lxv, (float)(s6 * acc[u].x));
            dd_add(hyv, lyv, (float)(s6 * acc[u].y));
            yh[u] = cmk((T)hxv, (T)hyv);
            yl[u] = cmk((T)lxv, (T)lyv);
          } else {
            yh[u] = cmk(yh[u].x + s6 * acc[u].x, yh[u].y + s6 * acc[u].y);
          }
          xout[el] = yh[u];
        }
      }
    }
    if ((step + 1) % p.save_every == 0) save((step + 1) / p.save_every);
  }
  cluster.sync();  // peers may still read this CTA's buffers
}

// out = RHS(x) in FP64 (the equation of motion as a callable).
__global__ void __launch_bounds__(256)
    heom_rhs_kernel(HeomP p, const double2* __restrict__ x, double2* __restrict__ out, int npc) {
  extern __shared__ __align__(16) unsigned char smraw[];
  HeomSmem<double> sm = heom_carve<double>(smraw, p, npc);
  const int64_t b = blockIdx.y;
  const int n0 = blockIdx.x * npc;
  heom_stage_smem<double>(p, x, b, n0, npc, sm);
  const int local = threadIdx.x / p.E, e = threadIdx.x % p.E;
  const int node = n0 + local;
  if (local >= npc || node >= p.nnodes) return;
  double2 k;
  heom_rhs_elem<double>(p, x, b, local, e, sm, k);
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
  QSX_CHECK_ARG(a->variant >= 0 && a->variant <= 4, "qsx_heom: variant must be in 0..4");
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
  p.gamma = (const double2*)a->gamma;
  p.Wraw = a->Wraw;
  p.uc = a->unit_convert;
  p.h = a->h;
  return p;
}

template <typename T, int EPT>
static cudaError_t launch_heom_cluster(const HeomCP& p, size_t smem, cudaStream_t s,
                                       int* clusters, bool one_wave) {
  auto kern = heom_cluster_kernel<T, EPT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(p.batch * p.csize));
  cfg.blockDim = dim3(512);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)p.csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  *clusters = 0;
  e = cudaOccupancyMaxActiveClusters(clusters, kern, &cfg);
  if (e != cudaSuccess || *clusters < 1) return e;
  // the library's choice takes this form only when every sample's cluster is
  // resident at once: a second wave would rerun the whole time loop
  if (one_wave && p.batch > *clusters) {
    *clusters = 0;
    return cudaSuccess;
  }
  return cudaLaunchKernelEx(&cfg, kern, p);
}

// The persistent cluster form when the shapes allow it (and, for variant 0,
// when all samples fit in one wave): returns 1 if it ran (or failed with *st
// set), 0 to fall back to the per-stage kernels.
template <typename T>
static int heom_rk4_cluster(const qsx_heom_args* a, double2* saves, cudaStream_t s, int* st) {
  const int E = a->nx * a->ny;
  const int C = std::min(8, a->nnodes);
  const int npcta = (a->nnodes + C - 1) / C;
  const int ept = (npcta * E + 511) / 512;
  const size_t smem =
      heom_cluster_smem_bytes<T>(a->nx, a->ny, a->n_sites, E, npcta, std::max(a->nterms, 1));
  // register budget: at most 8 elements a thread in FP32 and 4 in FP64 (the
  // builds beyond spill; the spilled FP64 build at 8 elements a thread gave
  // results off by 1e-3 on the 495-node hierarchy, so those shapes take the
  // per-stage kernels)
  if (ept > (sizeof(T) == 4 ? 8 : 4) || smem > 200 * 1024) return 0;
  HeomCP p;
  p.nx = a->nx;
  p.ny = a->ny;
  p.E = E;
  p.nnodes = a->nnodes;
  p.nterms = std::max(a->nterms, 0);
  p.n_sites = a->n_sites;
  p.nsave = a->nsteps / a->save_every + 1;
  p.save_every = a->save_every;
  p.nsteps = a->nsteps;
  p.keep = a->save_nodes;
  p.csize = C;
  p.npcta = npcta;
  p.batch = a->batch;
  p.Hx_stride = a->H_stride ? (int64_t)a->nx * a->nx : 0;
  p.Hy_stride = a->H_stride ? (int64_t)a->ny * a->ny : 0;
  p.y0_stride = a->y0_stride ? (int64_t)a->nnodes * E : 0;
  p.Hx = a->Hx;
  p.Hy = a->Hy;
  p.occx = a->occx;
  p.occy = a->occy;
  p.W = a->W;
  p.shift = a->shift;
  p.nbr = a->nbr;
  p.site = a->site;
  p.alpha = (const double2*)a->alpha;
  p.beta = (const double2*)a->beta;
  p.gamma = (const double2*)a->gamma;
  p.Wraw = a->Wraw;
  p.uc = a->unit_convert;
  p.h = a->h;
  p.y0 = (const double2*)a->y0;
  p.saves = saves;
  p.status = a->status;
  int clusters = 0;
  cudaError_t e;
  if (ept <= 1)
    e = launch_heom_cluster<T, 1>(p, smem, s, &clusters, a->variant == 0);
  else if (ept <= 2)
    e = launch_heom_cluster<T, 2>(p, smem, s, &clusters, a->variant == 0);
  else if (ept <= 4)
    e = launch_heom_cluster<T, 4>(p, smem, s, &clusters, a->variant == 0);
  else if constexpr (sizeof(T) == 4)
    e = launch_heom_cluster<T, 8>(p, smem, s, &clusters, a->variant == 0);
  else
    return 0;
  if (e != cudaSuccess) {
    *st = cuda_status(e, "qsx_heom_rk4 (cluster form)");
    return 1;
  }
  if (clusters < 1) return 0;   // cannot be scheduled: per-stage kernels
  return 1;
}

static size_t heom_state_elems(const qsx_heom_args* a) {
  return (size_t)a->batch * a->nnodes * a->nx * a->ny;
}

__global__ void f64_to_f32_kernel(const double* __restrict__ src, float* __restrict__ dst,
                                  int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

// element counts of the FP32 table copies: Hx, Hy, occx, occy, W, shift and
// Wraw (slots 6..8 are empty: the term tables are packed separately)
static void heom_table_counts(const qsx_heom_args* a, int64_t c[10]) {
  const int64_t hb = a->H_stride ? a->batch : 1;
  c[0] = hb * a->nx * a->nx;
  c[1] = hb * a->ny * a->ny;
  c[2] = (int64_t)a->n_sites * a->nx;
  c[3] = (int64_t)a->n_sites * a->ny;
  c[4] = a->W ? (int64_t)a->nx * a->ny : 0;
  c[5] = a->nnodes;
  c[6] = c[7] = c[8] = 0;   // the term tables go into the packed records
  c[9] = a->Wraw ? (int64_t)a->nx * a->ny : 0;
}

static size_t heom_table_bytes(const qsx_heom_args* a) {
  int64_t c[10];
  heom_table_counts(a, c);
  size_t b = 0;
  for (int i = 0; i < 10; ++i) b += ((size_t)c[i] * sizeof(float) + 255) & ~(size_t)255;
  return b;
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
  const size_t tables = a->precision == QSX_FP32 ? heom_table_bytes(a) + 256 : 0;
  const size_t terms = (size_t)a->nnodes * a->nterms *
                       (a->precision == QSX_FP32 ? sizeof(HTerm<float>) : sizeof(HTerm<double>));
  // the terms again, grouped by site, and their counts (per-stage kernels
  // for blocks up to 8 x 8)
  const size_t site_terms = (size_t)a->nnodes * a->n_sites * std::max(a->nterms, 2) *
                            (a->precision == QSX_FP32 ? sizeof(HTerm<float>) : sizeof(HTerm<double>));
  *bytes = states + saves + 256 + tables + terms + 256 + site_terms + 256;
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
  const size_t smem = heom_smem_bytes<double>(p.nx, p.ny, p.n_sites, p.E, npc, p.nterms);
  QSX_CHECK_ARG(smem <= 227 * 1024, "qsx_heom_rhs: node tables too large for shared memory");
  cudaError_t ce = cudaFuncSetAttribute(heom_rhs_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (ce != cudaSuccess) return cuda_status(ce, "qsx_heom_rhs");
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
  const int64_t per = (int64_t)p.nnodes * p.E;
  double2* node0 = a->out_state ? (double2*)a->out_state : nullptr;
  const int keep = a->save_nodes;
  unsigned char* ws = (unsigned char*)a->workspace;
  auto run = [&](auto tag) -> int {
    using T = decltype(tag);
    using C = typename cplx<T>::type;
    if (a->variant == 0 || a->variant == 2) {
      // the whole loop in one launch, one cluster per sample
      double2* saves = (double2*)(((size_t)ws + 255) & ~(size_t)255);
      double2* dst = node0 ? node0 : saves;
      int cst = QSX_OK;
      if (heom_rk4_cluster<T>(a, dst, s, &cst)) {
        if (cst) return cst;
        if (a->out_mean) {
          const int64_t m = (int64_t)p.nsave * keep * p.E;
          heom_mean_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(
              dst, p.batch, m, 1.0 / (double)p.batch, (double2*)a->out_mean);
          QSX_LAUNCH_CHECK("qsx_heom_rk4 mean");
        }
        return QSX_OK;
      }
    }
    C* yh = (C*)ws;
    C* yl = sizeof(T) == 4 ? yh + n : nullptr;
    C* acc = (sizeof(T) == 4 ? yl : yh) + n;
    C* s0 = acc + n;
    C* s1 = s0 + n;
    double2* saves = (double2*)(((size_t)(s1 + n) + 255) & ~(size_t)255);
    if (!node0) node0 = saves;
    const int nsave_ = p.nsave;
    const size_t save_bytes =
        a->out_mean ? (size_t)p.batch * nsave_ * keep * p.E * sizeof(double2) : 0;
    unsigned char* tp = (unsigned char*)((((size_t)saves + save_bytes) + 255) & ~(size_t)255);
    HeomWP w;
    w.nx = p.nx;
    w.ny = p.ny;
    w.E = p.E;
    w.nnodes = p.nnodes;
    w.nterms = p.nterms;
    w.n_sites = p.n_sites;
    w.items = p.batch * p.nnodes;
    w.Hx_stride = p.Hx_stride;
    w.Hy_stride = p.Hy_stride;
    w.has_gamma = a->gamma != nullptr;
    w.uc = p.uc;
    w.h = p.h;
    if constexpr (sizeof(T) == 4) {
      // FP32 copies of the tables after the saves
      int64_t c[10];
      heom_table_counts(a, c);
      const double* src[10] = {a->Hx, a->Hy, a->occx, a->occy, a->W, a->shift, a->alpha,
                               a->beta, a->gamma, a->Wraw};
      float* dst[10];
      for (int i = 0; i < 10; ++i) {
        dst[i] = (float*)tp;
        tp += ((size_t)c[i] * sizeof(float) + 255) & ~(size_t)255;
        if (c[i] > 0 && src[i])
          f64_to_f32_kernel<<<(unsigned)((c[i] + 255) / 256), 256, 0, s>>>(src[i], dst[i], c[i]);
      }
      QSX_LAUNCH_CHECK("qsx_heom_rk4 tables");
      w.Hx = dst[0];
      w.Hy = dst[1];
      w.occx = dst[2];
      w.occy = dst[3];
      w.W = a->W ? dst[4] : nullptr;
      w.shift = dst[5];
      w.Wraw = a->Wraw ? dst[9] : nullptr;
    } else {
      w.Hx = a->Hx;
      w.Hy = a->Hy;
      w.occx = a->occx;
      w.occy = a->occy;
      w.W = a->W;
      w.shift = a->shift;
      w.Wraw = a->Wraw;
    }
    // packed term records
    HTerm<T>* terms = (HTerm<T>*)tp;
    const int64_t nrec = (int64_t)p.nnodes * p.nterms;
    if (nrec > 0) {
      heom_pack_terms_kernel<T><<<(unsigned)((nrec + 255) / 256), 256, 0, s>>>(
          a->nbr, a->site, (const double2*)a->alpha, (const double2*)a->beta,
          (const double2*)a->gamma, nrec, terms);
      QSX_LAUNCH_CHECK("qsx_heom_rk4 terms");
    }
    w.terms = terms;
    w.site_terms = nullptr;
    w.site_slots = std::max(p.nterms, 2);
    // blocks up to 8 x 8: the specialised kernel; wider ones: EPL elements a lane
    const int epl = p.E <= 32 ? 1 : (p.E <= 64 ? 2 : (p.E <= 128 ? 4 : 8));
    const bool small = p.nx <= 8 && p.ny <= 8;
    // blocks up to 8 x 8: the coupling terms grouped by site (variant 4: the
    // term loop over every term of the node instead)
    const bool by_site = small && a->variant != 4 && nrec > 0;
    if (by_site) {
      HTerm<T>* sterms = (HTerm<T>*)((((size_t)(terms + nrec)) + 255) & ~(size_t)255);
      const int64_t ns = (int64_t)p.nnodes * p.n_sites;
      heom_pack_site_terms_kernel<T><<<(unsigned)((ns + 255) / 256), 256, 0, s>>>(
          terms, p.nnodes, p.nterms, p.n_sites, w.site_slots, sterms);
      QSX_LAUNCH_CHECK("qsx_heom_rk4 site terms");
      w.site_terms = sterms;
    }
    auto kern = by_site    ? (p.nx == 8 && p.ny == 8 ? heom_warp_site_kernel<T, 8, (sizeof(T) == 4 ? 2 : 1)>
                                                     : heom_warp_site_kernel<T, 0, (sizeof(T) == 4 ? 2 : 1)>)
                : small    ? (p.nx == 8 && p.ny == 8 ? heom_warp_small_kernel<T, 8, 4, (sizeof(T) == 4 ? 2 : 1)>
                                                     : heom_warp_small_kernel<T, 0, 4, (sizeof(T) == 4 ? 2 : 1)>)
                : epl == 1 ? heom_warp_stage_kernel<T, 1>
                : epl == 2 ? heom_warp_stage_kernel<T, 2>
                : epl == 4 ? heom_warp_stage_kernel<T, 4>
                           : heom_warp_stage_kernel<T, 8>;
    const int wthreads = 256;
    const size_t wsmem =
        small ? (size_t)(wthreads / 32) * 64 * sizeof(C) * (by_site ? 2 : 1) +
                    (size_t)p.n_sites * (p.nx + p.ny) * sizeof(T) +
                    (by_site ? (size_t)(wthreads / 32) * 4 * p.n_sites * sizeof(HTerm<T>) : 0)
              : (size_t)(wthreads / 32) * 32 * epl * sizeof(C);
    if (wsmem > 48 * 1024) {
      cudaError_t fe = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)wsmem);
      if (fe != cudaSuccess) return cuda_status(fe, "qsx_heom_rk4");
    }
    // contiguous ranges of node blocks per warp, sized so one wave of
    // resident warps covers them
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (ce == cudaSuccess)
      ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, wthreads, wsmem);
    if (ce != cudaSuccess) return cuda_status(ce, "qsx_heom_rk4");
    const int64_t resident = std::max<int64_t>(1, (int64_t)sms * std::max(per_sm, 1) * (wthreads / 32));
    w.per_warp = (int)((w.items + resident - 1) / resident);
    const int64_t warps = (w.items + w.per_warp - 1) / w.per_warp;
    const unsigned wgrid = (unsigned)((warps + wthreads / 32 - 1) / (wthreads / 32));
    // variant 3: FP32 blocks up to 8 x 8 with the node commutators on the
    // tensor cores (heom_tc_stage_kernel); other shapes take the kernels above
    bool tc_stage = false;
    size_t tsmem = 0;
    unsigned tgrid = 0;
    if constexpr (sizeof(T) == 4) {
      if (a->variant == 3 && small) {
        tc_stage = true;
        tsmem = heom_tc_smem_bytes(p.E, p.n_sites, p.nx, p.ny);
        cudaError_t te = cudaFuncSetAttribute(heom_tc_stage_kernel,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)tsmem);
        if (te != cudaSuccess) return cuda_status(te, "qsx_heom_rk4");
        const int64_t tiles = p.batch * ((p.nnodes + HTC_NODES - 1) / HTC_NODES);
        tgrid = (unsigned)std::min<int64_t>(tiles, 2 * (int64_t)sms);
      }
    }
    heom_init_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        (const double2*)a->y0, a->y0_stride ? per : 0, per, p.batch, yh, yl);
    QSX_LAUNCH_CHECK("qsx_heom_rk4 init");
    const unsigned sg = (unsigned)((p.batch * keep * p.E + 255) / 256);
    heom_save_kernel<T><<<sg, 256, 0, s>>>(yh, yl, p.nnodes, p.E, keep, p.batch, 0, p.nsave,
                                          node0, a->status);
    for (int step = 1; step <= p.nsteps; ++step) {
      if constexpr (sizeof(T) == 4) {
        if (tc_stage) {
          heom_tc_stage_kernel<<<tgrid, 256, tsmem, s>>>(w, 0, yh, yh, yl, acc, s0, a->status);
          heom_tc_stage_kernel<<<tgrid, 256, tsmem, s>>>(w, 1, s0, yh, yl, acc, s1, a->status);
          heom_tc_stage_kernel<<<tgrid, 256, tsmem, s>>>(w, 2, s1, yh, yl, acc, s0, a->status);
          heom_tc_stage_kernel<<<tgrid, 256, tsmem, s>>>(w, 3, s0, yh, yl, acc, nullptr,
                                                         a->status);
          if (step % p.save_every == 0)
            heom_save_kernel<T><<<sg, 256, 0, s>>>(yh, yl, p.nnodes, p.E, keep, p.batch,
                                                  step / p.save_every, p.nsave, node0,
                                                  a->status);
          continue;
        }
      }
      kern<<<wgrid, wthreads, wsmem, s>>>(w, 0, yh, yh, yl, acc, s0);
      kern<<<wgrid, wthreads, wsmem, s>>>(w, 1, s0, yh, yl, acc, s1);
      kern<<<wgrid, wthreads, wsmem, s>>>(w, 2, s1, yh, yl, acc, s0);
      kern<<<wgrid, wthreads, wsmem, s>>>(w, 3, s0, yh, yl, acc, nullptr);
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

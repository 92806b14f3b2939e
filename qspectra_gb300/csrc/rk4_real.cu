// K-step blocked RK4 time loop in the real form of a Hermitian block.
//
// A Redfield generator maps Hermitian density matrices to Hermitian ones
// (H real symmetric), so on a diagonal Liouville block such as 'ee' the one-
// step propagator is a REAL matrix in the coordinates x[a + n b] = Re rho_ab
// (a <= b), Im rho_ba (a > b): every step costs m^2 real multiply-adds
// instead of m^2 complex ones (4 m^2).  The populations rho_aa are
// coordinates themselves.  This loop is the real counterpart of the complex
// blocked kernels in rk4.cu, fed by qsx_rk4_block_matrix_real_batched or
// qsx_rk4_block_matrix_real_tc: rows 0..m-1 of each sample's matrix advance
// K steps (P_r^K - I), the following nsel (K - 1) rows give the selected
// coordinates at the K - 1 intermediate steps.  The state is split-word
// FP32 throughout.  Three forms, chosen by the plan:
//   - two passes (the default when the selected rows and block-steps fit
//     128): rk4_hchain_f32 runs the state chain one warp per sample and
//     stores every block-start state; rk4_hcontract_tc then forms the
//     selected coordinates of all samples as one long-K tcgen05 GEMM summed
//     in tensor memory;
//   - rk4_hblock_ws_f32: one chain warp and trailing selected-row warps per
//     sample in one kernel;
//   - rk4_hblock_f32: one thread per row, G samples per CTA (any group size).
// Each form keeps per-CTA partial sums of the selected coordinates, every
// (step, coordinate) added by one owner in program order, and the CTA
// slices are summed in a fixed order, so results are reproducible.
#include <algorithm>

#include "qsx_common.cuh"
#include "qsx_tc.cuh"

namespace qsx {

struct HbP {
  int m, nsteps, nsave, nselect;
  int64_t batch;
  const float* matrix;     // [batch][RT][m]
  const double* y0;        // [batch][m] or shared [m] (y0_stride 0)
  int64_t y0_stride;
  const int* select;
  double* partial;         // [grid][nsave][nselect]
  int* status;
  int local_sums;          // 1: partial sums kept in shared memory until the end
};

// Paired FP32 multiply-add (sm_100+: two FMA per instruction, each rounded
// like fmaf): acc += a * b elementwise.
__device__ __forceinline__ void ffma2(float2& acc, float2 a, float2 b) {
  acc = __ffma2_rn(a, b, acc);
}

template <int M>
__global__ void __launch_bounds__(512, 1) rk4_hblock_f32(HbP p, int64_t ngroups, int G, int K) {
  constexpr int MP = (M + 3) & ~3;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int64_t sstride = ((int64_t)(M + p.nselect * (K - 1)) * M + 3) & ~(int64_t)3;
  float* mbuf = (float*)smraw;          // [G][sstride] next group's matrices (prefetched)
  float* xbuf = mbuf + G * sstride;     // [2][G][MP]
  float* stash = xbuf + 2 * G * MP;     // [2][K][G][nsel]
  // with p.local_sums the CTA's ensemble partial sums stay in shared memory
  // ([nsave][nsel] FP32) until the end instead of one FP64 atomic per step
  float* lsum = stash + 2 * K * G * p.nselect;
  const int nsel = p.nselect;
  if (!select_table_valid(p.select, nsel, M, p.status)) return;
  const int RT = M + nsel * (K - 1);
  const int tid = threadIdx.x;
  const int g = tid / RT, r = tid % RT;
  const bool active = tid < G * RT;
  const bool main_row = active && r < M;
  const int kx = main_row ? K : (r - M) / nsel + 1;
  const int qx = main_row ? -1 : (r - M) % nsel;
  int myq = -1;
  if (main_row)
    for (int q = 0; q < nsel; ++q)
      if (p.select[q] == r) { myq = q; break; }
  const int selr = (active && !main_row) ? p.select[qx] : 0;
  const int gs = active ? g : 0;
  // this thread's output slot (a selected coordinate at some step offset) in
  // both stash parities, and its partial-sum job: (k, q) = (tid / nsel,
  // tid % nsel) for tid < K nsel, fixed for the whole kernel
  const bool writes = main_row ? myq >= 0 : active;
  const int slot = writes ? ((main_row ? K - 1 : kx - 1) * G + g) * nsel + (main_row ? myq : qx) : 0;
  const int pstride = K * G * nsel;  // between the two stash parities
  const bool sums = tid < K * nsel;
  const int pk = sums ? tid / nsel : 0, pq = sums ? tid % nsel : 0;
  const int pslot = (pk * G) * nsel + pq;
  for (int e = tid; e < 2 * G * MP; e += blockDim.x) xbuf[e] = 0.f;
  if (p.local_sums)
    for (int e = tid; e < p.nsave * nsel; e += blockDim.x) lsum[e] = 0.f;
  __syncthreads();
  auto stash_at = [&](int par, int k, int gg, int q) -> float& {
    return stash[((par * K + k) * G + gg) * nsel + q];
  };
  // the group's matrices arrive in shared memory by 16-byte asynchronous
  // copies issued one group ahead (coalesced, overlapping the previous
  // group's time loop); each thread then moves its row into registers
  auto prefetch = [&](int64_t grp) {
    const int64_t s0 = grp * G;
    const int nvec = (int)(G * sstride / 4);
    const int64_t avail = (p.batch - s0) * sstride / 4;  // vectors of real samples
    const float* src = p.matrix + s0 * sstride;
    const unsigned dst = (unsigned)__cvta_generic_to_shared(mbuf);
    for (int i = tid; i < nvec && i < avail; i += blockDim.x)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16u * i),
                   "l"(src + 4 * (int64_t)i));
    asm volatile("cp.async.commit_group;");
  };
  if (blockIdx.x < ngroups) prefetch(blockIdx.x);
  int parity = 0;
  for (int64_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int64_t s = grp * G + gs;
    const bool valid = active && s < p.batch;
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    float2 drow[MP / 2];  // the row as pairs (j, j + 1), zero past M
    const float* dm = mbuf + gs * sstride + r * M;
#pragma unroll
    for (int j = 0; j < MP; j += 2)
      drow[j / 2] = make_float2((valid && j < M) ? dm[j] : 0.f,
                                (valid && j + 1 < M) ? dm[j + 1] : 0.f);
    __syncthreads();  // every row is in registers: the buffer is free
    if (grp + gridDim.x < ngroups) prefetch(grp + gridDim.x);
    float xh = 0.f, xl = 0.f;
    if (valid && main_row) {
      const double v = p.y0[s * p.y0_stride + r];
      xh = (float)v;
      xl = (float)(v - (double)xh);
    }
    if (main_row) xbuf[g * MP + r] = xh;
    if (myq >= 0) stash_at(parity, 0, g, myq) = xh;
    __syncthreads();
    for (int q = tid; q < nsel; q += blockDim.x) {
      float acc = 0.f;
      for (int gg = 0; gg < G; ++gg) acc += stash_at(parity, 0, gg, q);
      if (p.local_sums)
        lsum[q] += acc;
      else
        atomicAdd(p.partial + (int64_t)blockIdx.x * p.nsave * nsel + q, (double)acc);
    }
    parity ^= 1;
    const int nblk = p.nsteps / K;
    const float* cur0 = xbuf + gs * MP;
    const int xflip = G * MP;                      // offset of the other state buffer
    float* lrow = lsum + (pk + 1) * nsel + pq;     // advanced by K nsel per block-step
    double* grow = p.partial + ((int64_t)blockIdx.x * p.nsave + pk + 1) * nsel + pq;
    for (int bs = 0; bs < nblk; ++bs) {
      const int odd = bs & 1;
      const float* cur = cur0 + odd * xflip;
      // four paired accumulators: a quarter of the row each, two FMA per
      // instruction
      float2 a0 = make_float2(0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
#pragma unroll
      for (int j = 0; j < MP; j += 4) {
        const float4 v = *reinterpret_cast<const float4*>(cur + j);
        if ((j / 4) % 2 == 0) {
          ffma2(a0, drow[j / 2], make_float2(v.x, v.y));
          ffma2(a1, drow[j / 2 + 1], make_float2(v.z, v.w));
        } else {
          ffma2(a2, drow[j / 2], make_float2(v.x, v.y));
          ffma2(a3, drow[j / 2 + 1], make_float2(v.z, v.w));
        }
      }
      const float sum = ((a0.x + a0.y) + (a1.x + a1.y)) + ((a2.x + a2.y) + (a3.x + a3.y));
      float out = 0.f;
      if (main_row) {
        dd_add(xh, xl, sum);
        xbuf[(1 - odd) * xflip + g * MP + r] = xh;
        out = xh;
      } else if (active) {
        out = cur[selr] + sum;
      }
      if (writes) stash[parity * pstride + slot] = valid ? out : 0.f;
      __syncthreads();
      if (sums) {
        const float* src = stash + parity * pstride + pslot;
        float acc = 0.f;
        for (int gg = 0; gg < G; ++gg) acc += src[gg * nsel];
        if (p.local_sums)
          *lrow += acc;
        else
          atomicAdd(grow, (double)acc);
      }
      lrow += K * nsel;
      grow += K * nsel;
      parity ^= 1;
    }
    if (valid && main_row && p.status && !isfinite(xh)) atomicOr(p.status, QSX_ERR_NONFINITE);
    __syncthreads();
  }
  if (p.local_sums) {
    // every (step, coordinate) was last updated by one thread before the
    // final barrier of the loop; write this CTA's slice
    double* dst = p.partial + (int64_t)blockIdx.x * p.nsave * nsel;
    for (int e = tid; e < p.nsave * nsel; e += blockDim.x) dst[e] = (double)lsum[e];
  }
}

// Warp-specialised form of the same loop (the default).  Warp 0 holds the M
// state rows (P^K - I), two per lane (rows l and l + 32), and runs the
// sequential chain alone: each block-step is one pass over the state (each
// 16-byte load feeds both rows' paired FMA), the split-word update of the
// lane's own coordinates and a __syncwarp, with no CTA barrier.  The
// block-start states go into a ring of 2 CH + 1 slots in shared memory.  The
// following warps hold the nsel (K - 1) selected rows, 64 per warp, and trail
// the chain by one chunk of CH block-steps: for each block-start state of the
// previous chunk they form their selected coordinates at the K - 1
// intermediate steps, again with no barrier inside the chunk.  Every (step,
// coordinate) of the CTA's partial sums has one owning thread, which adds to
// it in shared memory directly; the two sides meet at one CTA barrier per
// chunk.  Each thread loads its rows from global memory into registers at the
// start of a sample; the next sample's matrices are prefetched into L2.
template <int M>
__device__ __forceinline__ void dot2_rows(const float* __restrict__ cur,
                                          const float2 (&ra)[((M + 3) & ~3) / 2],
                                          const float2 (&rb)[((M + 3) & ~3) / 2], float& sa,
                                          float& sb) {
  constexpr int MP = (M + 3) & ~3;
  float2 a0 = make_float2(0.f, 0.f), a1 = a0, a2 = a0, a3 = a0;
  float2 b0 = a0, b1 = a0, b2 = a0, b3 = a0;
#pragma unroll
  for (int j = 0; j < MP; j += 4) {
    const float4 v = *reinterpret_cast<const float4*>(cur + j);
    const float2 lo = make_float2(v.x, v.y), hi = make_float2(v.z, v.w);
    if ((j / 4) % 2 == 0) {
      ffma2(a0, ra[j / 2], lo);
      ffma2(a1, ra[j / 2 + 1], hi);
      ffma2(b0, rb[j / 2], lo);
      ffma2(b1, rb[j / 2 + 1], hi);
    } else {
      ffma2(a2, ra[j / 2], lo);
      ffma2(a3, ra[j / 2 + 1], hi);
      ffma2(b2, rb[j / 2], lo);
      ffma2(b3, rb[j / 2 + 1], hi);
    }
  }
  sa = ((a0.x + a0.y) + (a1.x + a1.y)) + ((a2.x + a2.y) + (a3.x + a3.y));
  sb = ((b0.x + b0.y) + (b1.x + b1.y)) + ((b2.x + b2.y) + (b3.x + b3.y));
}

template <int M>
__device__ __forceinline__ void load_row(const float* __restrict__ src, bool act,
                                         float2 (&d)[((M + 3) & ~3) / 2]) {
  constexpr int MP = (M + 3) & ~3;
#pragma unroll
  for (int j = 0; j < MP; j += 2)
    d[j / 2] = make_float2((act && j < M) ? __ldg(src + j) : 0.f,
                           (act && j + 1 < M) ? __ldg(src + j + 1) : 0.f);
}

template <int M, int MAXT>
__global__ void __launch_bounds__(MAXT, MAXT == 64 ? 6 : 1)
    rk4_hblock_ws_f32(HbP p, int K, int chunk) {
  constexpr int MP = (M + 3) & ~3;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int nsel = p.nselect;
  if (!select_table_valid(p.select, nsel, M, p.status)) return;
  const int nR = nsel * (K - 1);
  const int RT = M + nR;
  const int64_t sstride = ((int64_t)RT * M + 3) & ~(int64_t)3;
  const int nslot = 2 * chunk + 1;
  float* __restrict__ ring = reinterpret_cast<float*>(smraw);   // [nslot][MP] block-start states
  float* __restrict__ lsum = ring + nslot * MP;                 // [nsave][nsel] partial sums
  const int tid = threadIdx.x, lane = tid & 31;
  const bool mainw = tid < 32;
  // this lane's two rows: state rows lane, lane + 32; or selected rows i, i + 32
  const int ia = mainw ? lane : 64 * ((tid >> 5) - 1) + lane, ib = ia + 32;
  const bool acta = mainw ? ia < M : ia < nR, actb = mainw ? ib < M : ib < nR;
  const int rowa = mainw ? ia : M + ia, rowb = mainw ? ib : M + ib;
  int qa = -1, qb = -1, sela = 0, selb = 0;
  if (mainw) {
    for (int q = 0; q < nsel; ++q) {
      if (acta && p.select[q] == ia) qa = q;
      if (actb && p.select[q] == ib) qb = q;
    }
  } else {
    if (acta) sela = p.select[ia % nsel];
    if (actb) selb = p.select[ib % nsel];
    sela = (sela >= 0 && sela < M) ? sela : 0;
    selb = (selb >= 0 && selb < M) ? selb : 0;
  }
  // threads 32 .. 32 + nsel - 1 also own the selected coordinates at the
  // block boundaries (steps (b + 1) K)
  const int bq = (tid >= 32 && tid - 32 < nsel) ? tid - 32 : -1;
  int bsel = bq >= 0 ? p.select[bq] : 0;
  bsel = (bsel >= 0 && bsel < M) ? bsel : 0;
  for (int e = tid; e < nslot * MP; e += blockDim.x) ring[e] = 0.f;
  for (int e = tid; e < p.nsave * nsel; e += blockDim.x) lsum[e] = 0.f;
  __syncthreads();
  const int nblk = p.nsteps / K;
  const int nch = (nblk + chunk - 1) / chunk;
  // output slots: state rows at steps (b + 1) K, selected rows at b K + k;
  // both advance by K nsel per block-step
  float* const owna = lsum + (mainw ? max(qa, 0) : (ia / nsel + 1) * nsel + ia % nsel);
  float* const ownb = lsum + (mainw ? max(qb, 0) : (ib / nsel + 1) * nsel + ib % nsel);
  const bool wa = mainw ? qa >= 0 : acta, wb = mainw ? qb >= 0 : actb;
  for (int64_t s = blockIdx.x; s < p.batch; s += gridDim.x) {
    if (tid == 0 && s + gridDim.x < p.batch) {
      const float* nxt = p.matrix + (s + gridDim.x) * sstride;
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(nxt),
                   "r"((unsigned)(sstride * 4))
                   : "memory");
    }
    float2 da[MP / 2], db[MP / 2];
    {
      const float* src = p.matrix + s * sstride;
      load_row<M>(src + (int64_t)rowa * M, acta, da);
      load_row<M>(src + (int64_t)rowb * M, actb, db);
    }
    float xha = 0.f, xla = 0.f, xhb = 0.f, xlb = 0.f;
    if (mainw) {
      const double* y0 = p.y0 + s * p.y0_stride;
      if (acta) {
        const double v = y0[ia];
        xha = (float)v;
        xla = (float)(v - (double)xha);
        ring[ia] = xha;
        if (wa) owna[0] += xha;
      }
      if (actb) {
        const double v = y0[ib];
        xhb = (float)v;
        xlb = (float)(v - (double)xhb);
        ring[ib] = xhb;
        if (wb) ownb[0] += xhb;
      }
    }
    __syncthreads();
    for (int c = 0; c <= nch; ++c) {
      if (mainw) {
        if (c < nch) {
          const int b0 = c * chunk, b1 = min(b0 + chunk, nblk);
          int slot = b0 % nslot;
          for (int b = b0; b < b1; ++b) {
            float sa, sb;
            dot2_rows<M>(ring + slot * MP, da, db, sa, sb);
            slot = slot + 1 == nslot ? 0 : slot + 1;
            float* nxt = ring + slot * MP;
            if (acta) {
              dd_add(xha, xla, sa);
              nxt[ia] = xha;
            }
            if (actb) {
              dd_add(xhb, xlb, sb);
              nxt[ib] = xhb;
            }
            __syncwarp();
          }
        }
      } else if (c >= 1) {
        const int b0 = (c - 1) * chunk, b1 = min(b0 + chunk, nblk);
        int slot = b0 % nslot;
        int64_t off = (int64_t)b0 * K * nsel;
        for (int b = b0; b < b1; ++b) {
          const float* cur = ring + slot * MP;
          float sa, sb;
          dot2_rows<M>(cur, da, db, sa, sb);
          if (wa) owna[off] += cur[sela] + sa;
          if (wb) ownb[off] += cur[selb] + sb;
          off += K * nsel;
          slot = slot + 1 == nslot ? 0 : slot + 1;
          // the selected coordinates of the next block-start state (step
          // (b + 1) K), written by the chain in this chunk
          if (bq >= 0) lsum[(int64_t)(b + 1) * K * nsel + bq] += ring[slot * MP + bsel];
        }
      }
      __syncthreads();
    }
    if (mainw && p.status && ((acta && !isfinite(xha)) || (actb && !isfinite(xhb))))
      atomicOr(p.status, QSX_ERR_NONFINITE);
  }
  // every (step, coordinate) was last updated by its owner before the final
  // barrier; write this CTA's slice
  double* dst = p.partial + (int64_t)blockIdx.x * p.nsave * nsel;
  for (int e = tid; e < p.nsave * nsel; e += blockDim.x) dst[e] = (double)lsum[e];
}

// out[e] = scale * sum over slots of partial[slot][e].  One CTA per 32
// consecutive e: warp w adds slots w, w + 8, ... (each load a coalesced
// 256-byte row), then warp 0 adds the eight warp sums in warp order, so the
// summation order is fixed and results are reproducible.
__global__ void __launch_bounds__(256) hblock_reduce_kernel(const double* __restrict__ partial,
                                                            int64_t nslots, int64_t per,
                                                            double scale,
                                                            double* __restrict__ out) {
  __shared__ double red[8][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t e = (int64_t)blockIdx.x * 32 + lane;
  double acc = 0.0;
  if (e < per)
    for (int64_t sl = warp; sl < nslots; sl += 8) acc += partial[sl * per + e];
  red[warp][lane] = acc;
  __syncthreads();
  if (warp == 0 && e < per) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += red[w][lane];
    out[e] = t * scale;
  }
}

// Two-pass form of the loop.
//
// Pass 1 (rk4_hchain_f32): the state chain alone, one warp per sample and
// two state rows per lane (rows l, l + 32) in registers, so each SM holds
// about twelve independent chains.  Each block-step forms x_{b+1} =
// x_b + (P^K - I) x_b in split-word FP32 and stores the leading word of
// x_{b+1} both to a two-slot ring in shared memory (the next step's input)
// and to Y[s][b + 1] in global memory; no CTA barrier, one __syncwarp.
//
// Pass 2 (rk4_hcontract_tc, below): the selected coordinates at the
// intermediate steps, out[b K + k][q] = x_b[sel_q] + (row R_k,q) . x_b,
// summed over the samples, on the tensor cores.
template <int M>
__global__ void __launch_bounds__(32, 12)
    rk4_hchain_f32(const float* __restrict__ matrix, int64_t sstride, const double* __restrict__ y0,
                   int64_t y0_stride, int64_t batch, int nblk, float* __restrict__ Y,
                   int* status) {
  constexpr int MP = (M + 3) & ~3;
  __shared__ __align__(16) float ring[2][MP];
  const int lane = threadIdx.x;
  const int ia = lane, ib = lane + 32;
  const bool acta = ia < M, actb = ib < M;
  for (int e = lane; e < 2 * MP; e += 32) (&ring[0][0])[e] = 0.f;
  __syncwarp();
  const int64_t ystride = (int64_t)(nblk + 1) * MP;
  for (int64_t s = blockIdx.x; s < batch; s += gridDim.x) {
    if (lane == 0 && s + gridDim.x < batch) {
      const float* nxt = matrix + (s + gridDim.x) * sstride;
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(nxt),
                   "r"((unsigned)((int64_t)M * M * 4 + 15) & ~15u)
                   : "memory");
    }
    float2 da[MP / 2], db[MP / 2];
    const float* src = matrix + s * sstride;
    load_row<M>(src + (int64_t)ia * M, acta, da);
    load_row<M>(src + (int64_t)ib * M, actb, db);
    float* ys = Y + s * ystride;
    float xha = 0.f, xla = 0.f, xhb = 0.f, xlb = 0.f;
    if (acta) {
      const double v = y0[s * y0_stride + ia];
      xha = (float)v;
      xla = (float)(v - (double)xha);
      ring[0][ia] = xha;
    }
    if (ia < MP) ys[ia] = xha;
    if (actb) {
      const double v = y0[s * y0_stride + ib];
      xhb = (float)v;
      xlb = (float)(v - (double)xhb);
      ring[0][ib] = xhb;
    }
    if (ib < MP) ys[ib] = xhb;   // the padding columns of the stored states are zero
    __syncwarp();
    int cur = 0;
    for (int b = 0; b < nblk; ++b) {
      float sa, sb;
      dot2_rows<M>(ring[cur], da, db, sa, sb);
      cur ^= 1;
      float* yn = ys + (int64_t)(b + 1) * MP;
      if (acta) {
        dd_add(xha, xla, sa);
        ring[cur][ia] = xha;
      }
      if (ia < MP) yn[ia] = xha;
      if (actb) {
        dd_add(xhb, xlb, sb);
        ring[cur][ib] = xhb;
      }
      if (ib < MP) yn[ib] = xhb;
      __syncwarp();
    }
    if (status && ((acta && !isfinite(xha)) || (actb && !isfinite(xhb))))
      atomicOr(status, QSX_ERR_NONFINITE);
  }
}

constexpr int HC_THREADS = 128, HC_FLUSH = 4;

// Shapes and shared memory of pass 2: A = the nR selected rows (M = 128
// accumulator rows, K = KP), B = the nblk block-start states (N = nblk
// rounded up to 16, at most 128); hi/lo planes of both, the boundary sums
// [nblk + 1][nsel], the mbarrier and the tensor-memory address.
struct HcShape {
  int kp, nb, tmem_cols, arows;
  size_t smem;
};

// A planes hold `arows` rows: 64 when nR <= 64, since the MMA's rows 64..127
// may then read whatever follows (their accumulator rows are never used),
// else 128.  The staging scratch holds either the raw selected rows or the
// raw states of one sample.
inline size_t hcontract_scratch_floats(int m, int nR, int nblk) {
  const size_t mp = (size_t)((m + 3) & ~3);
  return std::max((size_t)nR * m, (size_t)(nblk + 1) * mp);
}

inline bool hcontract_shape(int m, int nR, int nblk, int nsel, HcShape* sh) {
  if (nR > tc::ROWS || nblk < 1 || nblk > 128) return false;
  sh->kp = (m + 7) & ~7;
  sh->nb = (nblk + 15) & ~15;
  sh->arows = nR <= 64 ? 64 : tc::ROWS;
  // two tiles: the MMA tile and the running sum
  sh->tmem_cols = 32;
  while (sh->tmem_cols < 2 * sh->nb) sh->tmem_cols *= 2;
  const size_t planes = 2 * (size_t)sh->arows * sh->kp * 4 + 2 * (size_t)sh->nb * sh->kp * 4;
  sh->smem = ((planes + hcontract_scratch_floats(m, nR, nblk) * 4 + (size_t)(nblk + 1) * nsel * 4 +
               15) & ~(size_t)15) + 16;
  // the A operand of each MMA spans 128 rows from its plane's start: with
  // 64-row planes the lo plane's rows 64..127 end at 3 x 64 rows, which
  // must lie inside the allocation
  sh->smem = std::max(sh->smem, (size_t)3 * 64 * sh->kp * 4);
  return sh->smem <= 227 * 1024;
}

// Pass 2 on the tensor cores.  Summed over the samples, the intermediate
// coordinates are out[b K + k][q] = sum_s (R_s)_{k,q} . x^s_b + sum_s
// x^s_b[sel_q]: the first term is the product of the stacked selected rows
// [R_1 | R_2 | ...] with the stacked states [X_1; X_2; ...], i.e. one long-K
// GEMM, which the tcgen05 accumulator forms by adding every sample's
// 3xTF32 chain into the same TMEM tile.  Per sample the CTA loads the rows
// and states into registers (ahead of the previous chain's completion),
// splits them into TF32 hi/lo planes and issues one chain of 3 KP / 8 MMAs;
// the second term (the block-boundary coordinates, also the outputs at steps
// b K) is summed by the thread that stages state b.  Two CTAs share an SM so
// that one stages while the other's chain runs; at the end the CTA writes
// its slice from TMEM.  Every barrier wait is bounded.
template <int M>
__global__ void __launch_bounds__(HC_THREADS, 2)
    rk4_hcontract_tc(const float* __restrict__ matrix, int64_t sstride, const float* __restrict__ Y,
                     int64_t batch, int nblk, int K, const int* __restrict__ select, int nsel,
                     int nb, int tmem_cols, int arows, double* __restrict__ partial, int nsave,
                     int* status) {
  using namespace tc;
  constexpr int MP = (M + 3) & ~3;
  constexpr int KP = (M + 7) & ~7;
  extern __shared__ __align__(128) unsigned char smraw[];
  const uint32_t sbo = KP * 32u;
  const uint32_t PA = (uint32_t)arows * KP * 4, PB = (uint32_t)nb * KP * 4;
  unsigned char* a_hi = smraw;
  unsigned char* a_lo = a_hi + PA;
  unsigned char* b_hi = a_lo + PA;
  unsigned char* b_lo = b_hi + PB;
  const int nR_ = nsel * (K - 1);
  const int nsc = max(nR_ * M, (nblk + 1) * MP);
  float* sc = reinterpret_cast<float*>(b_lo + PB);      // staging scratch [nsc]
  float* bsum = sc + nsc;                               // [nblk + 1][nsel]
  const uint32_t off_mbar =
      (2 * PA + 2 * PB + (uint32_t)(nsc + (nblk + 1) * nsel) * 4 + 15) & ~15u;
  uint64_t* mbar_p = reinterpret_cast<uint64_t*>(smraw + off_mbar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar_p + 1);
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int nR = nsel * (K - 1);
  const uint32_t mbar = (uint32_t)__cvta_generic_to_shared(mbar_p);
  const uint64_t da_hi = smem_desc((uint32_t)__cvta_generic_to_shared(a_hi), sbo);
  const uint64_t da_lo = smem_desc((uint32_t)__cvta_generic_to_shared(a_lo), sbo);
  const uint64_t db_hi = smem_desc((uint32_t)__cvta_generic_to_shared(b_hi), sbo);
  const uint64_t db_lo = smem_desc((uint32_t)__cvta_generic_to_shared(b_lo), sbo);
  const uint32_t idesc = make_idesc(nb);
  if (!select_table_valid(select, nsel, M, status)) return;   // before any TMEM is held
  for (uint32_t e = tid; e < (2 * PA + 2 * PB) / 16; e += HC_THREADS)
    reinterpret_cast<uint4*>(smraw)[e] = make_uint4(0, 0, 0, 0);
  for (int e = tid; e < (nblk + 1) * nsel; e += HC_THREADS) bsum[e] = 0.f;
  if (tid == 0) {
    s_abort = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(tmem_slot)),
                 "r"(tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // this thread's selected row (A row = TMEM lane = tid) and states b = tid,
  // tid + 128 (B rows; the boundary sums also take b = nblk)
  const bool arow = tid < nR;
  const int64_t ystride = (int64_t)(nblk + 1) * MP;
  uint32_t parity = 0;
  bool first = true;
  int nacc = 0;   // samples summed in tensor memory since the last flush
  const bool brow = tid < nblk;   // this thread stages state b = tid
  double* dst = partial + (int64_t)blockIdx.x * nsave * nsel;
  const int k = arow ? tid / nsel + 1 : 0, q = arow ? tid % nsel : 0;
  // Every HC_FLUSH samples the MMA tile (columns 0 .. nb) is added, in
  // IEEE FP32, into a second tile (columns tmem_cols / 2 ..) that holds the
  // running sum, so that at most HC_FLUSH x 3 KP / 8 MMAs add into the MMA
  // tile before it restarts (the tensor-core accumulation is not rounded to
  // nearest at every add).
  const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16);
  const uint32_t long_addr = lane_addr + (uint32_t)(tmem_cols / 2);
  bool have_long = false;
  auto flush = [&]() {
    for (int c0 = 0; c0 < nb; c0 += 16) {
      float v[16];
      tmem_load(lane_addr + (uint32_t)c0, v);
      if (have_long) {
        float w[16];
        tmem_load(long_addr + (uint32_t)c0, w);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] += w[j];
      }
      tmem_store(long_addr + (uint32_t)c0, v);
    }
    have_long = true;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  };
  // per-sample loads, coalesced: the selected rows (nR x M floats, from a
  // 4-byte-aligned start) and the states ((nblk + 1) x MP floats, 16-byte
  // aligned), each thread taking every HC_THREADS-th element / vector
  constexpr int RA = (128 * 64 + HC_THREADS - 1) / HC_THREADS;          // bound for nR M
  constexpr int RY = ((129 * MP) / 4 + HC_THREADS - 1) / HC_THREADS;    // bound for (nblk + 1) MP / 4
  const int na = nR * M, ny4 = (nblk + 1) * MP / 4;
  for (int64_t s = blockIdx.x; s < batch; s += gridDim.x) {
    if (tid == 0 && s + gridDim.x < batch) {
      // the next sample's selected rows and states into L2
      const int64_t n = s + gridDim.x;
      const uintptr_t r0 = reinterpret_cast<uintptr_t>(matrix + n * sstride + (int64_t)M * M) & ~(uintptr_t)15;
      const uintptr_t r1 = (reinterpret_cast<uintptr_t>(matrix + n * sstride + (int64_t)(M + nR) * M) + 15) &
                           ~(uintptr_t)15;
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(r0), "r"((unsigned)(r1 - r0))
                   : "memory");
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(Y + n * ystride),
                   "r"((unsigned)(ystride * 4))
                   : "memory");
    }
    // this sample's data into registers while the previous chain runs
    const float* rsrc = matrix + s * sstride + (int64_t)M * M;
    const float4* ysrc = reinterpret_cast<const float4*>(Y + s * ystride);
    float ra[RA];
    float4 ry[RY];
#pragma unroll
    for (int j = 0; j < RA; ++j) {
      const int e = tid + HC_THREADS * j;
      ra[j] = e < na ? __ldg(rsrc + e) : 0.f;
    }
#pragma unroll
    for (int j = 0; j < RY; ++j) {
      const int e = tid + HC_THREADS * j;
      ry[j] = e < ny4 ? __ldg(ysrc + e) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (!first) {
      if (tid == 0 && !wait_parity(mbar, parity)) {
        if (status) atomicOr(status, QSX_ERR_CUDA);
        s_abort = 1;
      }
      __syncthreads();
      if (s_abort) break;
      parity ^= 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (nacc == HC_FLUSH) {
        flush();
        nacc = 0;
      }
    }
    // selected rows: scratch (row-major, stride M), then each row's owner
    // splits it into the A planes
#pragma unroll
    for (int j = 0; j < RA; ++j) {
      const int e = tid + HC_THREADS * j;
      if (e < na) sc[e] = ra[j];
    }
    __syncthreads();
    if (arow) {
      float a[KP];
#pragma unroll
      for (int c = 0; c < KP; ++c) a[c] = c < M ? sc[tid * M + c] : 0.f;
#pragma unroll
      for (int g = 0; g < KP / 4; ++g)
        st_split4(a_hi, a_lo, op_offset(tid, 4 * g, sbo), a[4 * g], a[4 * g + 1], a[4 * g + 2],
                  a[4 * g + 3]);
    }
    __syncthreads();
    // states: scratch ([nblk + 1][MP]), then state b = tid into the B planes
    // and the boundary coordinates of states b = tid, tid + 128, ...
#pragma unroll
    for (int j = 0; j < RY; ++j) {
      const int e = tid + HC_THREADS * j;
      if (e < ny4) reinterpret_cast<float4*>(sc)[e] = ry[j];
    }
    __syncthreads();
    if (brow) {
      float x[KP];
#pragma unroll
      for (int c4 = 0; c4 < KP; c4 += 4) {
        const float4 v = c4 < MP ? *reinterpret_cast<const float4*>(sc + tid * MP + c4)
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
        x[c4] = v.x;
        x[c4 + 1] = v.y;
        x[c4 + 2] = v.z;
        x[c4 + 3] = v.w;
      }
#pragma unroll
      for (int g = 0; g < KP / 4; ++g)
        st_split4(b_hi, b_lo, op_offset(tid, 4 * g, sbo), x[4 * g], x[4 * g + 1], x[4 * g + 2],
                  x[4 * g + 3]);
    }
    for (int b = tid; b <= nblk; b += HC_THREADS)
      for (int q = 0; q < nsel; ++q) {
        int c = __ldg(select + q);
        c = (c >= 0 && c < M) ? c : 0;
        bsum[b * nsel + q] += sc[b * MP + c];
      }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0)
      issue_product(tmem, da_hi, da_lo, db_hi, db_lo, KP / 8, idesc, mbar, nacc > 0 ? 1u : 0u);
    first = false;
    ++nacc;
  }
  if (!first && !s_abort) {
    if (tid == 0 && !wait_parity(mbar, parity)) {
      if (status) atomicOr(status, QSX_ERR_CUDA);
      s_abort = 1;
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!s_abort) {
    if (nacc > 0) flush();
    for (int c0 = 0; c0 < nb; c0 += 16) {
      float v[16];
      if (have_long) {
        tmem_load(long_addr + (uint32_t)c0, v);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0.f;
      }
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int b = c0 + j;
        if (arow && b < nblk)
          dst[((int64_t)b * K + k) * nsel + q] = (double)v[j] + (double)bsum[b * nsel + q];
      }
    }
    for (int e = tid; e < (nblk + 1) * nsel; e += HC_THREADS) {
      const int bb = e / nsel;
      dst[(int64_t)bb * K * nsel + (e - bb * nsel)] = (double)bsum[e];
    }
  } else if (tid == 0) {
    wait_parity(mbar, parity);   // let an unfinished chain drain before freeing TMEM
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(tmem_cols)
                 : "memory");
}

#define QSX_HBLOCK_SIZES(X) X(9) X(16) X(25) X(36) X(49) X(64)

struct HbPlan {
  int G, threads, local_sums;
  int ws, chunk;   // warp-specialised kernel and its chunk of block-steps
  int tp;          // two-pass form: chain, then contraction
  int nb, tmem_cols, arows;   // two-pass: padded states, tensor-memory columns, A plane rows
  int64_t ngroups, grid, chain_grid;
  size_t smem;
  size_t ybytes;   // two-pass: the block-start states, after the partial slices
};

// launch configuration of the two-pass form, if it applies
static cudaError_t hblock_tp_plan(int m, int64_t batch, int K, int nsteps, int nselect, int group,
                                  HbPlan* pl, bool* ok) {
  *ok = false;
  const int nR = nselect * (K - 1);
  const int nblk = nsteps / K;
  HcShape sh;
  if (group > 1 || K < 2 || !hcontract_shape(m, nR, nblk, nselect, &sh)) return cudaSuccess;
  int dev = 0, sms = 0, occ_c = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
#define X(MM)                                                                                 \
  if (e == cudaSuccess && m == MM) {                                                          \
    e = cudaFuncSetAttribute(rk4_hcontract_tc<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             (int)sh.smem);                                                   \
    if (e == cudaSuccess)                                                                     \
      e = cudaFuncSetAttribute(rk4_hcontract_tc<MM>,                                          \
                               cudaFuncAttributePreferredSharedMemoryCarveout,                \
                               (int)cudaSharedmemCarveoutMaxShared);                          \
    if (e == cudaSuccess)                                                                     \
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_c, rk4_hchain_f32<MM>, 32, 0);   \
  }
  QSX_HBLOCK_SIZES(X)
#undef X
  if (e != cudaSuccess) return e;
  pl->tp = 1;
  pl->ws = 0;
  pl->G = 1;
  pl->smem = sh.smem;
  pl->local_sums = 1;
  pl->ngroups = batch;
  pl->nb = sh.nb;
  pl->tmem_cols = sh.tmem_cols;
  pl->arows = sh.arows;
  // two contraction CTAs per SM (one stages while the other's chain runs);
  // the occupancy query can report fewer for tcgen05 kernels, and a second
  // wave is harmless because every CTA strides over the samples on its own
  pl->grid = std::max<int64_t>(1, std::min<int64_t>(batch, 2 * (int64_t)sms));
  pl->chain_grid = std::max<int64_t>(1, std::min<int64_t>(batch, (int64_t)sms * std::max(occ_c, 1)));
  pl->ybytes = (size_t)batch * (nblk + 1) * ((m + 3) & ~3) * sizeof(float);
  *ok = true;
  return cudaSuccess;
}

// launch configuration of the warp-specialised kernel, if it applies:
// one sample per CTA, partial sums in shared memory, at most 448 selected rows
static bool hblock_ws_plan(int m, int K, int nsteps, int nselect, int group, HbPlan* pl) {
  const int nR = nselect * (K - 1);
  if (group > 1 || nR > 448 || nselect > 224) return false;
  const int MP = (m + 3) & ~3;
  const size_t lsum = (size_t)(nsteps + 1) * nselect * sizeof(float);
  for (int chunk = 16; chunk >= 2; chunk /= 2) {
    const size_t smem = (size_t)(2 * chunk + 1) * MP * sizeof(float) + lsum;
    if (smem <= 96 * 1024) {
      pl->ws = 1;
      pl->chunk = chunk;
      pl->G = 1;
      // warp 0 runs the chain; the others hold 64 selected rows each and
      // own the nsel block-boundary outputs (at least one such warp)
      pl->threads = 32 + 32 * std::max(std::max((nR + 63) / 64, (nselect + 31) / 32), 1);
      pl->smem = smem;
      pl->local_sums = 1;
      return true;
    }
  }
  return false;
}

template <int M>
static cudaError_t hblock_ws_occupancy(const HbPlan& pl, int* occ) {
  cudaError_t e;
  if (pl.threads <= 64) {
    e = cudaFuncSetAttribute(rk4_hblock_ws_f32<M, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)pl.smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(rk4_hblock_ws_f32<M, 64>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, rk4_hblock_ws_f32<M, 64>,
                                                        pl.threads, pl.smem);
  } else {
    e = cudaFuncSetAttribute(rk4_hblock_ws_f32<M, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)pl.smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, rk4_hblock_ws_f32<M, 256>,
                                                        pl.threads, pl.smem);
  }
  return e;
}

template <int M>
static void hblock_ws_launch(const HbPlan& pl, const HbP& p, int K, cudaStream_t s) {
  if (pl.threads <= 64)
    rk4_hblock_ws_f32<M, 64><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(p, K, pl.chunk);
  else
    rk4_hblock_ws_f32<M, 256><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(p, K, pl.chunk);
}


static int hblock_plan(int m, int64_t batch, int K, int nsteps, int nselect, int group,
                       HbPlan* pl) {
  const int RT = m + nselect * (K - 1);
  QSX_CHECK_ARG(RT <= 512, "qsx_rk4_real_block_mean: %d blocked rows per sample exceed 512", RT);
  QSX_CHECK_ARG(group >= 0 && group * RT <= 512,
                "qsx_rk4_real_block_mean: %d samples of %d rows exceed 512 threads", group, RT);
  pl->ws = 0;
  pl->chunk = 0;
  pl->tp = 0;
  pl->chain_grid = 0;
  pl->ybytes = 0;
  {
    bool ok = false;
    cudaError_t e = hblock_tp_plan(m, batch, K, nsteps, nselect, group, pl, &ok);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_real_block_mean plan");
    if (ok) return QSX_OK;
  }
  if (hblock_ws_plan(m, K, nsteps, nselect, group, pl)) {
    pl->ngroups = batch;
    int dev = 0, sms = 0, occ = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
#define X(MM) \
    if (e == cudaSuccess && m == MM) e = hblock_ws_occupancy<MM>(*pl, &occ);
    QSX_HBLOCK_SIZES(X)
#undef X
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_real_block_mean plan");
    pl->grid = std::max<int64_t>(1, std::min<int64_t>(batch, (int64_t)sms * std::max(occ, 1)));
    return QSX_OK;
  }
  // one sample per CTA by default: each CTA is an independent pipeline with
  // its own barrier, several resident per SM
  pl->G = group ? group : 1;
  pl->threads = ((pl->G * RT + 31) / 32) * 32;
  const int MP = (m + 3) & ~3;
  const size_t sstride = ((size_t)RT * m + 3) & ~(size_t)3;
  pl->smem = ((size_t)pl->G * sstride + 2 * (size_t)pl->G * MP +
              2 * (size_t)K * pl->G * nselect) * sizeof(float);
  // keep the CTA's partial sums in shared memory when they fit beside it
  const size_t lsum = (size_t)(nsteps + 1) * nselect * sizeof(float);
  pl->local_sums = pl->smem + lsum <= 64 * 1024;
  if (pl->local_sums) pl->smem += lsum;
  pl->ngroups = (batch + pl->G - 1) / pl->G;
  int dev = 0, sms = 0, occ = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
#define X(MM)                                                                         \
  if (e == cudaSuccess && m == MM) {                                                  \
    e = cudaFuncSetAttribute(rk4_hblock_f32<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             (int)pl->smem);                                          \
    if (e == cudaSuccess)                                                             \
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rk4_hblock_f32<MM>,     \
                                                        pl->threads, pl->smem);       \
  }
  QSX_HBLOCK_SIZES(X)
#undef X
  if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_real_block_mean plan");
  pl->grid = std::max<int64_t>(1, std::min<int64_t>(pl->ngroups, (int64_t)sms * std::max(occ, 1)));
  return QSX_OK;
}

static int hblock_check(int m, int64_t batch, int K, int nsteps, int nselect) {
  QSX_CHECK_ARG(m == 9 || m == 16 || m == 25 || m == 36 || m == 49 || m == 64,
                "qsx_rk4_real_block_mean: m must be n^2 for n in 3..8 (got %d)", m);
  QSX_CHECK_ARG(batch >= 0 && batch <= 0x7fffffffLL && K >= 1 && K <= 64 && nsteps >= 0 &&
                    nsteps % K == 0 && nselect >= 1 && nselect <= m,
                "qsx_rk4_real_block_mean: bad sizes (K=%d, nsteps=%d, nselect=%d)", K, nsteps,
                nselect);
  return QSX_OK;
}

}  // namespace qsx

using namespace qsx;

// the CTA partial slices, rounded up to 256 bytes (the two-pass states follow)
static size_t hblock_partial_bytes(const HbPlan& pl, int nsteps, int nselect) {
  return ((size_t)pl.grid * (nsteps + 1) * nselect * sizeof(double) + 255) & ~(size_t)255;
}

extern "C" size_t qsx_rk4_real_block_workspace_bytes(int m, int64_t batch, int K, int nsteps,
                                                     int nselect, int group) {
  if (hblock_check(m, batch, K, nsteps, nselect) != QSX_OK || batch == 0) return 0;
  HbPlan pl;
  if (hblock_plan(m, batch, K, nsteps, nselect, group, &pl) != QSX_OK) return 0;
  return hblock_partial_bytes(pl, nsteps, nselect) + pl.ybytes;
}

extern "C" int qsx_rk4_real_block_mean(const float* matrix, int m, int64_t batch, int K,
                                       int nsteps, const double* y0, int64_t y0_stride,
                                       const int* select, int nselect, int group,
                                       double* out_mean, void* workspace,
                                       size_t workspace_bytes, int32_t* status, void* stream) {
  int st = hblock_check(m, batch, K, nsteps, nselect);
  if (st) return st;
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(matrix && y0 && select && out_mean && workspace,
                "qsx_rk4_real_block_mean: null pointer");
  HbPlan pl;
  st = hblock_plan(m, batch, K, nsteps, nselect, group, &pl);
  if (st) return st;
  const int64_t per = (int64_t)(nsteps + 1) * nselect;
  const size_t need = hblock_partial_bytes(pl, nsteps, nselect) + pl.ybytes;
  QSX_CHECK_ARG(workspace_bytes >= need,
                "qsx_rk4_real_block_mean: workspace of %zu bytes needed (got %zu)", need,
                workspace_bytes);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  HbP p;
  p.m = m;
  p.nsteps = nsteps;
  p.nsave = nsteps + 1;
  p.nselect = nselect;
  p.batch = batch;
  p.matrix = matrix;
  p.y0 = y0;
  p.y0_stride = y0_stride;
  p.select = select;
  p.partial = (double*)workspace;
  p.status = status;
  p.local_sums = pl.local_sums;
  if (pl.tp) {
    const int nblk = nsteps / K;
    const int MP = (m + 3) & ~3;
    const int64_t sstride = ((int64_t)(m + nselect * (K - 1)) * m + 3) & ~(int64_t)3;
    float* Y = reinterpret_cast<float*>(static_cast<char*>(workspace) +
                                        hblock_partial_bytes(pl, nsteps, nselect));
    (void)MP;
#define X(MM)                                                                                  \
    if (m == MM) {                                                                             \
      rk4_hchain_f32<MM><<<(unsigned)pl.chain_grid, 32, 0, s>>>(matrix, sstride, y0, y0_stride, \
                                                                batch, nblk, Y, status);       \
      rk4_hcontract_tc<MM><<<(unsigned)pl.grid, HC_THREADS, pl.smem, s>>>(                     \
          matrix, sstride, Y, batch, nblk, K, select, nselect, pl.nb, pl.tmem_cols, pl.arows,   \
          (double*)workspace, nsteps + 1, status);                                              \
    }
    QSX_HBLOCK_SIZES(X)
#undef X
    QSX_LAUNCH_CHECK("qsx_rk4_real_block_mean");
    hblock_reduce_kernel<<<(unsigned)((per + 31) / 32), 256, 0, s>>>(
        (const double*)workspace, pl.grid, per, 1.0 / (double)batch, out_mean);
    QSX_LAUNCH_CHECK("qsx_rk4_real_block_mean reduce");
    return QSX_OK;
  }
  if (pl.ws) {
#define X(MM) \
    if (m == MM) hblock_ws_launch<MM>(pl, p, K, s);
    QSX_HBLOCK_SIZES(X)
#undef X
    QSX_LAUNCH_CHECK("qsx_rk4_real_block_mean");
    hblock_reduce_kernel<<<(unsigned)((per + 31) / 32), 256, 0, s>>>(
        (const double*)workspace, pl.grid, per, 1.0 / (double)batch, out_mean);
    QSX_LAUNCH_CHECK("qsx_rk4_real_block_mean reduce");
    return QSX_OK;
  }
  if (!pl.local_sums) {  // the FP64 atomics accumulate into zeroed slices
    e = cudaMemsetAsync(workspace, 0, need, s);
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_real_block_mean memset");
  }
#define X(MM)                                                                          \
  if (m == MM) {                                                                       \
    e = cudaFuncSetAttribute(rk4_hblock_f32<MM>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             (int)pl.smem);                                            \
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_real_block_mean");            \
  }
  QSX_HBLOCK_SIZES(X)
#undef X
#define X(MM)                                                                               \
  if (m == MM) rk4_hblock_f32<MM><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(p, pl.ngroups, \
                                                                                pl.G, K);
  QSX_HBLOCK_SIZES(X)
#undef X
  QSX_LAUNCH_CHECK("qsx_rk4_real_block_mean");
  hblock_reduce_kernel<<<(unsigned)((per + 31) / 32), 256, 0, s>>>(
      (const double*)workspace, pl.grid, per, 1.0 / (double)batch, out_mean);
  QSX_LAUNCH_CHECK("qsx_rk4_real_block_mean reduce");
  return QSX_OK;
}

// K-step blocked RK4 time loop in the real form of a Hermitian block.
//
// A Redfield generator maps Hermitian density matrices to Hermitian ones
// (H real symmetric), so on a diagonal Liouville block such as 'ee' the one-
// step propagator is a REAL matrix in the coordinates x[a + n b] = Re rho_ab
// (a <= b), Im rho_ba (a > b): every step costs m^2 real multiply-adds
// instead of m^2 complex ones (4 m^2).  The populations rho_aa are
// coordinates themselves.  This loop is the real counterpart of the complex
// blocked kernels in rk4.cu, fed by qsx_rk4_block_matrix_real_batched:
// rows 0..m-1 of each sample's matrix advance K steps (P_r^K - I), the
// following nsel (K - 1) rows give the selected coordinates at the K - 1
// intermediate steps.  One thread per matrix row (the row in registers),
// G samples per CTA, a persistent grid; the state is split-word FP32.  The
// ensemble mean of the selected coordinates is accumulated per CTA, each
// (step, coordinate) always by the same thread in program order: in FP32 in
// shared memory when [nsteps + 1][nsel] fits there (written out once at the
// end), else by FP64 atomics into the CTA's global slice.  The CTA slices
// are summed in a fixed order, so results are reproducible.
#include <algorithm>

#include "qsx_common.cuh"

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
  extern __shared__ __align__(16) unsigned char smraw[];
  const int64_t sstride = ((int64_t)(M + p.nselect * (K - 1)) * M + 3) & ~(int64_t)3;
  float* mbuf = (float*)smraw;          // [G][sstride] next group's matrices (prefetched)
  float* xbuf = mbuf + G * sstride;     // [2][G][MP]
  float* stash = xbuf + 2 * G * MP;     // [2][K][G][nsel]
  // with p.local_sums the CTA's ensemble partial sums stay in shared memory
  // ([nsave][nsel] FP32) until the end instead of one FP64 atomic per step
  float* lsum = stash + 2 * K * G * p.nselect;
  const int nsel = p.nselect;
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

// out[e] = scale * sum over slots of partial[slot][e], slots in order.
__global__ void hblock_reduce_kernel(const double* __restrict__ partial, int64_t nslots,
                                     int64_t per, double scale, double* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= per) return;
  double acc = 0.0;
  for (int64_t sl = 0; sl < nslots; ++sl) acc += partial[sl * per + e];
  out[e] = acc * scale;
}

struct HbPlan {
  int G, threads, local_sums;
  int64_t ngroups, grid;
  size_t smem;
};

#define QSX_HBLOCK_SIZES(X) X(9) X(16) X(25) X(36) X(49) X(64)

static int hblock_plan(int m, int64_t batch, int K, int nsteps, int nselect, int group,
                       HbPlan* pl) {
  const int RT = m + nselect * (K - 1);
  QSX_CHECK_ARG(RT <= 512, "qsx_rk4_real_block_mean: %d blocked rows per sample exceed 512", RT);
  QSX_CHECK_ARG(group >= 0 && group * RT <= 512,
                "qsx_rk4_real_block_mean: %d samples of %d rows exceed 512 threads", group, RT);
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

extern "C" size_t qsx_rk4_real_block_workspace_bytes(int m, int64_t batch, int K, int nsteps,
                                                     int nselect, int group) {
  if (hblock_check(m, batch, K, nsteps, nselect) != QSX_OK || batch == 0) return 0;
  HbPlan pl;
  if (hblock_plan(m, batch, K, nsteps, nselect, group, &pl) != QSX_OK) return 0;
  return (size_t)pl.grid * (nsteps + 1) * nselect * sizeof(double);
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
  const size_t need = (size_t)pl.grid * per * sizeof(double);
  QSX_CHECK_ARG(workspace_bytes >= need,
                "qsx_rk4_real_block_mean: workspace of %zu bytes needed (got %zu)", need,
                workspace_bytes);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
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
#define X(MM)                                                                               \
  if (m == MM) rk4_hblock_f32<MM><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(p, pl.ngroups, \
                                                                                pl.G, K);
  QSX_HBLOCK_SIZES(X)
#undef X
  QSX_LAUNCH_CHECK("qsx_rk4_real_block_mean");
  hblock_reduce_kernel<<<(unsigned)((per + 255) / 256), 256, 0, s>>>(
      (const double*)workspace, pl.grid, per, 1.0 / (double)batch, out_mean);
  QSX_LAUNCH_CHECK("qsx_rk4_real_block_mean reduce");
  return QSX_OK;
}

// K-step blocked RK4 loop for projected signals of small blocks (M <= 8),
// the time loop behind the Heisenberg-picture linear response
// (qspectra/simulate/response.py:15-43: signal(t) = proj . y(t), y the bra
// state evolved with the transposed 'eg' generator).
//
// Per sample the host-side build gives the (M + P K) x M complex matrix
//   rows 0..M-1          D_K = P^K - I            (advances K steps)
//   row  M + k P + p     W_{k,p} = proj_p P^k     (k = 0..K-1)
// so one pass over the rows at step n yields the signals at steps
// n .. n + K - 1 and the state at n + K: per K steps (M + P K) M complex
// multiply-adds instead of K (M^2 + P M).  One thread per row and a
// split-word FP32 state: one sample per warp when the M + P K rows fit 32
// (rk4_projblock_w_f32), else G samples per CTA (rk4_projblock_f32).  The
// ensemble mean is accumulated in shared memory, each (step, projection) by
// one thread in program order, and the CTA slices are summed in a fixed
// order.
#include <algorithm>

#include "qsx_common.cuh"

namespace qsx {

// ---------------------------------------------------------------- build
// Per sample: P = I + D (complex64, M x M) in shared memory, the projection
// rows W_k = W_{k-1} P and D_K by binary powering with
// (I + X)(I + Y) - I = X + Y + X Y.  One warp per sample (eight samples per
// CTA): each warp works in its own shared-memory slices and synchronises
// with __syncwarp, so the ~K + 2 log2 K dependent small products need no CTA
// barrier.
constexpr int PBW_WARPS = 8;

__global__ void __launch_bounds__(32 * PBW_WARPS)
    proj_block_build_w_kernel(const float2* __restrict__ D, int M, int K,
                              const double2* __restrict__ proj, int P, int64_t batch,
                              float2* __restrict__ out) {
  __shared__ float2 sm[PBW_WARPS][6][8 * 8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t b = (int64_t)blockIdx.x * PBW_WARPS + w;
  if (b >= batch) return;   // whole warps only: no CTA barrier follows
  float2* sP = sm[w][0];
  float2* sX = sm[w][1];
  float2* sY = sm[w][2];
  float2* sZ = sm[w][3];
  float2* sW[2] = {sm[w][4], sm[w][5]};
  const int mm = M * M, rows = M + P * K;
  const float2* d = D + b * mm;
  float2* o = out + b * (int64_t)rows * M;
  for (int e = lane; e < mm; e += 32) {
    sX[e] = d[e];
    sP[e] = cmk(d[e].x + ((e / M) == (e % M) ? 1.f : 0.f), d[e].y);
  }
  for (int e = lane; e < P * M; e += 32) {
    const double2 v = proj[e];
    sW[0][e] = cmk((float)v.x, (float)v.y);
    o[(int64_t)M * M + e] = sW[0][e];  // k = 0
  }
  __syncwarp();
  for (int k = 1; k < K; ++k) {
    const float2* wprev = sW[(k - 1) & 1];
    float2* wnext = sW[k & 1];
    for (int e = lane; e < P * M; e += 32) {
      const int p = e / M, c = e % M;
      float2 acc = cmk(0.f, 0.f);
      for (int j = 0; j < M; ++j) cfma(acc, wprev[p * M + j], sP[j * M + c]);
      wnext[e] = acc;
      o[(int64_t)(M + k * P) * M + e] = acc;
    }
    __syncwarp();
  }
  // D_K: base = D_{2^j} in sX, result accumulated in sY
  bool have = false;
  for (int kk = K; kk > 0; kk >>= 1) {
    if (kk & 1) {
      if (!have) {
        for (int e = lane; e < mm; e += 32) sY[e] = sX[e];
        have = true;
      } else {
        for (int e = lane; e < mm; e += 32) {
          const int r = e / M, c = e % M;
          float2 acc = cadd2(sY[e], sX[e]);
          for (int j = 0; j < M; ++j) cfma(acc, sY[r * M + j], sX[j * M + c]);
          sZ[e] = acc;
        }
        __syncwarp();
        for (int e = lane; e < mm; e += 32) sY[e] = sZ[e];
      }
      __syncwarp();
    }
    if (kk > 1) {
      for (int e = lane; e < mm; e += 32) {
        const int r = e / M, c = e % M;
        float2 acc = cadd2(sX[e], sX[e]);
        for (int j = 0; j < M; ++j) cfma(acc, sX[r * M + j], sX[j * M + c]);
        sZ[e] = acc;
      }
      __syncwarp();
      for (int e = lane; e < mm; e += 32) sX[e] = sZ[e];
      __syncwarp();
    }
  }
  for (int e = lane; e < mm; e += 32) o[e] = sY[e];
}

// ----------------------------------------------------------------- loop
struct PbP {
  int nsteps, nsave, P;
  int64_t batch;
  const float2* matrix;     // [batch][M + P K][M]
  const double2* y0;        // [batch][M] or shared
  int64_t y0_stride;
  double2* partial;         // [grid][nsave][P]
  int* status;
};

template <int M>
__global__ void __launch_bounds__(256) rk4_projblock_f32(PbP p, int64_t ngroups, int G, int K) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int P = p.P, RT = M + P * K;
  float2* ybuf = (float2*)smraw;             // [2][G][M]
  float2* stash = ybuf + 2 * G * M;          // [2][K][G][P]
  float2* lsum = stash + 2 * K * G * P;      // [nsave][P]
  const int tid = threadIdx.x;
  const int g = tid / RT, r = tid % RT;
  const bool active = tid < G * RT;
  const bool main_row = active && r < M;
  const int kx = main_row ? 0 : (r - M) / P, px = main_row ? 0 : (r - M) % P;
  const int gs = active ? g : 0;
  const bool sums = tid < K * P;
  const int pk = sums ? tid / P : 0, pp = sums ? tid % P : 0;
  for (int e = tid; e < 2 * G * M; e += blockDim.x) ybuf[e] = cmk(0.f, 0.f);
  for (int e = tid; e < p.nsave * P; e += blockDim.x) lsum[e] = cmk(0.f, 0.f);
  __syncthreads();
  int parity = 0;
  for (int64_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int64_t s = grp * G + gs;
    const bool valid = active && s < p.batch;
    float2 row[M];
    const float2* dm = p.matrix + (valid ? (s * RT + r) * (int64_t)M : 0);
#pragma unroll
    for (int j = 0; j < M; ++j) row[j] = valid ? dm[j] : cmk(0.f, 0.f);
    float yhx = 0.f, yhy = 0.f, ylx = 0.f, yly = 0.f;
    if (valid && main_row) {
      const double2 v = p.y0[s * p.y0_stride + r];
      yhx = (float)v.x;
      yhy = (float)v.y;
      ylx = (float)(v.x - (double)yhx);
      yly = (float)(v.y - (double)yhy);
    }
    if (main_row) ybuf[g * M + r] = cmk(yhx, yhy);
    __syncthreads();
    const int nblk = p.nsteps / K;
    for (int bs = 0; bs <= nblk; ++bs) {
      const float2* cur = ybuf + ((bs & 1) * G + gs) * M;
      const bool last = bs == nblk;  // only the step-nsteps signal remains
      float2 a0 = cmk(0.f, 0.f), a1 = a0;
#pragma unroll
      for (int j = 0; j < M; j += 2) {
        cfma(a0, row[j], cur[j]);
        if (j + 1 < M) cfma(a1, row[j + 1], cur[j + 1]);
      }
      const float sx = a0.x + a1.x, sy = a0.y + a1.y;
      if (main_row) {
        if (!last) {
          dd_add(yhx, ylx, sx);
          dd_add(yhy, yly, sy);
          ybuf[(((bs + 1) & 1) * G + g) * M + r] = cmk(yhx, yhy);
        }
      } else if (active && (!last || kx == 0)) {
        stash[((parity * K + kx) * G + g) * P + px] = valid ? cmk(sx, sy) : cmk(0.f, 0.f);
      }
      __syncthreads();
      if (sums && (!last || pk == 0)) {
        float2 acc = cmk(0.f, 0.f);
        for (int gg = 0; gg < G; ++gg) acc = cadd2(acc, stash[((parity * K + pk) * G + gg) * P + pp]);
        float2* l = lsum + (bs * K + pk) * P + pp;
        *l = cadd2(*l, acc);
      }
      parity ^= 1;
    }
    if (valid && main_row && p.status && !(isfinite(yhx) && isfinite(yhy)))
      atomicOr(p.status, QSX_ERR_NONFINITE);
    __syncthreads();
  }
  double2* dst = p.partial + (int64_t)blockIdx.x * p.nsave * P;
  for (int e = tid; e < p.nsave * P; e += blockDim.x)
    dst[e] = make_double2((double)lsum[e].x, (double)lsum[e].y);
}

// Warp-per-sample form (the default when the M + P K rows fit one warp):
// lane l holds row l, the state goes through a two-slot ring in shared
// memory with a __syncwarp per block-step and no CTA barrier, and each warp
// keeps its own partial sums [nsave][P] in shared memory, every (step,
// projection) owned by one lane.  At the end the warps' sums are added in
// warp order into the CTA's slice, so results are reproducible.
constexpr int PW_WARPS = 4;

template <int M>
__global__ void __launch_bounds__(32 * PW_WARPS) rk4_projblock_w_f32(PbP p, int K) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int P = p.P, RT = M + P * K;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float2* ybuf = reinterpret_cast<float2*>(smraw) + w * 16;          // [2][8] per warp
  float2* lsum = reinterpret_cast<float2*>(smraw) + PW_WARPS * 16 +  // [nsave][P] per warp
                 (size_t)w * p.nsave * P;
  const bool main_row = lane < M, act = lane < RT;
  const int kx = main_row ? 0 : (lane - M) / P, px = main_row ? 0 : (lane - M) % P;
  for (int e = lane; e < p.nsave * P; e += 32) lsum[e] = cmk(0.f, 0.f);
  if (lane < 16) ybuf[lane] = cmk(0.f, 0.f);
  __syncwarp();
  const int nblk = p.nsteps / K;
  for (int64_t s = (int64_t)blockIdx.x * PW_WARPS + w; s < p.batch;
       s += (int64_t)gridDim.x * PW_WARPS) {
    float2 row[M];
    const float2* dm = p.matrix + (s * RT + (act ? lane : 0)) * (int64_t)M;
#pragma unroll
    for (int j = 0; j < M; ++j) row[j] = act ? dm[j] : cmk(0.f, 0.f);
    float yhx = 0.f, yhy = 0.f, ylx = 0.f, yly = 0.f;
    if (main_row) {
      const double2 v = p.y0[s * p.y0_stride + lane];
      yhx = (float)v.x;
      yhy = (float)v.y;
      ylx = (float)(v.x - (double)yhx);
      yly = (float)(v.y - (double)yhy);
      ybuf[lane] = cmk(yhx, yhy);
    }
    __syncwarp();
    for (int bs = 0; bs <= nblk; ++bs) {
      const float2* cur = ybuf + (bs & 1) * 8;
      const bool last = bs == nblk;  // only the step-nsteps signal remains
      float2 a0 = cmk(0.f, 0.f), a1 = a0;
#pragma unroll
      for (int j = 0; j < M; j += 2) {
        cfma(a0, row[j], cur[j]);
        if (j + 1 < M) cfma(a1, row[j + 1], cur[j + 1]);
      }
      const float sx = a0.x + a1.x, sy = a0.y + a1.y;
      if (main_row) {
        if (!last) {
          dd_add(yhx, ylx, sx);
          dd_add(yhy, yly, sy);
          ybuf[((bs + 1) & 1) * 8 + lane] = cmk(yhx, yhy);
        }
      } else if (act && (!last || kx == 0)) {
        float2* l = lsum + ((int64_t)bs * K + kx) * P + px;
        *l = cadd2(*l, cmk(sx, sy));
      }
      __syncwarp();
    }
    if (main_row && p.status && !(isfinite(yhx) && isfinite(yhy)))
      atomicOr(p.status, QSX_ERR_NONFINITE);
  }
  __syncthreads();
  const float2* all = reinterpret_cast<const float2*>(smraw) + PW_WARPS * 16;
  double2* dst = p.partial + (int64_t)blockIdx.x * p.nsave * P;
  for (int e = threadIdx.x; e < p.nsave * P; e += blockDim.x) {
    double x = 0.0, y = 0.0;
#pragma unroll
    for (int ww = 0; ww < PW_WARPS; ++ww) {
      const float2 v = all[(size_t)ww * p.nsave * P + e];
      x += (double)v.x;
      y += (double)v.y;
    }
    dst[e] = make_double2(x, y);
  }
}

// One CTA per 32 consecutive e: warp w adds slots w, w + 8, ... (each load a
// coalesced row), then warp 0 adds the eight warp sums in warp order, so the
// summation order is fixed and results are reproducible.
__global__ void __launch_bounds__(256) projblock_reduce_kernel(const double2* __restrict__ partial,
                                                               int64_t nslots, int64_t per,
                                                               double scale,
                                                               double2* __restrict__ out) {
  __shared__ double2 red[8][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t e = (int64_t)blockIdx.x * 32 + lane;
  double2 acc = make_double2(0.0, 0.0);
  if (e < per)
    for (int64_t sl = warp; sl < nslots; sl += 8) acc = cadd(acc, partial[sl * per + e]);
  red[warp][lane] = acc;
  __syncthreads();
  if (warp == 0 && e < per) {
    double2 t = make_double2(0.0, 0.0);
#pragma unroll
    for (int w = 0; w < 8; ++w) t = cadd(t, red[w][lane]);
    out[e] = cscale(t, scale);
  }
}

struct PbPlan {
  int G, threads, warp_form;
  int64_t ngroups, grid;
  size_t smem;
};

static int projblock_plan(int m, int64_t batch, int K, int nsteps, int P, PbPlan* pl) {
  const int RT = m + P * K;
  QSX_CHECK_ARG(RT <= 256, "qsx_rk4_proj_block_mean: %d rows per sample exceed 256", RT);
  pl->warp_form = 0;
  {
    const size_t smem = ((size_t)PW_WARPS * 16 + (size_t)PW_WARPS * (nsteps + 1) * P) *
                        sizeof(float2);
    if (RT <= 32 && smem <= 110 * 1024) {
      int dev = 0, sms = 0, occ = 0;
      cudaError_t e = cudaGetDevice(&dev);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      switch (m) {
#define C(MM)                                                                               \
  case MM:                                                                                  \
    if (e == cudaSuccess)                                                                   \
      e = cudaFuncSetAttribute(rk4_projblock_w_f32<MM>,                                     \
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);     \
    if (e == cudaSuccess)                                                                   \
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rk4_projblock_w_f32<MM>,      \
                                                        32 * PW_WARPS, smem);               \
    break;
        C(1) C(2) C(3) C(4) C(5) C(6) C(7) C(8)
#undef C
      }
      if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_proj_block_mean plan");
      pl->warp_form = 1;
      pl->G = PW_WARPS;
      pl->threads = 32 * PW_WARPS;
      pl->smem = smem;
      pl->ngroups = (batch + PW_WARPS - 1) / PW_WARPS;
      pl->grid = std::max<int64_t>(1, std::min<int64_t>(pl->ngroups, (int64_t)sms * std::max(occ, 1)));
      return QSX_OK;
    }
  }
  pl->G = std::max(1, 256 / RT);
  pl->threads = ((pl->G * RT + 31) / 32) * 32;
  pl->smem = ((size_t)2 * pl->G * m + 2 * (size_t)K * pl->G * P + (size_t)(nsteps + 1) * P) *
             sizeof(float2);
  QSX_CHECK_ARG(pl->smem <= 160 * 1024, "qsx_rk4_proj_block_mean: %zu bytes of shared memory",
                pl->smem);
  pl->ngroups = (batch + pl->G - 1) / pl->G;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_proj_block_mean plan");
  // two CTAs per SM keep the per-CTA partial slices (nsave x P) few
  pl->grid = std::max<int64_t>(1, std::min<int64_t>(pl->ngroups, 2 * (int64_t)sms));
  return QSX_OK;
}

}  // namespace qsx

using namespace qsx;

extern "C" int qsx_rk4_proj_block_build(const void* D, int m, int64_t batch, int K,
                                        const double* proj, int nproj, void* out, void* stream) {
  QSX_CHECK_ARG(m >= 1 && m <= 8 && K >= 1 && K <= 256 && nproj >= 1 && nproj <= 4 &&
                    batch >= 0,
                "qsx_rk4_proj_block_build: bad sizes (m=%d, K=%d, nproj=%d)", m, K, nproj);
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(D && proj && out, "qsx_rk4_proj_block_build: null pointer");
  proj_block_build_w_kernel<<<(unsigned)((batch + PBW_WARPS - 1) / PBW_WARPS), 32 * PBW_WARPS, 0,
                              (cudaStream_t)stream>>>((const float2*)D, m, K,
                                                      (const double2*)proj, nproj, batch,
                                                      (float2*)out);
  QSX_LAUNCH_CHECK("qsx_rk4_proj_block_build");
  return QSX_OK;
}

extern "C" size_t qsx_rk4_proj_block_workspace_bytes(int m, int64_t batch, int K, int nsteps,
                                                     int nproj) {
  PbPlan pl;
  if (m < 1 || m > 8 || K < 1 || nproj < 1 || batch <= 0 ||
      projblock_plan(m, batch, K, nsteps, nproj, &pl) != QSX_OK)
    return 0;
  return (size_t)pl.grid * (nsteps + 1) * nproj * sizeof(double2);
}

extern "C" int qsx_rk4_proj_block_mean(const void* matrix, int m, int64_t batch, int K,
                                       int nsteps, const double* y0, int64_t y0_stride,
                                       int nproj, double* out_mean, void* workspace,
                                       size_t workspace_bytes, int32_t* status, void* stream) {
  QSX_CHECK_ARG(m >= 1 && m <= 8 && K >= 1 && nsteps >= 0 && nsteps % K == 0 && nproj >= 1 &&
                    nproj <= 4 && batch >= 0 && batch <= 0x7fffffffLL,
                "qsx_rk4_proj_block_mean: bad sizes (m=%d, K=%d, nsteps=%d, nproj=%d)", m, K,
                nsteps, nproj);
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(matrix && y0 && out_mean && workspace, "qsx_rk4_proj_block_mean: null pointer");
  PbPlan pl;
  int st = projblock_plan(m, batch, K, nsteps, nproj, &pl);
  if (st) return st;
  const int64_t per = (int64_t)(nsteps + 1) * nproj;
  const size_t need = (size_t)pl.grid * per * sizeof(double2);
  QSX_CHECK_ARG(workspace_bytes >= need,
                "qsx_rk4_proj_block_mean: workspace of %zu bytes needed (got %zu)", need,
                workspace_bytes);
  PbP p;
  p.nsteps = nsteps;
  p.nsave = nsteps + 1;
  p.P = nproj;
  p.batch = batch;
  p.matrix = (const float2*)matrix;
  p.y0 = (const double2*)y0;
  p.y0_stride = y0_stride;
  p.partial = (double2*)workspace;
  p.status = status;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaSuccess;
  if (pl.warp_form) {
    switch (m) {
#define C(MM)                                                                               \
  case MM:                                                                                  \
    rk4_projblock_w_f32<MM><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(p, K);            \
    break;
      C(1) C(2) C(3) C(4) C(5) C(6) C(7) C(8)
#undef C
    }
    QSX_LAUNCH_CHECK("qsx_rk4_proj_block_mean");
    projblock_reduce_kernel<<<(unsigned)((per + 31) / 32), 256, 0, s>>>(
        (const double2*)workspace, pl.grid, per, 1.0 / (double)batch, (double2*)out_mean);
    QSX_LAUNCH_CHECK("qsx_rk4_proj_block_mean reduce");
    return QSX_OK;
  }
  switch (m) {
#define C(MM)                                                                             \
  case MM:                                                                                \
    e = cudaFuncSetAttribute(rk4_projblock_f32<MM>,                                       \
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem);  \
    if (e == cudaSuccess)                                                                 \
      rk4_projblock_f32<MM><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(p, pl.ngroups, \
                                                                           pl.G, K);      \
    break;
    C(1) C(2) C(3) C(4) C(5) C(6) C(7) C(8)
#undef C
  }
  if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_proj_block_mean");
  QSX_LAUNCH_CHECK("qsx_rk4_proj_block_mean");
  projblock_reduce_kernel<<<(unsigned)((per + 31) / 32), 256, 0, s>>>(
      (const double2*)workspace, pl.grid, per, 1.0 / (double)batch, (double2*)out_mean);
  QSX_LAUNCH_CHECK("qsx_rk4_proj_block_mean reduce");
  return QSX_OK;
}

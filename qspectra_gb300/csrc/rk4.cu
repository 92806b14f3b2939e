// Batched fixed-step RK4 time loop for dy/dt = L y (one independent L per
// disorder sample), replacing integrate() of qspectra/simulate/utils.py:16-109
// and the serial ensemble loop of qspectra/simulate/decorators.py:40-64.
//
// Three kernels, chosen by qsx_rk4_batched:
//   rk4_small_f32<M>  M <= 8, one thread per sample, propagator D = P - I in
//                     registers, split-word FP32 state (absorption 'eg').
//   rk4_rows_f32<M,G> M in {9,16,25,36,49,64}: one thread per row of D held
//                     in registers, G samples per CTA, persistent grid,
//                     state broadcast through shared memory (population 'ee').
//   rk4_generic<T>    any M <= 4096, FP64 or FP32, propagator or RK4 stage
//                     form, one CTA per sample, matrix in shared memory when
//                     it fits (the plain FP64 form and odd sizes).
// Ensemble means are reduced deterministically: every kernel writes partial
// sums per "slot" (warp, CTA or sample) into caller workspace and
// rk4_reduce_kernel sums the slots in a fixed order in FP64.
#include <atomic>
#include <algorithm>

#include "qsx_common.cuh"

namespace qsx {

struct Rk4P {
  int m, nsteps, save_every, nsave, nproj, nselect, nout, form;
  int64_t batch;
  const void* matrix;
  int64_t matrix_stride;
  double h;
  const double2* y0;
  int64_t y0_stride;
  const double2* proj;
  int64_t proj_stride;
  const int* select;
  double2* out_state;
  double2* out_proj;
  double2* partial;   // generic kernel: [nslots][nsave][nout] double2, or null
  float2* partial32;  // FP32 kernels: [nslots][nsave][nout] float2, or null
  int* status;
};

__device__ __forceinline__ float2 f2(double2 v) { return make_float2((float)v.x, (float)v.y); }

// ---------------------------------------------------------------- small M
// rk4_lanes_f32<M>: M <= 8.  LPS lanes per sample (a power of two dividing
// 32), lane q holding rows [q*R, q*R + R) of D and of the state in registers.
// One lane per sample (the default) keeps the whole M x M matrix and state in
// the lane's registers: no gather shuffles, 32 samples per warp, so the loop
// issues a few instructions per sample-step instead of the shuffle traffic.
// Each step gathers the M state values with shuffles, updates its rows in
// split-word FP32 and, at save steps, folds the projections of all samples
// of the warp into one FP32 partial sum per warp (slot = warp).
template <int M>
__host__ __device__ constexpr int lanes_per_sample() {
  return M == 8 ? 2 : 1;  // M = 8 on one lane would exceed the register budget
}

__host__ __device__ constexpr int lanes_per_sample_rt(int m) {
  return m == 8 ? 2 : 1;
}

constexpr int LANES_MAXPROJ = 4;

template <int M>
__global__ void __launch_bounds__(128) rk4_lanes_f32(Rk4P p) {
  constexpr int LPS = lanes_per_sample<M>();
  constexpr int R = (M + LPS - 1) / LPS;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t s = gt / LPS;
  const int q = (int)(gt % LPS);
  const bool valid = s < p.batch;
  const unsigned lane = threadIdx.x & 31;
  const int base = (int)(lane & ~(unsigned)(LPS - 1));
  const int64_t slot = gt >> 5;
  float2 D[R][M];
  float yh[R][2], yl[R][2];
  const float2* dm = (const float2*)p.matrix + (valid ? s * p.matrix_stride : 0);
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int row = q * R + i;
#pragma unroll
    for (int j = 0; j < M; ++j)
      D[i][j] = (valid && row < M) ? dm[row * M + j] : make_float2(0.f, 0.f);
    double2 v = (valid && row < M) ? p.y0[s * p.y0_stride + row] : make_double2(0.0, 0.0);
    yh[i][0] = (float)v.x;
    yh[i][1] = (float)v.y;
    yl[i][0] = (float)(v.x - (double)yh[i][0]);
    yl[i][1] = (float)(v.y - (double)yh[i][1]);
  }
  // projection rows for this lane's state components, in FP32 registers
  float2 W[LANES_MAXPROJ][R];
#pragma unroll
  for (int k = 0; k < LANES_MAXPROJ; ++k)
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int row = q * R + i;
      W[k][i] = (k < p.nproj && valid && row < M)
                    ? f2(p.proj[(p.proj_stride ? s * p.proj_stride : 0) + k * M + row])
                    : make_float2(0.f, 0.f);
    }
  int selrow[LANES_MAXPROJ];
#pragma unroll
  for (int k = 0; k < LANES_MAXPROJ; ++k) selrow[k] = k < p.nselect ? p.select[k] : -1;
  auto save = [&](int k) {
    if (p.out_state && valid) {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int row = q * R + i;
        if (row < M)
          p.out_state[(s * p.nsave + k) * M + row] =
              make_double2((double)yh[i][0] + (double)yl[i][0], (double)yh[i][1] + (double)yl[i][1]);
      }
    }
#pragma unroll
    for (int o = 0; o < LANES_MAXPROJ; ++o) {
      if (o >= p.nout) break;
      float vx = 0.f, vy = 0.f;
#pragma unroll
      for (int i = 0; i < R; ++i) {
        if (p.nproj) {
          vx = fmaf(W[o][i].x, yh[i][0], vx);
          vx = fmaf(-W[o][i].y, yh[i][1], vx);
          vy = fmaf(W[o][i].x, yh[i][1], vy);
          vy = fmaf(W[o][i].y, yh[i][0], vy);
        } else if (q * R + i == selrow[o]) {
          vx = yh[i][0];
          vy = yh[i][1];
        }
      }
      if (!valid) vx = vy = 0.f;
      // per-sample value: sum over the sample's LPS lanes
      float sx = vx, sy = vy;
#pragma unroll
      for (int d = 1; d < LPS; d <<= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, d);
        sy += __shfl_xor_sync(0xffffffffu, sy, d);
      }
      if (p.out_proj && valid && q == 0)
        p.out_proj[(s * p.nsave + k) * p.nout + o] = make_double2(sx, sy);
      if (p.partial32) {
#pragma unroll
        for (int d = LPS; d < 32; d <<= 1) {
          sx += __shfl_xor_sync(0xffffffffu, sx, d);
          sy += __shfl_xor_sync(0xffffffffu, sy, d);
        }
        if (lane == 0) p.partial32[(slot * p.nsave + k) * p.nout + o] = make_float2(sx, sy);
      }
    }
  };
  save(0);
  for (int step = 1; step <= p.nsteps; ++step) {
    // two partial sums per row (even / odd j) halve the dependent FMA chain
    float zx[R][2], zy[R][2];
#pragma unroll
    for (int i = 0; i < R; ++i) zx[i][0] = zy[i][0] = zx[i][1] = zy[i][1] = 0.f;
#pragma unroll
    for (int j = 0; j < M; ++j) {
      // one lane per sample holds the whole state; otherwise gather it
      const float vx = LPS == 1 ? yh[j][0] : __shfl_sync(0xffffffffu, yh[j % R][0], base + j / R);
      const float vy = LPS == 1 ? yh[j][1] : __shfl_sync(0xffffffffu, yh[j % R][1], base + j / R);
#pragma unroll
      for (int i = 0; i < R; ++i) {
        zx[i][j & 1] = fmaf(D[i][j].x, vx, zx[i][j & 1]);
        zx[i][j & 1] = fmaf(-D[i][j].y, vy, zx[i][j & 1]);
        zy[i][j & 1] = fmaf(D[i][j].x, vy, zy[i][j & 1]);
        zy[i][j & 1] = fmaf(D[i][j].y, vx, zy[i][j & 1]);
      }
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
      dd_add(yh[i][0], yl[i][0], zx[i][0] + zx[i][1]);
      dd_add(yh[i][1], yl[i][1], zy[i][0] + zy[i][1]);
    }
    if (step % p.save_every == 0) save(step / p.save_every);
  }
  if (valid && p.status) {
    bool ok = true;
#pragma unroll
    for (int i = 0; i < R; ++i) ok = ok && isfinite(yh[i][0]) && isfinite(yh[i][1]);
    if (!ok) atomicOr(p.status, QSX_ERR_NONFINITE);
  }
}

// ------------------------------------------------------------- rows (ee)
__host__ __device__ constexpr int rows_stride(int M) {
  // float2 elements per sample slot: even (16-byte pairs) and == 2 mod 16 so
  // the samples sharing a warp read from different bank quads.
  int mp = (M % 2) ? M + 1 : M;
  while (mp % 16 != 2) mp += 2;
  return mp;
}

template <int M, int G, int MINB>
__global__ void __launch_bounds__(256, MINB) rk4_rows_f32(Rk4P p, int64_t ngroups) {
  constexpr int ST = rows_stride(M);
  constexpr int MP = (M % 2) ? M + 1 : M;
  __shared__ __align__(16) float2 ybuf[2][G][ST];
  __shared__ float2 stash[2][G][M];
  const int tid = threadIdx.x;
  const int g = tid / M, r = tid % M;
  const bool active = tid < G * M;
  // zero the padding column once (pairs read up to MP - 1)
  if (tid < G) {
    for (int j = M; j < ST; ++j) {
      ybuf[0][tid][j] = make_float2(0.f, 0.f);
      ybuf[1][tid][j] = make_float2(0.f, 0.f);
    }
  }
  // this thread's output slot: the first q with select[q] == r (host checks
  // that the select entries are distinct and in range)
  int myq = -1;
  if (active)
    for (int q = 0; q < p.nout; ++q)
      if (p.select[q] == r) { myq = q; break; }
  int savecount = 0;
  for (int64_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int64_t s = grp * G + g;
    const bool valid = active && s < p.batch;
    float2 drow[M];
    const float2* dm = (const float2*)p.matrix + (valid ? s * p.matrix_stride + (int64_t)r * M : 0);
#pragma unroll
    for (int j = 0; j < M; ++j) drow[j] = valid ? dm[j] : make_float2(0.f, 0.f);
    float yhx = 0.f, yhy = 0.f, ylx = 0.f, yly = 0.f;
    if (valid) {
      double2 v = p.y0[s * p.y0_stride + r];
      yhx = (float)v.x;
      yhy = (float)v.y;
      ylx = (float)(v.x - (double)yhx);
      yly = (float)(v.y - (double)yhy);
    }
    if (active) ybuf[0][g][r] = make_float2(yhx, yhy);
    __syncthreads();
    // per-sample outputs go straight to global memory; ensemble partial sums
    // are staged per sample in shared memory and summed over the G samples
    // by threads q < nout after the step barrier, then stored (no
    // read-modify-write) into this group's slot of the workspace.
    auto save = [&](int k, int par) {
      if (!active) return;
      if (p.out_state && valid)
        p.out_state[(s * p.nsave + k) * M + r] =
            make_double2((double)yhx + (double)ylx, (double)yhy + (double)yly);
      if (myq >= 0) {
        if (p.out_proj && valid)
          p.out_proj[(s * p.nsave + k) * p.nout + myq] =
              make_double2((double)yhx + (double)ylx, (double)yhy + (double)yly);
        if (p.partial32) stash[par][g][myq] = valid ? make_float2(yhx, yhy) : make_float2(0.f, 0.f);
      }
    };
    auto reduce = [&](int k, int par) {
      if (!p.partial32) return;
      for (int q = tid; q < p.nout; q += blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int gg = 0; gg < G; ++gg) {
          acc.x += stash[par][gg][q].x;
          acc.y += stash[par][gg][q].y;
        }
        p.partial32[(grp * p.nsave + k) * p.nout + q] = acc;
      }
    };
    save(0, savecount & 1);
    __syncthreads();
    reduce(0, savecount & 1);
    ++savecount;
    for (int step = 1; step <= p.nsteps; ++step) {
      const float2* cur = ybuf[(step - 1) & 1][active ? g : 0];
      float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < MP; j += 2) {
        const float4 v = *reinterpret_cast<const float4*>(&cur[j]);
        cfma(a0, drow[j], make_float2(v.x, v.y));
        if (j + 1 < M) cfma(a1, drow[j + 1], make_float2(v.z, v.w));
      }
      dd_add(yhx, ylx, a0.x + a1.x);
      dd_add(yhy, yly, a0.y + a1.y);
      if (active) ybuf[step & 1][g][r] = make_float2(yhx, yhy);
      const bool sv = (step % p.save_every) == 0;
      if (sv) save(step / p.save_every, savecount & 1);
      __syncthreads();
      if (sv) {
        reduce(step / p.save_every, savecount & 1);
        ++savecount;
      }
    }
    if (valid && p.status && !(isfinite(yhx) && isfinite(yhy))) atomicOr(p.status, QSX_ERR_NONFINITE);
    __syncthreads();
  }
}

// ---------------------------------------------------- K-step blocked rows
// rk4_block_f32<M>: the matrix of each sample has RT = M + nsel (K-1) rows
// (qsx_rk4_block_matrix_batched): rows < M hold D_K = P^K - I, row
// M + (k-1) nsel + q holds row select[q] of D_k.  One pass of the same
// row-per-thread matrix-vector product as rk4_rows_f32 then advances the
// state by K RK4 steps (main rows, split-word FP32) and yields the selected
// components at the K - 1 intermediate steps (extra rows: y[sel] + z).
// Outputs every step; ensemble partial sums per group as in rk4_rows_f32.
template <int M>
__global__ void __launch_bounds__(256, 2) rk4_block_f32(Rk4P p, int64_t ngroups, int G, int K) {
  constexpr int ST = rows_stride(M);
  constexpr int MP = (M % 2) ? M + 1 : M;
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* ybuf = (float2*)smraw;             // [2][G][ST]
  float2* stash = ybuf + 2 * G * ST;         // [2][K][G][nsel]
  const int nsel = p.nselect;
  if (!select_table_valid(p.select, nsel, M, p.status)) return;
  const int RT = M + nsel * (K - 1);
  const int tid = threadIdx.x;
  const int g = tid / RT, r = tid % RT;
  const bool active = tid < G * RT;
  const bool main_row = active && r < M;
  const int kx = main_row ? K : (r - M) / nsel + 1;  // step offset this row yields
  const int qx = main_row ? -1 : (r - M) % nsel;
  int myq = -1;  // main rows: the select slot this row fills at offset K
  if (main_row)
    for (int q = 0; q < nsel; ++q)
      if (p.select[q] == r) { myq = q; break; }
  const int selr = (active && !main_row) ? p.select[qx] : 0;
  for (int e = tid; e < 2 * G * ST; e += blockDim.x) ybuf[e] = make_float2(0.f, 0.f);
  __syncthreads();
  auto stash_at = [&](int par, int k, int gg, int q) -> float2& {
    return stash[((par * K + k) * G + gg) * nsel + q];
  };
  int parity = 0;
  for (int64_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int64_t s = grp * G + g;
    const bool valid = active && s < p.batch;
    float2 drow[M];
    const float2* dm = (const float2*)p.matrix + (valid ? s * p.matrix_stride + (int64_t)r * M : 0);
#pragma unroll
    for (int j = 0; j < M; ++j) drow[j] = valid ? dm[j] : make_float2(0.f, 0.f);
    float yhx = 0.f, yhy = 0.f, ylx = 0.f, yly = 0.f;
    if (valid && main_row) {
      double2 v = p.y0[s * p.y0_stride + r];
      yhx = (float)v.x;
      yhy = (float)v.y;
      ylx = (float)(v.x - (double)yhx);
      yly = (float)(v.y - (double)yhy);
    }
    if (main_row) ybuf[g * ST + r] = make_float2(yhx, yhy);
    // step 0: selected components of y0
    if (myq >= 0) {
      stash_at(parity, 0, g, myq) = make_float2(yhx, yhy);
      if (p.out_proj && valid)
        p.out_proj[(s * p.nsave) * p.nout + myq] =
            make_double2((double)yhx + (double)ylx, (double)yhy + (double)yly);
    }
    __syncthreads();
    // ensemble partial sums: FP64 fire-and-forget adds into this CTA's slice;
    // a given (step, q) is always added by the same thread, in program order
    if (p.partial)
      for (int q = tid; q < nsel; q += blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
        for (int gg = 0; gg < G; ++gg) acc = cadd2(acc, stash_at(parity, 0, gg, q));
        double2* dst = p.partial + ((int64_t)blockIdx.x * p.nsave) * p.nout + q;
        atomicAdd(&dst->x, (double)acc.x);
        atomicAdd(&dst->y, (double)acc.y);
      }
    parity ^= 1;
    const int nblk = p.nsteps / K;
    for (int bs = 0; bs < nblk; ++bs) {
      const float2* cur = ybuf + ((bs & 1) * G + (active ? g : 0)) * ST;
      float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < MP; j += 2) {
        const float4 v = *reinterpret_cast<const float4*>(&cur[j]);
        cfma(a0, drow[j], make_float2(v.x, v.y));
        if (j + 1 < M) cfma(a1, drow[j + 1], make_float2(v.z, v.w));
      }
      const int step0 = bs * K;
      if (main_row) {
        dd_add(yhx, ylx, a0.x + a1.x);
        dd_add(yhy, yly, a0.y + a1.y);
        ybuf[(((bs + 1) & 1) * G + g) * ST + r] = make_float2(yhx, yhy);
        if (myq >= 0) {
          stash_at(parity, K - 1, g, myq) = valid ? make_float2(yhx, yhy) : make_float2(0.f, 0.f);
          if (p.out_proj && valid)
            p.out_proj[(s * p.nsave + step0 + K) * p.nout + myq] =
                make_double2((double)yhx + (double)ylx, (double)yhy + (double)yly);
        }
      } else if (active) {
        const float2 base = cur[selr];
        const float2 v = valid ? make_float2(base.x + a0.x + a1.x, base.y + a0.y + a1.y)
                               : make_float2(0.f, 0.f);
        stash_at(parity, kx - 1, g, qx) = v;
        if (p.out_proj && valid)
          p.out_proj[(s * p.nsave + step0 + kx) * p.nout + qx] = make_double2(v.x, v.y);
      }
      __syncthreads();
      if (p.partial)
        for (int e = tid; e < K * nsel; e += blockDim.x) {
          const int k = e / nsel, q = e % nsel;
          float2 acc = make_float2(0.f, 0.f);
          for (int gg = 0; gg < G; ++gg) acc = cadd2(acc, stash_at(parity, k, gg, q));
          double2* dst = p.partial + ((int64_t)blockIdx.x * p.nsave + step0 + k + 1) * p.nout + q;
          atomicAdd(&dst->x, (double)acc.x);
          atomicAdd(&dst->y, (double)acc.y);
        }
      parity ^= 1;
    }
    if (valid && main_row && p.status && !(isfinite(yhx) && isfinite(yhy)))
      atomicOr(p.status, QSX_ERR_NONFINITE);
    __syncthreads();
  }
}

// rk4_block2_f32<M, LPR>: the same K-step blocked loop with each row split
// over LPR lanes of one warp (lanes l, l ^ 8, l ^ 16, ... holding column
// pairs [part HP, (part + 1) HP)): 1/LPR of the register-resident matrix row
// and of the dependent FMA chain per thread, log2(LPR) shuffles to combine.
// Rows of a sample fill whole warps (32 / LPR rows per warp), G samples per
// CTA.
template <int M, int LPR>
__global__ void __launch_bounds__(448, 2) rk4_block2_f32(Rk4P p, int64_t ngroups, int G, int K) {
  constexpr int ST = rows_stride(M);
  constexpr int MP = (M % 2) ? M + 1 : M;
  constexpr int NPAIR = MP / 2;
  constexpr int HP = (NPAIR + LPR - 1) / LPR;  // column pairs per lane
  constexpr int RPW = 32 / LPR;                // rows per warp
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* ybuf = (float2*)smraw;             // [2][G][ST]
  float2* stash = ybuf + 2 * G * ST;         // [2][K][G][nsel]
  const int nsel = p.nselect;
  if (!select_table_valid(p.select, nsel, M, p.status)) return;
  const int RT = M + nsel * (K - 1);
  const int wps = (RT + RPW - 1) / RPW;      // warps per sample
  const int tid = threadIdx.x, lane = tid & 31, wi = tid >> 5;
  const int g = wi / wps;
  const int r = (wi % wps) * RPW + (lane % RPW);
  const int part = lane / RPW;
  const bool active = g < G && r < RT;
  const bool main_row = active && r < M;
  const bool writer = active && part == 0;
  const int kx = main_row ? K : (active ? (r - M) / nsel + 1 : 0);
  const int qx = (active && !main_row) ? (r - M) % nsel : -1;
  int myq = -1;
  if (main_row)
    for (int q = 0; q < nsel; ++q)
      if (p.select[q] == r) { myq = q; break; }
  const int selr = (active && !main_row) ? p.select[qx] : 0;
  for (int e = tid; e < 2 * G * ST; e += blockDim.x) ybuf[e] = make_float2(0.f, 0.f);
  __syncthreads();
  auto stash_at = [&](int par, int k, int gg, int q) -> float2& {
    return stash[((par * K + k) * G + gg) * nsel + q];
  };
  const int gs = active ? g : 0;
  int parity = 0;
  for (int64_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int64_t s = grp * G + gs;
    const bool valid = active && s < p.batch;
    float2 drow[2 * HP];
    const float2* dm = (const float2*)p.matrix + (valid ? s * p.matrix_stride + (int64_t)r * M : 0);
#pragma unroll
    for (int t = 0; t < 2 * HP; ++t) {
      const int j = part * 2 * HP + t;
      drow[t] = (valid && j < M) ? dm[j] : make_float2(0.f, 0.f);
    }
    float yhx = 0.f, yhy = 0.f, ylx = 0.f, yly = 0.f;
    if (valid && main_row) {
      double2 v = p.y0[s * p.y0_stride + r];
      yhx = (float)v.x;
      yhy = (float)v.y;
      ylx = (float)(v.x - (double)yhx);
      yly = (float)(v.y - (double)yhy);
    }
    if (main_row && part == 0) ybuf[g * ST + r] = make_float2(yhx, yhy);
    if (myq >= 0 && part == 0) {
      stash_at(parity, 0, g, myq) = make_float2(yhx, yhy);
      if (p.out_proj && valid)
        p.out_proj[(s * p.nsave) * p.nout + myq] =
            make_double2((double)yhx + (double)ylx, (double)yhy + (double)yly);
    }
    __syncthreads();
    if (p.partial)
      for (int q = tid; q < nsel; q += blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
        for (int gg = 0; gg < G; ++gg) acc = cadd2(acc, stash_at(parity, 0, gg, q));
        double2* dst = p.partial + ((int64_t)blockIdx.x * p.nsave) * p.nout + q;
        atomicAdd(&dst->x, (double)acc.x);
        atomicAdd(&dst->y, (double)acc.y);
      }
    parity ^= 1;
    const int nblk = p.nsteps / K;
    for (int bs = 0; bs < nblk; ++bs) {
      const float2* cur = ybuf + ((bs & 1) * G + gs) * ST;
      float2 a0 = make_float2(0.f, 0.f), a1 = a0;
#pragma unroll
      for (int t = 0; t < HP; ++t) {
        const int pr = part * HP + t;
        if (pr < NPAIR) {
          const float4 v = *reinterpret_cast<const float4*>(&cur[2 * pr]);
          cfma(a0, drow[2 * t], make_float2(v.x, v.y));
          cfma(a1, drow[2 * t + 1], make_float2(v.z, v.w));
        }
      }
      float sx = a0.x + a1.x, sy = a0.y + a1.y;
#pragma unroll
      for (int o = 16; o >= RPW; o >>= 1) {
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
      }
      const int step0 = bs * K;
      if (writer && main_row) {
        dd_add(yhx, ylx, sx);
        dd_add(yhy, yly, sy);
        ybuf[(((bs + 1) & 1) * G + g) * ST + r] = make_float2(yhx, yhy);
        if (myq >= 0) {
          stash_at(parity, K - 1, g, myq) = valid ? make_float2(yhx, yhy) : make_float2(0.f, 0.f);
          if (p.out_proj && valid)
            p.out_proj[(s * p.nsave + step0 + K) * p.nout + myq] =
                make_double2((double)yhx + (double)ylx, (double)yhy + (double)yly);
        }
      } else if (writer) {
        const float2 base = cur[selr];
        const float2 v = valid ? make_float2(base.x + sx, base.y + sy) : make_float2(0.f, 0.f);
        stash_at(parity, kx - 1, g, qx) = v;
        if (p.out_proj && valid)
          p.out_proj[(s * p.nsave + step0 + kx) * p.nout + qx] = make_double2(v.x, v.y);
      }
      __syncthreads();
      if (p.partial)
        for (int e = tid; e < K * nsel; e += blockDim.x) {
          const int k = e / nsel, q = e % nsel;
          float2 acc = make_float2(0.f, 0.f);
          for (int gg = 0; gg < G; ++gg) acc = cadd2(acc, stash_at(parity, k, gg, q));
          double2* dst = p.partial + ((int64_t)blockIdx.x * p.nsave + step0 + k + 1) * p.nout + q;
          atomicAdd(&dst->x, (double)acc.x);
          atomicAdd(&dst->y, (double)acc.y);
        }
      parity ^= 1;
    }
    if (valid && main_row && part == 0 && p.status && !(isfinite(yhx) && isfinite(yhy)))
      atomicOr(p.status, QSX_ERR_NONFINITE);
    __syncthreads();
  }
}

// rk4_block3_f32<M, LPR>: the K-step blocked loop with each thread holding
// TWO rows over 1/LPR of the columns (lanes l, l ^ 8, l ^ 16, ... split the
// columns): every state value read from shared memory feeds two rows,
// halving the shared-memory traffic per FMA of rk4_block_f32, with
// log2(LPR) shuffles to combine.  Row pairs of a sample fill whole warps
// (32 / LPR pairs per warp), G samples per CTA.
template <int M, int LPR>
__global__ void __launch_bounds__(256, 2) rk4_block3_f32(Rk4P p, int64_t ngroups, int G, int K) {
  constexpr int ST = rows_stride(M);
  constexpr int MP = (M % 2) ? M + 1 : M;
  constexpr int NPAIR = MP / 2;
  constexpr int HP = (NPAIR + LPR - 1) / LPR;  // column pairs per lane
  constexpr int RPW = 32 / LPR;                // row pairs per warp
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* ybuf = (float2*)smraw;             // [2][G][ST]
  float2* stash = ybuf + 2 * G * ST;         // [2][K][G][nsel]
  const int nsel = p.nselect;
  if (!select_table_valid(p.select, nsel, M, p.status)) return;
  const int RT = M + nsel * (K - 1);
  const int NRP = (RT + 1) / 2;              // row pairs per sample
  const int wps = (NRP + RPW - 1) / RPW;     // warps per sample
  const int tid = threadIdx.x, lane = tid & 31, wi = tid >> 5;
  const int g = wi / wps;
  const int rp = (wi % wps) * RPW + (lane % RPW);
  const int part = lane / RPW;
  const int gs = g < G ? g : 0;
  int r2[2];
  bool act[2], mrow[2];
  int kx[2], qx[2], myq[2], selr[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int r = 2 * rp + u;
    r2[u] = r;
    act[u] = g < G && rp < NRP && r < RT;
    mrow[u] = act[u] && r < M;
    kx[u] = mrow[u] ? K : (act[u] ? (r - M) / nsel + 1 : 0);
    qx[u] = (act[u] && !mrow[u]) ? (r - M) % nsel : -1;
    myq[u] = -1;
    if (mrow[u])
      for (int q = 0; q < nsel; ++q)
        if (p.select[q] == r) { myq[u] = q; break; }
    selr[u] = (act[u] && !mrow[u]) ? p.select[qx[u]] : 0;
  }
  for (int e = tid; e < 2 * G * ST; e += blockDim.x) ybuf[e] = make_float2(0.f, 0.f);
  __syncthreads();
  auto stash_at = [&](int par, int k, int gg, int q) -> float2& {
    return stash[((par * K + k) * G + gg) * nsel + q];
  };
  int parity = 0;
  for (int64_t grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
    const int64_t s = grp * G + gs;
    const bool svalid = g < G && s < p.batch;
    float2 drow[2][2 * HP];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const bool v = svalid && act[u];
      const float2* dm = (const float2*)p.matrix + (v ? s * p.matrix_stride + (int64_t)r2[u] * M : 0);
#pragma unroll
      for (int t = 0; t < 2 * HP; ++t) {
        const int j = part * 2 * HP + t;
        drow[u][t] = (v && j < M) ? dm[j] : make_float2(0.f, 0.f);
      }
    }
    float yhx[2] = {0.f, 0.f}, yhy[2] = {0.f, 0.f}, ylx[2] = {0.f, 0.f}, yly[2] = {0.f, 0.f};
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (svalid && mrow[u]) {
        double2 v = p.y0[s * p.y0_stride + r2[u]];
        yhx[u] = (float)v.x;
        yhy[u] = (float)v.y;
        ylx[u] = (float)(v.x - (double)yhx[u]);
        yly[u] = (float)(v.y - (double)yhy[u]);
      }
      if (mrow[u] && part == 0) ybuf[g * ST + r2[u]] = make_float2(yhx[u], yhy[u]);
      if (myq[u] >= 0 && part == 0) {
        stash_at(parity, 0, g, myq[u]) = make_float2(yhx[u], yhy[u]);
        if (p.out_proj && svalid)
          p.out_proj[(s * p.nsave) * p.nout + myq[u]] =
              make_double2((double)yhx[u] + (double)ylx[u], (double)yhy[u] + (double)yly[u]);
      }
    }
    __syncthreads();
    if (p.partial)
      for (int q = tid; q < nsel; q += blockDim.x) {
        float2 acc = make_float2(0.f, 0.f);
        for (int gg = 0; gg < G; ++gg) acc = cadd2(acc, stash_at(parity, 0, gg, q));
        double2* dst = p.partial + ((int64_t)blockIdx.x * p.nsave) * p.nout + q;
        atomicAdd(&dst->x, (double)acc.x);
        atomicAdd(&dst->y, (double)acc.y);
      }
    parity ^= 1;
    const int nblk = p.nsteps / K;
    for (int bs = 0; bs < nblk; ++bs) {
      const float2* cur = ybuf + ((bs & 1) * G + gs) * ST;
      float2 a0[2], a1[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) a0[u] = a1[u] = make_float2(0.f, 0.f);
#pragma unroll
      for (int t = 0; t < HP; ++t) {
        const int pr = part * HP + t;
        if (pr < NPAIR) {
          const float4 v = *reinterpret_cast<const float4*>(&cur[2 * pr]);
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            cfma(a0[u], drow[u][2 * t], make_float2(v.x, v.y));
            cfma(a1[u], drow[u][2 * t + 1], make_float2(v.z, v.w));
          }
        }
      }
      const int step0 = bs * K;
      float sx[2], sy[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        sx[u] = a0[u].x + a1[u].x;
        sy[u] = a0[u].y + a1[u].y;
#pragma unroll
        for (int o = 16; o >= RPW; o >>= 1) {
          sx[u] += __shfl_xor_sync(0xffffffffu, sx[u], o);
          sy[u] += __shfl_xor_sync(0xffffffffu, sy[u], o);
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (part != 0 || !act[u]) continue;
        if (mrow[u]) {
          dd_add(yhx[u], ylx[u], sx[u]);
          dd_add(yhy[u], yly[u], sy[u]);
          ybuf[(((bs + 1) & 1) * G + g) * ST + r2[u]] = make_float2(yhx[u], yhy[u]);
          if (myq[u] >= 0) {
            stash_at(parity, K - 1, g, myq[u]) =
                svalid ? make_float2(yhx[u], yhy[u]) : make_float2(0.f, 0.f);
            if (p.out_proj && svalid)
              p.out_proj[(s * p.nsave + step0 + K) * p.nout + myq[u]] = make_double2(
                  (double)yhx[u] + (double)ylx[u], (double)yhy[u] + (double)yly[u]);
          }
        } else {
          const float2 base = cur[selr[u]];
          const float2 v = svalid ? make_float2(base.x + sx[u], base.y + sy[u])
                                  : make_float2(0.f, 0.f);
          stash_at(parity, kx[u] - 1, g, qx[u]) = v;
          if (p.out_proj && svalid)
            p.out_proj[(s * p.nsave + step0 + kx[u]) * p.nout + qx[u]] = make_double2(v.x, v.y);
        }
      }
      __syncthreads();
      if (p.partial)
        for (int e = tid; e < K * nsel; e += blockDim.x) {
          const int k = e / nsel, q = e % nsel;
          float2 acc = make_float2(0.f, 0.f);
          for (int gg = 0; gg < G; ++gg) acc = cadd2(acc, stash_at(parity, k, gg, q));
          double2* dst = p.partial + ((int64_t)blockIdx.x * p.nsave + step0 + k + 1) * p.nout + q;
          atomicAdd(&dst->x, (double)acc.x);
          atomicAdd(&dst->y, (double)acc.y);
        }
      parity ^= 1;
    }
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (svalid && mrow[u] && part == 0 && p.status &&
          !(isfinite(yhx[u]) && isfinite(yhy[u])))
        atomicOr(p.status, QSX_ERR_NONFINITE);
    __syncthreads();
  }
}

// -------------------------------------------------------------- generic
constexpr int GEN_MAXR = 4;  // rows per thread (M <= 4 * 1024)

template <typename T>
__global__ void __launch_bounds__(1024) rk4_generic(Rk4P p, int mat_in_smem) {
  using C = typename cplx<T>::type;
  constexpr bool SPLIT = sizeof(T) == 4;
  extern __shared__ __align__(16) unsigned char sm[];
  const int M = p.m;
  double2* red = (double2*)sm;      // [32] block reduction (16-byte aligned first)
  C* ybuf = (C*)(red + 32);         // [2][M] current state (hi) / stage input
  C* smat = ybuf + 2 * M;           // [M][M] when it fits
  const int64_t s = blockIdx.x;
  const int tid = threadIdx.x, nt = blockDim.x;
  const C* gm = (const C*)p.matrix + s * p.matrix_stride;
  const C* mat = mat_in_smem ? smat : gm;
  if (mat_in_smem)
    for (int64_t e = tid; e < (int64_t)M * M; e += nt) smat[e] = gm[e];
  // per-row state in registers: y (hi, lo for FP32) and the stage accumulator
  C yh[GEN_MAXR], yl[GEN_MAXR], kac[GEN_MAXR];
#pragma unroll
  for (int k = 0; k < GEN_MAXR; ++k) {
    int r = tid + k * nt;
    double2 v = r < M ? p.y0[s * p.y0_stride + r] : make_double2(0.0, 0.0);
    yh[k] = cmk((T)v.x, (T)v.y);
    yl[k] = SPLIT ? cmk((T)(v.x - (double)yh[k].x), (T)(v.y - (double)yh[k].y)) : cmk((T)0, (T)0);
    kac[k] = cmk((T)0, (T)0);
    if (r < M) ybuf[r] = yh[k];
  }
  __syncthreads();
  const double2* W = p.proj + (p.nproj ? s * p.proj_stride : 0);
  auto save = [&](int k, const C* ycur) {
    if (p.out_state) {
#pragma unroll
      for (int q = 0; q < GEN_MAXR; ++q) {
        int r = tid + q * nt;
        if (r < M)
          p.out_state[(s * p.nsave + k) * M + r] =
              make_double2((double)yh[q].x + (double)yl[q].x, (double)yh[q].y + (double)yl[q].y);
      }
    }
    if (p.nselect) {
      for (int q = tid; q < p.nselect; q += nt) {
        const int si = p.select[q];
        if (si < 0 || si >= M) {  // bad index table: record it, touch nothing
          if (p.status) atomicOr(p.status, QSX_ERR_INVALID_ARG);
          continue;
        }
        C v = ycur[si];
        double2 dv = make_double2((double)v.x, (double)v.y);
        if (p.out_proj) p.out_proj[(s * p.nsave + k) * p.nout + q] = dv;
        if (p.partial) p.partial[(s * p.nsave + k) * p.nout + q] = dv;
      }
    }
    for (int q = 0; q < p.nproj; ++q) {
      double2 acc = make_double2(0.0, 0.0);
#pragma unroll
      for (int k2 = 0; k2 < GEN_MAXR; ++k2) {
        int r = tid + k2 * nt;
        if (r < M) {
          double2 yv = make_double2((double)yh[k2].x + (double)yl[k2].x,
                                    (double)yh[k2].y + (double)yl[k2].y);
          cfma(acc, W[(int64_t)q * M + r], yv);
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
      }
      if ((tid & 31) == 0) red[tid >> 5] = acc;
      __syncthreads();
      if (tid == 0) {
        double2 t = make_double2(0.0, 0.0);
        for (int w = 0; w < (nt + 31) / 32; ++w) t = cadd(t, red[w]);
        if (p.out_proj) p.out_proj[(s * p.nsave + k) * p.nout + q] = t;
        if (p.partial) p.partial[(s * p.nsave + k) * p.nout + q] = t;
      }
      __syncthreads();
    }
  };
  // y_out = mat * x for this thread's rows
  auto matvec = [&](const C* x, C* out) {
#pragma unroll
    for (int q = 0; q < GEN_MAXR; ++q) {
      int r = tid + q * nt;
      C acc = cmk((T)0, (T)0);
      if (r < M) {
        const C* row = mat + (int64_t)r * M;
        for (int j = 0; j < M; ++j) cfma(acc, row[j], x[j]);
      }
      out[q] = acc;
    }
  };
  auto add_state = [&](int q, C z) {
    if (SPLIT) {
      float hx = yh[q].x, lx = yl[q].x, hy = yh[q].y, ly = yl[q].y;
      dd_add(hx, lx, (float)z.x);
      dd_add(hy, ly, (float)z.y);
      yh[q] = cmk((T)hx, (T)hy);
      yl[q] = cmk((T)lx, (T)ly);
    } else {
      yh[q] = cmk(yh[q].x + z.x, yh[q].y + z.y);
    }
  };
  save(0, ybuf);
  __syncthreads();
  const T h = (T)p.h;
  // Invariant at the start of a step: ybuf[cur] holds the state (hi part).
  int cur = 0;
  for (int step = 1; step <= p.nsteps; ++step) {
    C* b0 = ybuf + cur * M;
    C* b1 = ybuf + (1 - cur) * M;
    C z[GEN_MAXR];
    if (p.form == 0) {
      // propagator form: y <- y + D y
      matvec(b0, z);
#pragma unroll
      for (int q = 0; q < GEN_MAXR; ++q) {
        int r = tid + q * nt;
        if (r < M) {
          add_state(q, z[q]);
          b1[r] = yh[q];
        }
      }
      __syncthreads();
      cur = 1 - cur;
    } else {
      // classical RK4 stages: inputs alternate b0 -> b1 -> b0 -> b1, new y -> b0
      const T half = h / (T)2;
#pragma unroll 1
      for (int st = 0; st < 4; ++st) {
        const C* in = (st & 1) ? b1 : b0;
        C* outb = (st & 1) ? b0 : b1;
        matvec(in, z);
#pragma unroll
        for (int q = 0; q < GEN_MAXR; ++q) {
          int r = tid + q * nt;
          if (r >= M) continue;
          if (st == 0) {
            kac[q] = z[q];
            outb[r] = cmk(yh[q].x + half * z[q].x, yh[q].y + half * z[q].y);
          } else if (st == 1) {
            kac[q] = cmk(kac[q].x + (T)2 * z[q].x, kac[q].y + (T)2 * z[q].y);
            outb[r] = cmk(yh[q].x + half * z[q].x, yh[q].y + half * z[q].y);
          } else if (st == 2) {
            kac[q] = cmk(kac[q].x + (T)2 * z[q].x, kac[q].y + (T)2 * z[q].y);
            outb[r] = cmk(yh[q].x + h * z[q].x, yh[q].y + h * z[q].y);
          } else {
            C inc = cmk((kac[q].x + z[q].x) * (h / (T)6), (kac[q].y + z[q].y) * (h / (T)6));
            add_state(q, inc);
            outb[r] = yh[q];
          }
        }
        __syncthreads();
      }
    }
    if (step % p.save_every == 0) save(step / p.save_every, ybuf + cur * M);
    __syncthreads();
  }
  if (p.status) {
    bool ok = true;
#pragma unroll
    for (int q = 0; q < GEN_MAXR; ++q)
      if (tid + q * nt < M) ok = ok && isfinite((double)yh[q].x) && isfinite((double)yh[q].y);
    if (!ok) atomicOr(p.status, QSX_ERR_NONFINITE);
  }
}

// ----------------------------------------------------------------- reduce
// out[e] = scale * sum over slots of partial[slot][e]: 32 outputs per CTA
// (one per lane, coalesced), slots strided over the 8 warps, the 8 partial
// sums combined in a fixed order (deterministic).
template <typename P>
__global__ void __launch_bounds__(256)
    rk4_reduce_kernel(const P* __restrict__ partial, int64_t nslots, int64_t per, double scale,
                      double2* out) {
  __shared__ double2 red[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t e = (int64_t)blockIdx.x * 32 + lane;
  double2 acc = make_double2(0.0, 0.0);
  if (e < per) {
    for (int64_t sl = w; sl < nslots; sl += 8) {
      P v = partial[sl * per + e];
      acc.x += (double)v.x;
      acc.y += (double)v.y;
    }
  }
  red[w][lane] = acc;
  __syncthreads();
  if (w == 0 && e < per) {
    double2 t = red[0][lane];
#pragma unroll
    for (int i = 1; i < 8; ++i) t = cadd(t, red[i][lane]);
    out[e] = cscale(t, scale);
  }
}

// ------------------------------------------------------------------ plan
enum Kind { K_SMALL = 0, K_ROWS = 1, K_GENERIC = 2, K_BLOCK = 3 };

struct Plan {
  Kind kind;
  int G;
  int lpr;  // K_BLOCK: lanes per matrix row (1: rk4_block_f32, 2: rk4_block2_f32)
  int64_t nslots;
  int64_t grid;
  int threads;
  size_t smem;
  int mat_in_smem;
  int64_t ngroups;
};

template <int M, int G, int MINB>
static cudaError_t rows_occupancy(int* blocks) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, rk4_rows_f32<M, G, MINB>, 256, 0);
}

#define QSX_ROWS_TABLE(X) X(9, 28, 2) X(16, 16, 2) X(25, 10, 2) X(36, 7, 2) X(49, 5, 2) X(64, 4, 1)
static bool rows_supported(int m, int* G) {
#define X(MM, GG, BB) if (m == MM) { *G = GG; return true; }
  QSX_ROWS_TABLE(X)
#undef X
  return false;
}

static size_t partial_bytes(Kind k) {
  return (k == K_GENERIC || k == K_BLOCK) ? sizeof(double2) : sizeof(float2);
}

static int validate(const qsx_rk4_args* a) {
  QSX_CHECK_ARG(a != nullptr, "qsx_rk4: null args");
  QSX_CHECK_ARG(a->precision == QSX_FP32 || a->precision == QSX_FP64, "qsx_rk4: bad precision");
  QSX_CHECK_ARG(a->form == 0 || a->form == 1, "qsx_rk4: form must be 0 (propagator) or 1 (stages)");
  QSX_CHECK_ARG(a->m >= 1 && a->m <= GEN_MAXR * 1024, "qsx_rk4: need 1 <= m <= %d (got %d)",
                GEN_MAXR * 1024, a->m);
  QSX_CHECK_ARG(a->nsteps >= 0 && a->save_every >= 1 && a->nsteps % a->save_every == 0,
                "qsx_rk4: nsteps must be a non-negative multiple of save_every");
  QSX_CHECK_ARG(a->batch >= 0 && a->batch <= 0x7fffffffLL, "qsx_rk4: bad batch");
  QSX_CHECK_ARG(!(a->nproj > 0 && a->nselect > 0), "qsx_rk4: use proj or select, not both");
  QSX_CHECK_ARG(a->block_k >= 0 && a->block_k <= 64, "qsx_rk4: block_k must be in [0, 64]");
  QSX_CHECK_ARG(a->nproj >= 0 && a->nproj <= 64 && a->nselect >= 0 && a->nselect <= a->m,
                "qsx_rk4: bad nproj/nselect");
  QSX_CHECK_ARG(a->nproj == 0 || a->proj, "qsx_rk4: proj is null");
  QSX_CHECK_ARG(a->nselect == 0 || a->select, "qsx_rk4: select is null");
  QSX_CHECK_ARG((a->out_proj == nullptr && a->out_mean == nullptr) || a->nproj + a->nselect > 0,
                "qsx_rk4: projections requested without proj/select");
  QSX_CHECK_ARG(a->batch == 0 || (a->matrix && a->y0), "qsx_rk4: null matrix or y0");
  return QSX_OK;
}

static int make_plan(const qsx_rk4_args* a, Plan* pl) {
  int G = 0;
  const int m = a->m;
  if (a->block_k > 1) {
    // K-step blocked rows kernel (matrix from qsx_rk4_block_matrix_batched)
    const int K = a->block_k;
    QSX_CHECK_ARG(a->precision == QSX_FP32 && a->form == 0 && a->nproj == 0 &&
                      a->nselect >= 1 && a->save_every == 1 && a->out_state == nullptr &&
                      a->nsteps % K == 0 && rows_supported(m, &G),
                  "qsx_rk4: block_k needs FP32, form 0, select outputs only, save_every 1, "
                  "nsteps %% block_k == 0 and m in {9,16,25,36,49,64}");
    const int RT = m + a->nselect * (K - 1);
    QSX_CHECK_ARG(RT <= 256, "qsx_rk4: block_k rows per sample exceed 256");
    QSX_CHECK_ARG(a->variant >= 0, "qsx_rk4: variant must be 0..5");
    // the planner's default, or the variant an autotuner picked: 1 = one
    // thread per row, 2 / 4 = that many lanes per row, 3 / 5 = two rows per
    // thread over two / four lanes
    QSX_CHECK_ARG(a->variant <= 5, "qsx_rk4: variant must be 0..5");
    const int lpr = a->variant ? a->variant : 1;
    int threads;
    if (lpr == 3 || lpr == 5) {
      const int rpw = lpr == 3 ? 16 : 8;  // row pairs per warp
      const int wps = ((RT + 1) / 2 + rpw - 1) / rpw;
      G = std::max(1, 256 / (wps * 32));
      threads = G * wps * 32;
    } else if (lpr > 1) {
      const int wps = (RT + 32 / lpr - 1) / (32 / lpr);
      G = std::max(1, 448 / (wps * 32));
      threads = G * wps * 32;
    } else {
      G = std::max(1, 256 / RT);
      threads = ((G * RT + 31) / 32) * 32;
    }
    // each variant is compiled for a maximum block size
    const int max_threads = (lpr == 2 || lpr == 4) ? 448 : 256;
    if (threads > max_threads) {
      set_error("qsx_rk4: variant %d needs %d threads for %d blocked rows (at most %d)", lpr,
                threads, RT, max_threads);
      return QSX_ERR_UNSUPPORTED;
    }
    int dev = 0, sms = 0, occ = 0;
    pl->smem = (2 * (size_t)G * 66 + 2 * (size_t)K * G * a->nselect) * sizeof(float2);
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
#define X(MM, GG, BB)                                                                      \
  if (e == cudaSuccess && m == MM)                                                         \
    e = lpr == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(                          \
                       &occ, rk4_block3_f32<MM, 2>, threads, pl->smem)                     \
        : lpr == 5 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(                          \
                       &occ, rk4_block3_f32<MM, 4>, threads, pl->smem)                     \
        : lpr == 4 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(                          \
                       &occ, rk4_block2_f32<MM, 4>, threads, pl->smem)                     \
        : lpr == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(                          \
                       &occ, rk4_block2_f32<MM, 2>, threads, pl->smem)                     \
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rk4_block_f32<MM>, \
                                                                   threads, pl->smem);
    QSX_ROWS_TABLE(X)
#undef X
    if (e != cudaSuccess) return cuda_status(e, "qsx_rk4 plan");
    pl->lpr = lpr;
    pl->kind = K_BLOCK;
    pl->G = G;
    pl->threads = threads;
    pl->ngroups = (a->batch + G - 1) / G;
    pl->grid = std::max<int64_t>(1, std::min<int64_t>(pl->ngroups, (int64_t)sms * std::max(occ, 1)));
    pl->nslots = pl->grid;  // one FP64 accumulator slice per CTA
    return QSX_OK;
  }
  const int64_t nsave = a->nsteps / a->save_every + 1;
  (void)nsave;
  if (a->precision == QSX_FP32 && a->form == 0 && m <= 8 && a->nproj <= LANES_MAXPROJ &&
      a->nselect <= LANES_MAXPROJ) {
    const int lps = lanes_per_sample_rt(m);
    const int64_t threads = a->batch * lps;
    pl->kind = K_SMALL;
    pl->threads = 128;
    pl->grid = (threads + 127) / 128;
    pl->nslots = pl->grid * 4;
    pl->smem = 0;
    return QSX_OK;
  }
  if (a->precision == QSX_FP32 && a->form == 0 && rows_supported(m, &G)) {
    // nselect-only outputs (the per-row kernel has no dense projection)
    if (a->nproj == 0) {
      int dev = 0, sms = 0, occ = 0;
      cudaError_t e = cudaGetDevice(&dev);
      if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
#define X(MM, GG, BB) \
  if (e == cudaSuccess && m == MM) e = rows_occupancy<MM, GG, BB>(&occ);
      QSX_ROWS_TABLE(X)
#undef X
      if (e != cudaSuccess) return cuda_status(e, "qsx_rk4 plan");
      pl->kind = K_ROWS;
      pl->threads = 256;
      pl->ngroups = (a->batch + G - 1) / G;
      pl->grid = std::max<int64_t>(1, std::min<int64_t>(pl->ngroups, (int64_t)sms * std::max(occ, 1)));
      pl->nslots = pl->ngroups;
      pl->smem = 0;
      return QSX_OK;
    }
  }
  pl->kind = K_GENERIC;
  int nt = ((std::min(m, 1024) + 31) / 32) * 32;
  QSX_CHECK_ARG((m + nt - 1) / nt <= GEN_MAXR, "qsx_rk4: m too large");
  pl->threads = nt;
  pl->grid = a->batch;
  pl->nslots = a->batch;
  size_t cs = a->precision == QSX_FP32 ? sizeof(float2) : sizeof(double2);
  size_t base = 2 * (size_t)m * cs + 32 * sizeof(double2);
  size_t mat = (size_t)m * m * cs;
  pl->mat_in_smem = (base + mat) <= 160 * 1024;
  pl->smem = base + (pl->mat_in_smem ? mat : 0);
  return QSX_OK;
}

}  // namespace qsx

using namespace qsx;

extern "C" {

size_t qsx_rk4_args_bytes(void) { return sizeof(qsx_rk4_args); }

int qsx_rk4_workspace_bytes(const qsx_rk4_args* a, size_t* bytes) {
  int st = validate(a);
  if (st) return st;
  QSX_CHECK_ARG(bytes != nullptr, "qsx_rk4_workspace_bytes: null output");
  *bytes = 0;
  if (a->out_mean == nullptr || a->batch == 0) return QSX_OK;
  Plan pl;
  st = make_plan(a, &pl);
  if (st) return st;
  const int64_t nsave = a->nsteps / a->save_every + 1;
  const int64_t nout = a->nproj > 0 ? a->nproj : a->nselect;
  *bytes = (size_t)pl.nslots * nsave * nout * partial_bytes(pl.kind);
  return QSX_OK;
}

int qsx_rk4_batched(const qsx_rk4_args* a, void* stream) {
  int st = validate(a);
  if (st) return st;
  if (a->batch == 0) return QSX_OK;
  Plan pl;
  st = make_plan(a, &pl);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  Rk4P p;
  p.m = a->m;
  p.nsteps = a->nsteps;
  p.save_every = a->save_every;
  p.nsave = a->nsteps / a->save_every + 1;
  p.nproj = a->nproj;
  p.nselect = a->nselect;
  p.nout = a->nproj > 0 ? a->nproj : a->nselect;
  p.form = a->form;
  p.batch = a->batch;
  p.matrix = a->matrix;
  p.matrix_stride = a->matrix_stride;
  p.h = a->h;
  p.y0 = (const double2*)a->y0;
  p.y0_stride = a->y0_stride;
  p.proj = (const double2*)a->proj;
  p.proj_stride = a->proj_stride;
  p.select = a->select;
  p.out_state = (double2*)a->out_state;
  p.out_proj = (double2*)a->out_proj;
  p.partial = nullptr;
  p.partial32 = nullptr;
  p.status = a->status;
  const int64_t per = (int64_t)p.nsave * p.nout;
  if (a->out_mean) {
    size_t need = (size_t)pl.nslots * per * partial_bytes(pl.kind);
    QSX_CHECK_ARG(a->workspace && a->workspace_bytes >= need,
                  "qsx_rk4_batched: workspace of %zu bytes needed (got %zu)", need,
                  a->workspace_bytes);
    if (pl.kind == K_GENERIC) {
      p.partial = (double2*)a->workspace;
    } else if (pl.kind == K_BLOCK) {
      p.partial = (double2*)a->workspace;  // accumulated with atomic adds: start at zero
      cudaError_t e = cudaMemsetAsync(a->workspace, 0, need, s);
      if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_batched memset");
    } else {
      p.partial32 = (float2*)a->workspace;
    }
  }
  switch (pl.kind) {
    case K_SMALL: {
      switch (a->m) {
#define S(MM) case MM: rk4_lanes_f32<MM><<<(unsigned)pl.grid, pl.threads, 0, s>>>(p); break;
        S(1) S(2) S(3) S(4) S(5) S(6) S(7) S(8)
#undef S
      }
      break;
    }
    case K_ROWS: {
#define X(MM, GG, BB) \
  if (a->m == MM) rk4_rows_f32<MM, GG, BB><<<(unsigned)pl.grid, 256, 0, s>>>(p, pl.ngroups);
      QSX_ROWS_TABLE(X)
#undef X
      break;
    }
    case K_BLOCK: {
#define X(MM, GG, BB)                                                                   \
  if (a->m == MM)                                                                       \
    if (pl.lpr == 3)                                                                    \
      rk4_block3_f32<MM, 2><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(             \
          p, pl.ngroups, pl.G, a->block_k);                                             \
    else if (pl.lpr == 5)                                                               \
      rk4_block3_f32<MM, 4><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(             \
          p, pl.ngroups, pl.G, a->block_k);                                             \
    else if (pl.lpr == 4)                                                               \
      rk4_block2_f32<MM, 4><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(             \
          p, pl.ngroups, pl.G, a->block_k);                                             \
    else if (pl.lpr == 2)                                                               \
      rk4_block2_f32<MM, 2><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(             \
          p, pl.ngroups, pl.G, a->block_k);                                             \
    else                                                                                \
      rk4_block_f32<MM><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(p, pl.ngroups, pl.G, \
                                                                      a->block_k);
      QSX_ROWS_TABLE(X)
#undef X
      break;
    }
    case K_GENERIC: {
      cudaError_t e;
      if (a->precision == QSX_FP32) {
        e = cudaFuncSetAttribute(rk4_generic<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)pl.smem);
        if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_batched");
        rk4_generic<float><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(p, pl.mat_in_smem);
      } else {
        e = cudaFuncSetAttribute(rk4_generic<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)pl.smem);
        if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_batched");
        rk4_generic<double><<<(unsigned)pl.grid, pl.threads, pl.smem, s>>>(p, pl.mat_in_smem);
      }
      break;
    }
  }
  QSX_LAUNCH_CHECK("qsx_rk4_batched");
  if (a->out_mean) {
    const unsigned rg = (unsigned)((per + 31) / 32);
    if (pl.kind == K_GENERIC || pl.kind == K_BLOCK)
      rk4_reduce_kernel<double2><<<rg, 256, 0, s>>>(p.partial, pl.nslots, per, a->mean_scale,
                                                    (double2*)a->out_mean);
    else
      rk4_reduce_kernel<float2><<<rg, 256, 0, s>>>(p.partial32, pl.nslots, per,
                                                   a->mean_scale, (double2*)a->out_mean);
    QSX_LAUNCH_CHECK("qsx_rk4_batched reduce");
  }
  return QSX_OK;
}

}  // extern "C"

// ------------------------------------------------ no-allocation variant
// Some callers cannot call cudaMalloc: a host application that owns all
// device memory through its own pool and forbids allocations by plug-ins, an
// embedded runtime with a fixed memory budget, or code running where an
// allocation could fail late (e.g. inside the host's own out-of-memory
// handling).  For them, qsx_rk4_block_mean_noalloc runs the K-step blocked
// ensemble-mean loop with its partial sums in the file-scope device array
// below instead of caller workspace.  The array is NOALLOC_SCRATCH_BYTES
// (16 MiB); every GPU that loads this library keeps it until the process
// exits.  Its device address is looked up once per device, by the first call
// made with that device current, so make that first call before any stream
// capture.  All calls share the array: two calls that overlap on the GPU
// (different streams, or threads) race on it, and each call clears the part
// it uses before running.
namespace qsx {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)16 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
// per-device cache of the array's address; host threads may call
// concurrently, so every access is atomic
static std::atomic<void*> g_noalloc_ptr[NOALLOC_MAX_DEVICES];

// Device address of g_noalloc_scratch on the current device (host code may
// not take the address of a __device__ array directly).  Outside a stream
// capture the address is looked up on every call (cheap, and right after a
// device reset); inside one the cached address of an earlier call is used.
static int noalloc_scratch(cudaStream_t s, void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_block_mean_noalloc: cudaGetDevice");
  QSX_CHECK_ARG(dev >= 0 && dev < NOALLOC_MAX_DEVICES,
                "qsx_rk4_block_mean_noalloc: device index %d not supported", dev);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(s, &cap);
  if (e != cudaSuccess)
    return cuda_status(e, "qsx_rk4_block_mean_noalloc: cudaStreamIsCapturing");
  if (cap == cudaStreamCaptureStatusNone) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess)
      return cuda_status(e, "qsx_rk4_block_mean_noalloc: cudaGetSymbolAddress");
    g_noalloc_ptr[dev].store(ptr, std::memory_order_release);
  }
  void* ptr = g_noalloc_ptr[dev].load(std::memory_order_acquire);
  QSX_CHECK_ARG(ptr != nullptr,
                "qsx_rk4_block_mean_noalloc: the first call on device %d was made inside a "
                "stream capture; make one call before capturing", dev);
  *out = ptr;
  return QSX_OK;
}

}  // namespace qsx

extern "C" int qsx_rk4_block_mean_noalloc(const qsx_rk4_args* a, void* stream) {
  int st = validate(a);
  if (st) return st;
  QSX_CHECK_ARG(a->block_k > 1 && a->out_mean != nullptr,
                "qsx_rk4_block_mean_noalloc: needs block_k > 1 and out_mean");
  if (a->batch == 0) return QSX_OK;
  Plan pl;
  st = make_plan(a, &pl);
  if (st) return st;
  const int64_t nsave = a->nsteps / a->save_every + 1;
  const int64_t per = nsave * a->nselect;  // outputs per accumulator slice
  const size_t slice = (size_t)per * sizeof(double2);
  QSX_CHECK_ARG(slice <= NOALLOC_SCRATCH_BYTES,
                "qsx_rk4_block_mean_noalloc: (nsteps + 1) * nselect = %lld outputs need %zu "
                "bytes of scratch per slice; the built-in scratch holds %zu bytes",
                (long long)per, slice, NOALLOC_SCRATCH_BYTES);
  // fewer persistent CTAs when their slices would not all fit
  const int64_t grid = std::max<int64_t>(
      1, std::min<int64_t>(pl.grid, (int64_t)(NOALLOC_SCRATCH_BYTES / slice)));
  cudaStream_t s = (cudaStream_t)stream;
  void* scratch = nullptr;
  st = noalloc_scratch(s, &scratch);
  if (st) return st;
  cudaError_t e = cudaMemsetAsync(scratch, 0, (size_t)grid * slice, s);
  if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_block_mean_noalloc: memset");
  Rk4P p;
  p.m = a->m;
  p.nsteps = a->nsteps;
  p.save_every = a->save_every;
  p.nsave = (int)nsave;
  p.nproj = 0;
  p.nselect = a->nselect;
  p.nout = a->nselect;
  p.form = a->form;
  p.batch = a->batch;
  p.matrix = a->matrix;
  p.matrix_stride = a->matrix_stride;
  p.h = a->h;
  p.y0 = (const double2*)a->y0;
  p.y0_stride = a->y0_stride;
  p.proj = nullptr;
  p.proj_stride = 0;
  p.select = a->select;
  p.out_state = nullptr;
  p.out_proj = (double2*)a->out_proj;
  p.partial = (double2*)scratch;
  p.partial32 = nullptr;
  p.status = a->status;
#define X(MM, GG, BB)                                                                    \
  if (a->m == MM) {                                                                      \
    if (pl.lpr == 3)                                                                     \
      rk4_block3_f32<MM, 2><<<(unsigned)grid, pl.threads, pl.smem, s>>>(p, pl.ngroups,     \
                                                                        pl.G, a->block_k); \
    else if (pl.lpr == 5)                                                                \
      rk4_block3_f32<MM, 4><<<(unsigned)grid, pl.threads, pl.smem, s>>>(p, pl.ngroups,     \
                                                                        pl.G, a->block_k); \
    else if (pl.lpr == 4)                                                                \
      rk4_block2_f32<MM, 4><<<(unsigned)grid, pl.threads, pl.smem, s>>>(p, pl.ngroups,    \
                                                                        pl.G, a->block_k); \
    else if (pl.lpr == 2)                                                                \
      rk4_block2_f32<MM, 2><<<(unsigned)grid, pl.threads, pl.smem, s>>>(p, pl.ngroups,    \
                                                                        pl.G, a->block_k); \
    else                                                                                 \
      rk4_block_f32<MM><<<(unsigned)grid, pl.threads, pl.smem, s>>>(p, pl.ngroups, pl.G,  \
                                                                    a->block_k);         \
  }
  QSX_ROWS_TABLE(X)
#undef X
  QSX_LAUNCH_CHECK("qsx_rk4_block_mean_noalloc");
  rk4_reduce_kernel<double2><<<(unsigned)((per + 31) / 32), 256, 0, s>>>(
      p.partial, grid, per, a->mean_scale, (double2*)a->out_mean);
  QSX_LAUNCH_CHECK("qsx_rk4_block_mean_noalloc reduce");
  return QSX_OK;
}

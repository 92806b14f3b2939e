// Real K-step blocked matrices on the 5th-generation tensor cores (tcgen05).
//
// Same output as block_matrix_real_kernel (qsx_rk4_block_matrix_real_batched):
// per sample, rows 0..m-1 = D_K = P^K - I and the selected rows R_k of
// D_k = P^k - I (k = 1..K-1), for the FP32 real (Hermitian) form, m <= 64.
//
// Phase j multiplies the stacked operand A = [D_{2^j} ; R_1..R_{2^j}] by
// B = D_{2^j} in one M = 128, N = NP, K = KP tcgen05.mma chain: the square
// and the row product share B.  D rows sit in A rows 0..31 and 64..95, R rows
// in 32..63 and 96..127, so that each of the four TMEM lane quarters (one per
// SM sub-partition) carries half square work and half row work.  FP32
// accuracy comes from 3xTF32: A = A_hi + A_lo, B = B_hi + B_lo (each rounded
// to TF32), A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi, 3 KP / 8 MMAs into one
// FP32 accumulator in tensor memory.  The epilogue (eight warps: lane quarter
// = warp % 4, column half = warp / 4; tcgen05.ld) forms
// D_{2^{j+1}} = 2 D + D D and R_{i + 2^j} = R_i + R_{2^j} + R_i D_{2^j}, and
// writes the next operands back to shared memory: rows as 16-byte stores, the
// transposed B through a 4 x 4 quad-shuffle transpose.  D_K for K = 2^J + 1
// is a final chain D_1 D_{2^J} (powers of P commute), for K = 2^J the last
// square.
//
// The kernel is persistent: each CTA loops over samples, keeps its tensor
// memory, barrier and zero padding, and prefetches the next sample's D with
// cp.async while the current one is in the product chain.  Two CTAs share an
// SM, so one CTA's epilogue overlaps the other's MMAs.
//
// Operand layout (SWIZZLE_NONE, K-major): 8-row x 16-byte core matrices,
// element (r, k) at (r / 8) * SBO + (k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4
// bytes (LBO = 128 bytes between K-adjacent core matrices, SBO = 32 KP bytes
// between row groups), so one K = 8 step is the descriptor start + 256.
// B is stored the same way with n as the row (B^T row-major).
//
// Every wait on the MMA completion barrier is bounded; on a timeout the CTA
// records QSX_ERR_CUDA in the status word, stops issuing work, waits once more
// (bounded) for its MMA chain, and still frees its tensor memory.
#include <stdint.h>

#include <algorithm>

#include "qsx_common.cuh"
#include "qsx_tc.cuh"

namespace qsx {

namespace tc {

// One sample's D (m x m contiguous floats in global memory) into the staging
// buffer: the enclosing 16-byte-aligned range keeps its alignment, so the
// sample starts at float offset (address % 16) / 4 of sd; the interior moves
// in 16-byte cp.async chunks, the ragged head and tail element by element.
// Returns that offset.
__device__ __forceinline__ int prefetch_sample(const float* d, float* sd, int mm, int tid,
                                               int nthreads) {
  const uintptr_t a = reinterpret_cast<uintptr_t>(d);
  const int shift = (int)((a & 15) >> 2);
  const int head = (4 - shift) & 3;                         // elements before the first chunk
  const int nchunk = mm > head ? (mm - head) >> 2 : 0;
  const int tail0 = head + 4 * nchunk;
  const uint32_t base = (uint32_t)__cvta_generic_to_shared(sd + shift);
  for (int c = tid; c < nchunk; c += nthreads) {
    const int e = head + 4 * c;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(base + 4u * e), "l"(d + e)
                 : "memory");
  }
  const int nedge = min(head, mm) + (mm - tail0 > 0 ? mm - tail0 : 0);
  for (int t = tid; t < nedge; t += nthreads) {
    const int e = t < min(head, mm) ? t : tail0 + (t - min(head, mm));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(base + 4u * e), "l"(d + e)
                 : "memory");
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
  return shift;
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// A row of the 64-row R region for R row index i (0..63)
__device__ __forceinline__ int r_arow(int i) { return 32 + i + (i >= 32 ? 32 : 0); }

}  // namespace tc

// CPT accumulator columns per thread: the CTA has 4 x (64 / CPT) warps, warp
// w reading TMEM lane quarter w % 4 and columns CPT * (w / 4) ...
// smem: A hi/lo (2 x 128 x KP TF32), B^T hi/lo (2 x NP x KP), the staging
// copy of the sample's D (m*m + 4 FP32, contiguous), the R rows
// ((K-1) nsel x SP FP32, SP = m | 1), the mbarrier and the tensor-memory
// address.
template <int CPT>
__global__ void __launch_bounds__(4 * (64 / CPT) * 32, 2)
    block_matrix_tc_kernel(const float* __restrict__ D, int m, int K, int J,
                           const int* __restrict__ sel, int nsel, float* __restrict__ out,
                           int* status, int64_t batch) {
  using namespace tc;
  constexpr int NT = 4 * (64 / CPT) * 32;
  constexpr int NW = NT / 32;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int kp = (m + 7) & ~7, np = (m + 15) & ~15, sp = m | 1;
  const uint32_t sbo = (uint32_t)kp * 32u;
  const uint32_t PA = ROWS * kp * 4, PB = np * kp * 4;
  unsigned char* a_hi = smraw;
  unsigned char* a_lo = a_hi + PA;
  unsigned char* b_hi = a_lo + PA;
  unsigned char* b_lo = b_hi + PB;
  const int mm = m * m;
  float* Sd = reinterpret_cast<float*>(b_lo + PB);   // [mm + 4], 16-byte aligned
  float* Rp = Sd + ((mm + 4 + 3) & ~3);               // [(K-1) nsel][sp]
  const int nr = nsel * (K - 1);
  const uint32_t off_mbar =
      (2 * PA + 2 * PB + (uint32_t)(((mm + 4 + 3) & ~3) + nr * sp) * 4 + 15) & ~15u;
  uint64_t* mbar_p = reinterpret_cast<uint64_t*>(smraw + off_mbar);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar_p + 1);
  float* stg = reinterpret_cast<float*>(a_lo);      // D_K staging once the chain is done
  __shared__ int s_abort;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int lg = warp & 3, c0 = CPT * (warp >> 2);
  const bool dwarp = (lg & 1) == 0;           // D rows; otherwise R rows
  const int r = 32 * (lg >> 1) + lane;        // D row, or R row index
  const int arow = 32 * lg + lane;            // this thread's A row = TMEM lane
  const int myq = r % nsel;
  int mysel = 0;
  if (!dwarp && r < nsel) {
    mysel = sel[r];
    mysel = (mysel >= 0 && mysel < m) ? mysel : 0;
  }
  const int rows_out = m + nr;
  const int64_t ostride = ((int64_t)rows_out * m + 3) & ~(int64_t)3;
  const uint32_t mbar = (uint32_t)__cvta_generic_to_shared(mbar_p);
  const uint64_t da_hi = smem_desc((uint32_t)__cvta_generic_to_shared(a_hi), sbo);
  const uint64_t da_lo = smem_desc((uint32_t)__cvta_generic_to_shared(a_lo), sbo);
  const uint64_t db_hi = smem_desc((uint32_t)__cvta_generic_to_shared(b_hi), sbo);
  const uint64_t db_lo = smem_desc((uint32_t)__cvta_generic_to_shared(b_lo), sbo);
  const uint32_t idesc = make_idesc(np);
  const int ksteps = kp / 8;
  const bool pow2 = (K & (K - 1)) == 0;

  // zero padding of the operand planes (kept zero across samples)
  for (uint32_t e = tid; e < (2 * PA + 2 * PB) / 16; e += NT)
    reinterpret_cast<uint4*>(smraw)[e] = make_uint4(0, 0, 0, 0);
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
  const uint32_t taddr = tmem + ((uint32_t)(32 * lg) << 16) + (uint32_t)c0;

  int64_t s = blockIdx.x;
  int shift = 0, next_shift = 0;
  if (s < batch) next_shift = prefetch_sample(D + s * mm, Sd, mm, tid, NT);
  uint32_t parity = 0;
  for (; s < batch; s += gridDim.x) {
    const int64_t next = s + gridDim.x;
    shift = next_shift;
    const float* sd = Sd + shift;   // this sample's D, row-major, stride m
    cp_async_wait_all();
    __syncthreads();
    float dr[CPT];   // this thread's part of D_{2^j} (D warps)
    if (dwarp) {
#pragma unroll
      for (int c = 0; c < CPT; ++c) dr[c] = (r < m && c0 + c < m) ? sd[r * m + c0 + c] : 0.f;
      store_row<CPT>(a_hi, a_lo, arow, c0, kp, sbo, dr);
      store_cols<CPT>(b_hi, b_lo, r, c0, np, kp, sbo, dr, lane);
    } else if (r < nsel) {
      float v[CPT];
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        v[c] = c0 + c < m ? sd[mysel * m + c0 + c] : 0.f;
        if (c0 + c < m) Rp[r * sp + c0 + c] = v[c];
      }
      store_row<CPT>(a_hi, a_lo, arow, c0, kp, sbo, v);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (pow2 && next < batch) next_shift = prefetch_sample(D + next * mm, Sd, mm, tid, NT);

    int have = 1;
    for (int j = 0;; ++j) {
      const bool square = j < J;
      const int add = have < K - 1 ? min(1 << j, K - 1 - have) : 0;
      const bool last = !(j + 1 < J || have + add < K - 1);
      if (tid == 0) {
        issue_product(tmem, da_hi, da_lo, db_hi, db_lo, ksteps, idesc, mbar);
        if (!wait_parity(mbar, parity)) {
          if (status) atomicOr(status, QSX_ERR_CUDA);
          s_abort = 1;
        }
      }
      __syncthreads();  // the other threads wait here, off the issue slots
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (s_abort) break;
      parity ^= 1;
      float acc[CPT];
      tmem_load(taddr, acc);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      if (dwarp) {
        if (square) {
#pragma unroll
          for (int c = 0; c < CPT; ++c)
            dr[c] = (r < m && c0 + c < m) ? (dr[c] + dr[c]) + acc[c] : 0.f;
          if (!last) {
            store_row<CPT>(a_hi, a_lo, arow, c0, kp, sbo, dr);
            store_cols<CPT>(b_hi, b_lo, r, c0, np, kp, sbo, dr, lane);
          } else if (!pow2) {
            // operands of the final chain D_1 D_{2^J}; dr becomes D_{2^J} + D_1
            float d1[CPT];
#pragma unroll
            for (int c = 0; c < CPT; ++c) d1[c] = (r < m && c0 + c < m) ? sd[r * m + c0 + c] : 0.f;
            store_row<CPT>(a_hi, a_lo, arow, c0, kp, sbo, d1);
            store_cols<CPT>(b_hi, b_lo, r, c0, np, kp, sbo, dr, lane);
#pragma unroll
            for (int c = 0; c < CPT; ++c) dr[c] += d1[c];
          }
        }
      } else if (r < add * nsel) {
        const int dst = have * nsel + r;                   // new row R_{have + 1 + r / nsel}
        const int rb = ((1 << j) - 1) * nsel + myq;        // row of D_{2^j}
        float v[CPT];
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
          const int cc = c0 + c;
          v[c] = cc < m ? (Rp[r * sp + cc] + Rp[rb * sp + cc]) + acc[c] : 0.f;
          if (cc < m) Rp[dst * sp + cc] = v[c];
        }
        if (!last && dst < 64) store_row<CPT>(a_hi, a_lo, r_arow(dst), c0, kp, sbo, v);
      }
      have += add;
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (last) break;
    }
    if (s_abort) break;
    if (!pow2) {
      if (next < batch) next_shift = prefetch_sample(D + next * mm, Sd, mm, tid, NT);
      if (tid == 0) {
        issue_product(tmem, da_hi, da_lo, db_hi, db_lo, ksteps, idesc, mbar);
        if (!wait_parity(mbar, parity)) {
          if (status) atomicOr(status, QSX_ERR_CUDA);
          s_abort = 1;
        }
      }
      __syncthreads();  // the other threads wait here, off the issue slots
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (s_abort) break;
      parity ^= 1;
      float acc[CPT];
      tmem_load(taddr, acc);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
#pragma unroll
      for (int c = 0; c < CPT; ++c) dr[c] += acc[c];
    }
    if (dwarp && r < m) {
#pragma unroll
      for (int c = 0; c < CPT; ++c)
        if (c0 + c < m) stg[r * sp + c0 + c] = dr[c];
    }
    __syncthreads();
    float* o = out + s * ostride;
#pragma unroll 4
    for (int row = warp; row < rows_out; row += NW) {
      const float* src = row < m ? stg + row * sp : Rp + (row - m) * sp;
      const float v0 = lane < m ? src[lane] : 0.f;
      const float v1 = lane + 32 < m ? src[lane + 32] : 0.f;
      if (lane < m) o[row * m + lane] = v0;
      if (lane + 32 < m) o[row * m + lane + 32] = v1;
    }
    // the next iteration's first barrier orders these reads before new writes
  }
  cp_async_wait_all();
  if (s_abort && tid == 0) wait_parity(mbar, parity);  // let an unfinished chain drain
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
}

}  // namespace qsx

using namespace qsx;

// Shapes the tensor-core form handles: m <= 64, K = 2^J or 2^J + 1, and at
// most 64 selected rows entering a product.
extern "C" int qsx_rk4_block_matrix_real_tc_supported(int m, int K, int nselect) {
  if (m < 1 || m > 64 || K < 2 || K > 64 || nselect < 1 || nselect > m) return 0;
  const bool pow2 = (K & (K - 1)) == 0, pow2p1 = ((K - 1) & (K - 2)) == 0 && K > 2;
  if (!pow2 && !pow2p1) return 0;
  // the last doubling multiplies R_1..R_b, b the largest power of two < K - 1
  int b = 1;
  while (2 * b < K - 1) b *= 2;
  return b * nselect <= 64 ? 1 : 0;
}

#ifndef QSX_TC_CPT
#define QSX_TC_CPT 32
#endif

extern "C" int qsx_rk4_block_matrix_real_tc(const float* D, int m, int64_t batch, int K,
                                            const int* select, int nselect, float* out,
                                            int32_t* status, void* stream) {
  QSX_CHECK_ARG(batch >= 0 && batch <= 0x7fffffff, "qsx_rk4_block_matrix_real_tc: bad batch");
  if (!qsx_rk4_block_matrix_real_tc_supported(m, K, nselect)) {
    set_error("qsx_rk4_block_matrix_real_tc: shape m=%d K=%d nselect=%d not supported", m, K,
              nselect);
    return QSX_ERR_UNSUPPORTED;
  }
  if (batch == 0) return QSX_OK;
  QSX_CHECK_ARG(D && select && out, "qsx_rk4_block_matrix_real_tc: null pointer");
  QSX_CHECK_ARG((reinterpret_cast<uintptr_t>(D) & 3) == 0,
                "qsx_rk4_block_matrix_real_tc: D must be 4-byte aligned");
  constexpr int CPT = QSX_TC_CPT;
  constexpr int NT = 4 * (64 / CPT) * 32;
  int J = 0;
  while ((2 << J) <= K) ++J;
  const int kp = (m + 7) & ~7, np = (m + 15) & ~15, sp = m | 1;
  const int nr = nselect * (K - 1);
  // byte layout as in the kernel: planes, staging, R rows, then the 16-byte
  // aligned mbarrier and tensor-memory address
  const size_t smem = ((2 * (size_t)tc::ROWS * kp * 4 + 2 * (size_t)np * kp * 4 +
                        ((((size_t)m * m + 4 + 3) & ~(size_t)3) + (size_t)nr * sp) * 4 + 15) &
                       ~(size_t)15) + 16;
  auto kern = block_matrix_tc_kernel<CPT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  int dev = 0, sms = 0, per_sm = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
  if (e != cudaSuccess) return cuda_status(e, "qsx_rk4_block_matrix_real_tc");
  // Two resident CTAs per SM overlap one CTA's epilogue with the other's MMA
  // chain; the occupancy query can report fewer than fit, and a second wave
  // is harmless because every CTA strides over the samples on its own.
  const int64_t grid = std::min<int64_t>(batch, (int64_t)std::max(per_sm, 2) * sms);
  kern<<<(unsigned)grid, NT, smem, (cudaStream_t)stream>>>(D, m, K, J, select, nselect, out,
                                                            status, batch);
  QSX_LAUNCH_CHECK("qsx_rk4_block_matrix_real_tc");
  return QSX_OK;
}

// tcgen05 (5th-generation tensor core) helpers shared by the FP32 kernels that
// run 3xTF32 products: operand layout in shared memory, descriptors, the
// hi/lo TF32 split, MMA issue and commit, bounded barrier waits and tensor-
// memory loads.  M = 128 accumulator rows, one row per TMEM lane; operands
// K-major without swizzle: 8-row x 16-byte core matrices, element (r, k) at
// (r / 8) * SBO + (k / 4) * 128 + (r % 8) * 16 + (k % 4) * 4 bytes, SBO =
// 32 KP bytes for KP (a multiple of 8) K columns, so one K = 8 step is the
// descriptor start + 256 bytes.
#pragma once
#include <stdint.h>

namespace qsx {

namespace tc {

constexpr int ROWS = 128;       // accumulator rows (M)
constexpr uint32_t LBO = 128;
constexpr uint32_t TMEM_COLS = 64;
constexpr long long WAIT_LIMIT = 1ll << 26;

__device__ __forceinline__ uint32_t op_offset(int r, int k, uint32_t sbo) {
  return (uint32_t)(r >> 3) * sbo + (uint32_t)(k >> 2) * LBO + (uint32_t)((r & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(LBO >> 4) << 16;
  d |= (uint64_t)(sbo >> 4) << 32;
  d |= 1ull << 46;  // descriptor version for tcgen05; no swizzle, base offset 0
  return d;
}

// kind::tf32, D = F32, A = B = TF32, both K-major, N = np, M = 128
__device__ __forceinline__ uint32_t make_idesc(int np) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(np >> 3) << 17) |
         ((uint32_t)(ROWS >> 4) << 24);
}

// Round to the nearest TF32 value (10-bit mantissa), ties away from zero on
// the magnitude: add half a unit of the 13 dropped bits, then clear them.
// Integer ops only, so the split stays on the full-rate pipes.
__device__ __forceinline__ float tf32_round(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// hi / lo TF32 split of four consecutive-k values into the two planes
__device__ __forceinline__ void st_split4(unsigned char* hi, unsigned char* lo, uint32_t off,
                                          float a, float b, float c, float d) {
  const float4 h = make_float4(tf32_round(a), tf32_round(b), tf32_round(c), tf32_round(d));
  const float4 l = make_float4(tf32_round(a - h.x), tf32_round(b - h.y), tf32_round(c - h.z),
                               tf32_round(d - h.w));
  *reinterpret_cast<float4*>(hi + off) = h;
  *reinterpret_cast<float4*>(lo + off) = l;
}

// Operand row `arow` (K-major) from this thread's CPT values at columns
// c0..c0+CPT-1; columns at or above m must already be zero.
template <int CPT>
__device__ __forceinline__ void store_row(unsigned char* hi, unsigned char* lo, int arow, int c0,
                                          int kp, uint32_t sbo, const float (&v)[CPT]) {
#pragma unroll
  for (int g = 0; g < CPT / 4; ++g)
    if (c0 + 4 * g < kp)
      st_split4(hi, lo, op_offset(arow, c0 + 4 * g, sbo), v[4 * g], v[4 * g + 1], v[4 * g + 2],
                v[4 * g + 3]);
}

// Transposed operand: this thread holds row k = r of X (columns
// c0..c0+CPT-1); B^T row n = column n of X.  Lanes 4q..4q+3 (rows r & ~3 ..
// +3) transpose 4 x 4 blocks with two xor-shuffle rounds, then each lane
// writes 16 bytes (four consecutive k) of one B^T row.  Odd quads take the
// blocks in swapped pairs so that one store instruction covers all 32 banks.
template <int CPT>
__device__ __forceinline__ void store_cols(unsigned char* hi, unsigned char* lo, int r, int c0,
                                           int np, int kp, uint32_t sbo, const float (&v)[CPT],
                                           int lane) {
  const bool odd = (lane >> 2) & 1, b1 = lane & 1, b2 = (lane >> 1) & 1;
  const int kq = r & ~3;
#pragma unroll
  for (int jj = 0; jj < CPT / 4; ++jj) {
    float a0 = odd ? v[4 * (jj ^ 1)] : v[4 * jj];
    float a1 = odd ? v[4 * (jj ^ 1) + 1] : v[4 * jj + 1];
    float a2 = odd ? v[4 * (jj ^ 1) + 2] : v[4 * jj + 2];
    float a3 = odd ? v[4 * (jj ^ 1) + 3] : v[4 * jj + 3];
    {
      const float s0 = b2 ? a0 : a2, s1 = b2 ? a1 : a3;
      const float q0 = __shfl_xor_sync(0xffffffffu, s0, 2);
      const float q1 = __shfl_xor_sync(0xffffffffu, s1, 2);
      if (b2) { a0 = q0; a1 = q1; } else { a2 = q0; a3 = q1; }
    }
    {
      const float s0 = b1 ? a0 : a1, s1 = b1 ? a2 : a3;
      const float q0 = __shfl_xor_sync(0xffffffffu, s0, 1);
      const float q1 = __shfl_xor_sync(0xffffffffu, s1, 1);
      if (b1) { a0 = q0; a2 = q1; } else { a1 = q0; a3 = q1; }
    }
    const int n = c0 + 4 * (jj ^ (int)odd) + (lane & 3);
    if (n < np && kq < kp) st_split4(hi, lo, op_offset(n, kq, sbo), a0, a1, a2, a3);
  }
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      :
      : "r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// One 3xTF32 product chain into the accumulator, issued by one thread, then
// committed to the mbarrier; the chain adds to the accumulator when
// `accumulate` is set, else its first MMA overwrites it.  The descriptors' start-address field counts
// 16-byte units, so one K = 8 step (256 bytes) adds 16; the planes lie below
// 256 KB and the 14-bit field does not carry.
__device__ __forceinline__ void issue_product(uint32_t dtmem, uint64_t a_hi, uint64_t a_lo,
                                              uint64_t b_hi, uint64_t b_lo, int ksteps,
                                              uint32_t idesc, uint32_t mbar,
                                              uint32_t accumulate = 0) {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
  for (int s = 0; s < ksteps; ++s) {
    const uint64_t step = 16ull * (uint64_t)s;
    mma_tf32(dtmem, a_hi + step, b_hi + step, idesc, (s > 0 || accumulate) ? 1u : 0u);
    mma_tf32(dtmem, a_hi + step, b_lo + step, idesc, 1);
    mma_tf32(dtmem, a_lo + step, b_hi + step, idesc, 1);
  }
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               :
               : "r"(mbar)
               : "memory");
}

// bounded wait for the barrier phase with the given parity; false on timeout
__device__ __forceinline__ bool wait_parity(uint32_t mbar, uint32_t parity) {
  for (long long it = 0; it < WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// CPT consecutive accumulator columns of this thread's lane (16 or 32)
__device__ __forceinline__ void tmem_load(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_load(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive accumulator columns of this thread's lane from registers
__device__ __forceinline__ void tmem_store(uint32_t taddr, const float (&v)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
      "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};\n\t"
      "tcgen05.wait::st.sync.aligned;"
      :
      : "r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])),
        "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])),
        "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
        "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])),
        "r"(__float_as_uint(v[11])), "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])),
        "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15]))
      : "memory");
}

}  // namespace tc

}  // namespace qsx

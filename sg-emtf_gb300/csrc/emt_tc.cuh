// emt_tc.cuh -- Blackwell tensor-core primitives for the rotation GEMM:
// tcgen05 MMA (kind::tf32) with the accumulator in tensor memory, shared
// memory matrix descriptors for 128-byte-swizzled K-major operands, TMA tile
// loads, and mbarrier waits that give up after a time limit.
//
// Operand layout (both operands K-major, 128B swizzle): a tile holds R rows
// of 32 FP32 values (128 bytes); rows are grouped by 8 into 1024-byte atoms
// (stride byte offset 1024) and inside an atom the 16-byte chunk index of
// row r is XORed with r mod 8.  A K-step of 8 TF32 values is 32 bytes, so
// the descriptor of step ks starts 32*ks bytes into the tile; the swizzle is
// a function of the address bits, which is how TMA writes the same tiles.
#pragma once

#include <cstdint>

namespace emt {
namespace tc {

// Instruction descriptor, kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32
// (bits 7-9 = 2, bits 10-12 = 2), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Instruction descriptor, kind::f16 with BF16 operands: D = F32 (bits 4-5 =
// 1), A = B = BF16 (bits 7-9 = 1, bits 10-12 = 1), both K-major, N >> 3 in
// bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading
// byte offset (unused for swizzled K-major, 16 B), stride byte offset 1024 B
// (bits 32-45), descriptor version 1 (bits 46-47), swizzle mode 128B = 2
// (bits 61-63).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Byte offset of element (row, c) (c < 32) inside a 128B-swizzled tile.
__host__ __device__ __forceinline__ uint32_t sw128_offset(int row, int c) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((((c >> 2) ^ (row & 7)) & 7) << 4) +
                    ((c & 3) << 2));
}

// Byte offset of 16-bit element (row, c) (c < 64) inside a 128B-swizzled tile.
__host__ __device__ __forceinline__ uint32_t sw128_offset_b16(int row, int c) {
  return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((((c >> 3) ^ (row & 7)) & 7) << 4) +
                    ((c & 7) << 1));
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// D (+)= A B^T with BF16 operands (K = 16 per instruction), FP32 accumulator.
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Exact split of two FP32 values into three BF16 parts each, packed in pairs
// (element a in the low half, b in the high half): a = a0 + a1 + a2 exactly
// for normal FP32 a (each part is the round-to-nearest BF16 of what the
// previous parts leave; 8 + 8 + 8 significand bits cover FP32's 24).
__device__ __forceinline__ float bf16_lo_as_f32(uint32_t p) { return __uint_as_float(p << 16); }
__device__ __forceinline__ float bf16_hi_as_f32(uint32_t p) { return __uint_as_float(p & 0xFFFF0000u); }
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(b), "f"(a));
  return r;
}
__device__ __forceinline__ void split3_bf16x2(float a, float b, uint32_t& p0, uint32_t& p1,
                                              uint32_t& p2) {
  p0 = pack_bf16x2(a, b);
  const float ra = __fsub_rn(a, bf16_lo_as_f32(p0)), rb = __fsub_rn(b, bf16_hi_as_f32(p0));
  p1 = pack_bf16x2(ra, rb);
  p2 = pack_bf16x2(__fsub_rn(ra, bf16_lo_as_f32(p1)), __fsub_rn(rb, bf16_hi_as_f32(p1)));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;"); }

// Whole warp: allocate ncols (power of two >= 32) TMEM columns; the base
// address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_addr(slot)),
               "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

// 32 lanes x 16 consecutive FP32 columns: thread l of the warp gets lane
// (taddr lane + l), columns [col, col + 16).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%"
      "15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Default limit of a bounded wait: 2 s of %globaltimer.
constexpr uint64_t kWaitLimitNs = 2000000000ull;

// Waits for phase `parity` of the barrier; gives up after limit_ns and
// returns false, so a lost completion can never hang the GPU.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
                                          uint64_t limit_ns = kWaitLimitNs) {
  const uint64_t t0 = globaltimer();
  for (uint32_t it = 0;; ++it) {
    uint32_t ok;
    asm volatile(
        "{.reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0,1,0,p;}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((it & 63) == 63 && globaltimer() - t0 > limit_ns) return false;
  }
}

// TMA: 3-D tile of the tensor map into shared memory, completion counted on bar.
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const void* tmap, int x, int y, int z,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

}  // namespace tc
}  // namespace emt

// Thin inline-PTX wrappers for the Blackwell (sm_100-family) tensor-core
// path used by the guide network: TMEM allocation, UMMA shared-memory and
// instruction descriptors, tcgen05.mma issue and commit, TMEM loads, and
// mbarrier waits with an iteration limit.
//
// Operand tiles live in shared memory in the canonical K-major layout with
// 128-byte swizzle: rows of 64 bf16 (128 B), 8-row groups of 1024 B, the
// 16-byte chunk c of row r stored at chunk c ^ (r & 7).  Tiles start on a
// 1024-byte boundary.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lisa {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (row, k) in a K-major SW128 bf16 tile (k < 64)
__device__ __forceinline__ uint32_t sw128_offset(uint32_t row, uint32_t k) {
  const uint32_t chunk = (k >> 3) ^ (row & 7u);
  return row * 128u + chunk * 16u + (k & 7u) * 2u;
}

// UMMA shared-memory descriptor, K-major, 128-byte swizzle: start address,
// leading byte offset (unused for swizzled K-major; 16 B), stride byte
// offset 1024 B (8 rows x 128 B), descriptor version 1, layout SWIZZLE_128B.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// UMMA shared-memory descriptor, MN-major, 128-byte swizzle: the same tile
// image read the other way round.  Each 128-byte row holds 64 consecutive
// M (or N) elements of one K index; 8 rows (8 K indices) form a 1024-byte
// swizzle atom, so the stride byte offset (between 8-row K groups) is
// 1024 B and the leading byte offset is the stride between 64-element
// blocks along M (or N).  One K = 16 step spans two atoms (2048 B).
__device__ __forceinline__ uint64_t sw128_mn_desc(uint32_t saddr, uint32_t mn_block_stride) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((mn_block_stride & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B (both K-major) and
// an FP32 accumulator, shape M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t M, uint32_t N) {
  return (1u << 4)            // D format F32
         | (1u << 7)          // A format BF16
         | (1u << 10)         // B format BF16
         | ((N >> 3) << 17)   // N / 8
         | ((M >> 4) << 24);  // M / 16
}

// The same with A and B both MN-major (transpose bits 15 and 16).
__host__ __device__ constexpr uint32_t idesc_bf16_f32_mn(uint32_t M, uint32_t N) {
  return idesc_bf16_f32(M, N) | (1u << 15) | (1u << 16);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}

// Arrive on the mbarrier once every MMA this thread issued has completed.
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase with the given parity to complete, giving up after
// `limit` polls.  Returns false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t limit = (1u << 26)) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(mbar, parity)) return true;
  return false;
}

// TMEM allocation by one full warp; the base address is written to *dst.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Bulk copy (TMA, untiled) of `bytes` from global to shared memory,
// completing on `mbar` (transaction count).  Both addresses 16-byte aligned,
// bytes a multiple of 16.  Issued by one thread after mbar_expect_tx.
__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gmem_src, uint32_t bytes, uint64_t* mbar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(smem_dst)),
               "l"(gmem_src), "r"(bytes), "r"(smem_u32(mbar))
               : "memory");
}

// Arrive once on mbar and add `bytes` to its expected transaction count.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes) : "memory");
}

// Makes an mbarrier's initialisation visible to the async proxy (TMA).
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Copies `bytes` (a multiple of 16) from global to shared memory with bulk
// copies of at most 16 KB, all completing on `mbar`, issued by the calling
// thread; the caller waits for phase 0 of mbar (initialised with count 1).
__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gmem_src, uint32_t bytes, uint64_t* mbar) {
  mbar_expect_tx(mbar, bytes);
  for (uint32_t off = 0; off < bytes; off += 16384u) {
    const uint32_t n = bytes - off < 16384u ? bytes - off : 16384u;
    bulk_g2s((uint8_t*)smem_dst + off, (const uint8_t*)gmem_src + off, n, mbar);
  }
}

// CH x 16 consecutive FP32 columns of this thread's TMEM lane: all loads
// issued, then one wait.
template <int CH>
__device__ __forceinline__ void tmem_ld16x(uint32_t taddr, float* v) {
  uint32_t r[CH][16];
#pragma unroll
  for (int c = 0; c < CH; ++c)
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[c][0]), "=r"(r[c][1]), "=r"(r[c][2]), "=r"(r[c][3]), "=r"(r[c][4]), "=r"(r[c][5]), "=r"(r[c][6]),
          "=r"(r[c][7]), "=r"(r[c][8]), "=r"(r[c][9]), "=r"(r[c][10]), "=r"(r[c][11]), "=r"(r[c][12]),
          "=r"(r[c][13]), "=r"(r[c][14]), "=r"(r[c][15])
        : "r"(taddr + 16u * c));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  // The loaded registers may be read only after the wait: an empty volatile
  // statement that "modifies" them keeps every use below it.
#pragma unroll
  for (int c = 0; c < CH; ++c)
    asm volatile(""
                 : "+r"(r[c][0]), "+r"(r[c][1]), "+r"(r[c][2]), "+r"(r[c][3]), "+r"(r[c][4]), "+r"(r[c][5]),
                   "+r"(r[c][6]), "+r"(r[c][7]), "+r"(r[c][8]), "+r"(r[c][9]), "+r"(r[c][10]), "+r"(r[c][11]),
                   "+r"(r[c][12]), "+r"(r[c][13]), "+r"(r[c][14]), "+r"(r[c][15]));
#pragma unroll
  for (int c = 0; c < CH; ++c)
#pragma unroll
    for (int i = 0; i < 16; ++i) v[16 * c + i] = __uint_as_float(r[c][i]);
}

}  // namespace tc
}  // namespace lisa

// Fifth-generation tensor core (tcgen05) primitives for sm_100-family GPUs,
// as inline PTX: tensor-memory allocation, shared-memory matrix and
// instruction descriptors, the BF16 MMA with an FP32 accumulator in tensor
// memory, commit to an mbarrier, bounded mbarrier waits and tensor-memory
// loads.
//
// Operands live in shared memory in the canonical K-major layout without
// swizzling: 8 x 16-byte "core matrices" (8 rows x 8 BF16); core matrices
// adjacent along K are kLbo = 128 bytes apart, groups of 8 rows are
// (K / 8) * 128 bytes apart.  smem_offset() gives the byte offset of
// element (row, k) of such a tile.  D = A . B^T with A [M = 128][K] and
// B [N][K] both K-major; D row r lives in tensor-memory lane r, column j in
// the allocation's column base + j (FP32).
#pragma once

#include <stdint.h>

namespace pg {
namespace tc {

constexpr uint32_t kLbo = 128;

// byte offset of element (row, k) in a K-major tile with `k_dim` columns
__device__ __forceinline__ uint32_t smem_offset(uint32_t row, uint32_t k, uint32_t k_dim) {
  return (row >> 3) * (k_dim / 8) * 128 + (k >> 3) * kLbo + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: start address, leading (K) and stride
// (8-row group) byte offsets, version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t k_dim) {
  const uint64_t sbo = (uint64_t)(k_dim / 8) * 128;
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3ffffu) >> 4);
  d |= (uint64_t)(kLbo >> 4) << 16;
  d |= (sbo >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor: BF16 x BF16 -> F32, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

// D[tmem] (+)= A . B^T over one K = 16 slice; issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// arrive on the mbarrier once every earlier tcgen05 operation of this
// thread has completed
__device__ __forceinline__ void commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          mbar)
      : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count) : "memory");
}

// Waits for the phase with parity `phase` to complete, at most `limit`
// polls; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) {
      return true;
    }
  }
  return false;
}

// arrive on the mbarrier and expect `bytes` of asynchronous copies to
// complete on it in this phase
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar),
               "r"(bytes)
               : "memory");
}

// bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to this CTA's shared memory, completing on the mbarrier
__device__ __forceinline__ void bulk_g2s(uint32_t dst_smem, const void *src, uint32_t bytes,
                                         uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
      "[%3];\n" ::"r"(dst_smem),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

// barrier `id` (1..15) over `count` threads (a multiple of 32), returning
// whether `pred` held in every one of them
__device__ __forceinline__ bool bar_and(uint32_t id, uint32_t count, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %1, 0;\n\t"
      "bar.red.and.pred p, %2, %3, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(r)
      : "r"(pred ? 1u : 0u), "r"(id), "r"(count)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void bar_sync(uint32_t id, uint32_t count) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(count) : "memory");
}

// tensor-memory allocation of ncols columns (a power of two >= 32) by one
// whole warp; the base address is written to *dst (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                   dst_smem),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr),
               "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}

// make generic-proxy shared-memory writes visible to the tensor core
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// 16 consecutive FP32 columns of this thread's lane (warp w of a warpgroup
// reads lanes 32 (w % 4) ... 32 (w % 4) + 31)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    v[i] = __uint_as_float(r[i]);
  }
}

} // namespace tc
} // namespace pg

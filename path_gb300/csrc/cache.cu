// Neural radiance cache: hash-grid encoding and a BF16 MLP on the fifth-
// generation tensor cores (tcgen05, accumulators in tensor memory).
//
// This file holds the tensor-core building block (one 128-row tile of
// D = A . B^T, the operands staged in shared memory in the canonical
// K-major layout of tc.cuh) and its self-test entry point.
#include "kernels.h"
#include "tc.cuh"

#include <cuda_bf16.h>

namespace pg {
namespace dev {

constexpr uint32_t kTcWaitLimit = 1u << 24; // polls before a wait gives up

// D [128][n] = A [128][k] . B [n][k]^T, BF16 in, FP32 out, one CTA of 128
// threads.  err: set to 1 when the tensor core did not signal completion.
__global__ void __launch_bounds__(128) k_tc_gemm(const __nv_bfloat16 *a,
                                                 const __nv_bfloat16 *b, float *d,
                                                 uint32_t k_dim, uint32_t n_dim,
                                                 uint32_t *err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const uint32_t tid = threadIdx.x;
  unsigned char *sa = smem;
  unsigned char *sb = smem + 128 * k_dim * 2;
  // stage A and B in the canonical layout
  for (uint32_t i = tid; i < 128 * k_dim; i += 128) {
    const uint32_t r = i / k_dim, c = i % k_dim;
    *reinterpret_cast<__nv_bfloat16 *>(sa + tc::smem_offset(r, c, k_dim)) = a[i];
  }
  for (uint32_t i = tid; i < n_dim * k_dim; i += 128) {
    const uint32_t r = i / k_dim, c = i % k_dim;
    *reinterpret_cast<__nv_bfloat16 *>(sb + tc::smem_offset(r, c, k_dim)) = b[i];
  }
  uint32_t ncols = 32;
  while (ncols < n_dim) {
    ncols <<= 1;
  }
  if (tid < 32) {
    tc::tmem_alloc(tc::smem_addr(&tmem_base), ncols);
  }
  if (tid == 0) {
    tc::mbar_init(tc::smem_addr(&mbar), 1);
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16(128, n_dim);
    for (uint32_t k0 = 0; k0 < k_dim; k0 += 16) {
      const uint64_t ad = tc::smem_desc(tc::smem_addr(sa) + k0 * 16, k_dim);
      const uint64_t bd = tc::smem_desc(tc::smem_addr(sb) + k0 * 16, k_dim);
      tc::mma_bf16(tmem, ad, bd, idesc, k0 > 0 ? 1u : 0u);
    }
    tc::commit(tc::smem_addr(&mbar));
  }
  const bool ok = tc::mbar_wait(tc::smem_addr(&mbar), 0, kTcWaitLimit);
  tc::fence_after_sync();
  if (!ok) {
    if (tid == 0) {
      atomicExch(err, 1u);
    }
  } else {
    const uint32_t warp = tid / 32;
    const uint32_t row = tid;
    for (uint32_t c0 = 0; c0 < n_dim; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((warp * 32) << 16) + c0, v);
      for (int j = 0; j < 16; ++j) {
        d[(size_t)row * n_dim + c0 + j] = v[j];
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) {
    tc::tmem_dealloc(tmem, ncols);
  }
}

} // namespace dev

cudaError_t launch_tc_gemm(const void *a, const void *b, float *d, uint32_t k_dim,
                           uint32_t n_dim, uint32_t *err, cudaStream_t s) {
  const size_t smem = (size_t)(128 + n_dim) * k_dim * 2;
  cudaError_t e = cudaFuncSetAttribute(dev::k_tc_gemm,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    return e;
  }
  dev::k_tc_gemm<<<1, 128, smem, s>>>(static_cast<const __nv_bfloat16 *>(a),
                                      static_cast<const __nv_bfloat16 *>(b), d, k_dim, n_dim,
                                      err);
  return cudaGetLastError();
}

} // namespace pg

// Sobol points of the render path's RNG.
//
// The reference fills a [count][dimension_bound] table with cuRAND's
// scrambled Sobol generator, one curand_init + curand_uniform per value
// (src/rng/sobel/sobel.cu:21-93), and maps 1.0 to 0.0
// (include/lib/cuda/curand_utils.h:58-66).  Here each value is produced
// directly: the Gray-code ordered point x = c_d XOR (XOR of the direction
// vectors v_{d,j} for the set bits j of g = i ^ (i >> 1)) is accumulated in
// a register and mapped to (0, 1] as (x + 1/2) 2^-32, i.e. the centre of the
// x-th of 2^32 equal cells, rounded to float.  The direction vectors and
// scramble constants are the JoeKuo6 tables obtained at run time from
// cuRAND's host API (curandGetDirectionVectors32 / curandGetScrambleConstants32),
// exactly as the reference obtains them.  k_sobol_curand runs cuRAND's own
// device generator on the same tables so the two can be compared bit for bit.
#include "kernels.h"

#include <curand_kernel.h>

namespace pg {
namespace dev {

__global__ void k_sobol(const uint32_t *__restrict__ dirs,
                        const uint32_t *__restrict__ scramble, uint32_t dim_bound,
                        uint32_t count, float *__restrict__ out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)dim_bound * count) {
    return;
  }
  const uint32_t d = (uint32_t)(i % dim_bound);
  const uint32_t offset = (uint32_t)(i / dim_bound);
  uint32_t g = offset ^ (offset >> 1);
  uint32_t x = __ldg(scramble + d);
  const uint32_t *v = dirs + 32 * (size_t)d;
  while (g != 0) {
    const int j = __ffs(g) - 1;
    x ^= __ldg(v + j);
    g &= g - 1;
  }
  const float f = __fadd_rn(__fmul_rn(__uint2float_rn(x), 0x1p-32f), 0x1p-33f);
  out[i] = f == 1.0f ? 0.0f : f;
}

__global__ void k_sobol_curand(const uint32_t *dirs, const uint32_t *scramble,
                               uint32_t dim_bound, uint32_t count, float *out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)dim_bound * count) {
    return;
  }
  const uint32_t d = (uint32_t)(i % dim_bound);
  const uint32_t offset = (uint32_t)(i / dim_bound);
  curandStateScrambledSobol32_t state;
  curand_init(const_cast<uint32_t *>(dirs + 32 * (size_t)d), scramble[d], offset,
              &state);
  const float f = curand_uniform(&state);
  out[i] = f == 1.0f ? 0.0f : f;
}

} // namespace dev

cudaError_t launch_sobol_table(const uint32_t *dirs, const uint32_t *scramble,
                               uint32_t dimension_bound, uint32_t count,
                               float *out, cudaStream_t s) {
  const size_t n = (size_t)dimension_bound * count;
  if (n == 0) {
    return cudaSuccess;
  }
  const uint32_t bs = 256;
  dev::k_sobol<<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(dirs, scramble,
                                                            dimension_bound, count, out);
  return cudaGetLastError();
}

cudaError_t launch_sobol_curand(const uint32_t *dirs, const uint32_t *scramble,
                                uint32_t dimension_bound, uint32_t count,
                                float *out, cudaStream_t s) {
  const size_t n = (size_t)dimension_bound * count;
  if (n == 0) {
    return cudaSuccess;
  }
  const uint32_t bs = 256;
  dev::k_sobol_curand<<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(
      dirs, scramble, dimension_bound, count, out);
  return cudaGetLastError();
}

} // namespace pg

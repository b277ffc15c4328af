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

// Cost of the render's Sobol draws two ways, for the measurement behind
// the table design: every thread walks one path's draws -- sample index
// p mod spp, first dimension fnv(p / spp) mod 64 as a pixel's, then `draws`
// consecutive dimensions -- and sums them.  kMode 0 reads each value from
// the [spp][dim_bound] table (what the integrator does); kMode 1 forms each
// value from the direction vectors, XOR-ed in a register for the set bits
// of the Gray code of the sample index (k_sobol's arithmetic), with the
// vectors and scramble constants read through L1; kMode 2 the same with
// them staged in shared memory.  All three give the same sums bit for bit.
template <int kMode>
__global__ void __launch_bounds__(256) k_sobol_draws(const float *__restrict__ table,
                                                     const uint32_t *__restrict__ dirs,
                                                     const uint32_t *__restrict__ scramble,
                                                     uint32_t dim_bound, uint32_t spp,
                                                     uint32_t n_paths, uint32_t draws,
                                                     float *__restrict__ out) {
  extern __shared__ uint32_t s_vec[]; // kMode 2: [dim_bound][32] + [dim_bound]
  if constexpr (kMode == 2) {
    for (uint32_t i = threadIdx.x; i < dim_bound * 33; i += blockDim.x) {
      s_vec[i] = i < dim_bound * 32 ? dirs[i] : scramble[i - dim_bound * 32];
    }
    __syncthreads();
  }
  const uint32_t init_bound = dim_bound < 64 ? dim_bound : 64;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n_paths;
       p += gridDim.x * blockDim.x) {
    const uint32_t sample = p % spp;
    const uint32_t loc = p / spp;
    uint32_t h = 2166136261u;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      h ^= (loc >> (8 * i)) & 0xffu;
      h *= 16777619u;
    }
    uint32_t dim = h % init_bound;
    const uint32_t gray = sample ^ (sample >> 1);
    float acc = 0.f;
    for (uint32_t k = 0; k < draws; ++k) {
      float v;
      if constexpr (kMode == 0) {
        v = __ldg(table + (size_t)sample * dim_bound + dim);
      } else {
        const uint32_t *vec = kMode == 2 ? s_vec + 32 * dim : dirs + 32 * (size_t)dim;
        uint32_t x = kMode == 2 ? s_vec[32 * dim_bound + dim] : __ldg(scramble + dim);
        for (uint32_t g = gray; g != 0; g &= g - 1) {
          x ^= kMode == 2 ? vec[__ffs(g) - 1] : __ldg(vec + (__ffs(g) - 1));
        }
        const float f = __fadd_rn(__fmul_rn(__uint2float_rn(x), 0x1p-32f), 0x1p-33f);
        v = f == 1.0f ? 0.0f : f;
      }
      acc = __fadd_rn(acc, v);
      ++dim;
      dim = dim == dim_bound ? 0u : dim;
    }
    out[p] = acc;
  }
}

} // namespace dev

cudaError_t launch_sobol_draws(int mode, const float *table, const uint32_t *dirs,
                               const uint32_t *scramble, uint32_t dim_bound, uint32_t spp,
                               uint32_t n_paths, uint32_t draws, uint32_t grid, float *out,
                               cudaStream_t s) {
  if (n_paths == 0) {
    return cudaSuccess;
  }
  switch (mode) {
  case 0:
    dev::k_sobol_draws<0><<<grid, 256, 0, s>>>(table, dirs, scramble, dim_bound, spp, n_paths,
                                               draws, out);
    break;
  case 1:
    dev::k_sobol_draws<1><<<grid, 256, 0, s>>>(table, dirs, scramble, dim_bound, spp, n_paths,
                                               draws, out);
    break;
  default:
    dev::k_sobol_draws<2><<<grid, 256, (size_t)dim_bound * 33 * 4, s>>>(
        table, dirs, scramble, dim_bound, spp, n_paths, draws, out);
    break;
  }
  return cudaGetLastError();
}

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

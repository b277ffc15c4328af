// Kernels of the render path: the integration megakernel, the second-stage
// pixel reduction, bulk closest-hit queries and the transcendental-function
// probe.  Compiled with --fmad=false (see geom.h).
#include "integrator.cuh"

namespace pg {
namespace dev {

// Megakernel: one thread per (pixel, sample range) of the WorkDivision, the
// thread's samples summed serially in FP32 (rendering_equation.h:51-124),
// then the sample_block_size lanes of a pixel summed by the shuffle tree and
// written by the first lane (mega_kernel/run_impl.h:165-204).  Held to 64
// registers (4 CTAs of 256 per SM), which measured 4% faster than 80.
template <uint32_t kTrav, bool kCount, bool kUniform>
__global__ void __launch_bounds__(256, 4) k_render(const RenderParams P) {
  const uint32_t block = blockIdx.x + P.start_block;
  const uint32_t tid = threadIdx.x;
  const ThreadWork tw = band_work(P, block, tid);
  Counts cnt = {0, 0, 0};
  rgb total = zero_rgb();
  if (!tw.exit) {
    for (uint32_t s = tw.start; s < tw.end; ++s) {
      total = total + integrate_sample<kTrav, kCount, kUniform>(P, s, tw.x, tw.y, cnt);
    }
  }
  const uint32_t sbs = P.wd.sample_block_size;
  total = sub_block_reduce(total, tid, sbs);
  if (!tw.exit && tid % sbs == 0) {
    const uint32_t nsb = P.wd.num_sample_blocks;
    const size_t idx = (block % nsb) + (size_t)nsb * (tw.x + (size_t)tw.y * P.x_dim);
    if (nsb == 1) {
      total = total / (float)P.spp;
    }
    write_pixel(P.out_rgb, P.out_bgra, P.output_bgra && nsb == 1, idx, total);
  }
  if (kCount) {
    atomicAdd(P.counters + 0, (unsigned long long)cnt.rays);
    atomicAdd(P.counters + 1, (unsigned long long)cnt.nodes);
    atomicAdd(P.counters + 2, (unsigned long long)cnt.tris);
  }
}

// the mega kernel with OutputPerStep output (mega_kernel/run_impl.h:
// 160-185): per-thread step sums, one sub-block reduction per step
template <uint32_t kTrav, bool kUniform>
__global__ void __launch_bounds__(256) k_render_steps(const RenderParams P) {
  const uint32_t block = blockIdx.x + P.start_block;
  const uint32_t tid = threadIdx.x;
  const ThreadWork tw = band_work(P, block, tid);
  rgb steps[kMaxOutputSteps];
  for (uint32_t k = 0; k < P.n_steps; ++k) {
    steps[k] = zero_rgb();
  }
  if (!tw.exit) {
    for (uint32_t s = tw.start; s < tw.end; ++s) {
      integrate_sample_steps<kTrav, kUniform>(P, s, tw.x, tw.y, steps);
    }
  }
  const uint32_t sbs = P.wd.sample_block_size;
  const uint32_t nsb = P.wd.num_sample_blocks;
  const size_t idx = (block % nsb) + (size_t)nsb * (tw.x + (size_t)tw.y * P.x_dim);
  for (uint32_t k = 0; k < P.n_steps; ++k) {
    rgb total = sub_block_reduce(steps[k], tid, sbs);
    if (!tw.exit && tid % sbs == 0) {
      if (nsb == 1) {
        total = total / (float)P.spp;
      }
      write_pixel(P.out_rgb + k * P.step_stride, nullptr, false, idx, total);
    }
    __syncthreads(); // the next step reuses the reduction's shared memory
  }
}

// ReduceFloatRGB pass (mega_kernel/reduce_float_rgb_impl.h:17-63)
__global__ void __launch_bounds__(1024) k_reduce(const ReduceParams P) {
  const uint32_t block = blockIdx.x;
  const uint32_t tid = threadIdx.x;
  const ThreadWork tw = thread_work(P.wd, block, tid);
  rgb total = zero_rgb();
  if (!tw.exit) {
    for (uint32_t i = tw.start; i < tw.end; ++i) {
      const size_t k = i + (size_t)tw.x * P.reduction_factor;
      total = total + mkrgb(P.in[3 * k], P.in[3 * k + 1], P.in[3 * k + 2]);
    }
  }
  const uint32_t sbs = P.wd.sample_block_size;
  total = sub_block_reduce(total, tid, sbs);
  if (!tw.exit && tid % sbs == 0) {
    const uint32_t nsb = P.wd.num_sample_blocks;
    const size_t idx = (block % nsb) + (size_t)nsb * tw.x;
    if (nsb == 1) {
      total = total / (float)P.spp;
    }
    write_pixel(P.out, P.out_bgra, P.output_bgra && nsb == 1, idx, total);
  }
}

template <uint32_t kTrav>
__global__ void k_intersect(const RenderParams P, const float *rays, uint32_t n,
                            const uint32_t *bvh_to_orig, int32_t *idx_out,
                            float *t_out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  ray r;
  r.o = mk(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]);
  r.d = mk(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]);
  Counts cnt = {0, 0, 0};
  Hit h = trace<kTrav, false>(P, r, cnt, PG_INF, -PG_INF);
  idx_out[i] = h.ok ? (int32_t)bvh_to_orig[h.idx] : -1;
  t_out[i] = h.ok ? h.t : __int_as_float(0x7fc00000);
}

__global__ void k_pmath(uint32_t fn, const float *x, const float *y, float *out,
                        uint32_t n) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  switch (fn) {
  case 0:
    out[i] = pm::sin(x[i]);
    break;
  case 1:
    out[i] = pm::cos(x[i]);
    break;
  case 2:
    out[i] = pm::asin(x[i]);
    break;
  case 3:
    out[i] = pm::acos(x[i]);
    break;
  default:
    out[i] = pm::pow(x[i], y[i]);
    break;
  }
}

} // namespace dev

namespace {
template <uint32_t kTrav, bool kCount>
void render_variant(const RenderParams &p, dim3 grid, dim3 block, cudaStream_t s) {
  if (p.rng_uniform) {
    dev::k_render<kTrav, kCount, true><<<grid, block, 0, s>>>(p);
  } else {
    dev::k_render<kTrav, kCount, false><<<grid, block, 0, s>>>(p);
  }
}

template <uint32_t kTrav>
void render_steps_variant(const RenderParams &p, dim3 grid, dim3 block, cudaStream_t s) {
  if (p.rng_uniform) {
    dev::k_render_steps<kTrav, true><<<grid, block, 0, s>>>(p);
  } else {
    dev::k_render_steps<kTrav, false><<<grid, block, 0, s>>>(p);
  }
}
} // namespace

cudaError_t launch_render(const RenderParams &p, uint32_t traversal,
                          uint32_t n_blocks, bool counting, cudaStream_t s) {
  const dim3 grid(n_blocks), block(p.wd.block_size);
  if (traversal == kTravWide) {
    if (counting) {
      render_variant<kTravWide, true>(p, grid, block, s);
    } else {
      render_variant<kTravWide, false>(p, grid, block, s);
    }
  } else {
    if (counting) {
      render_variant<kTravBinary, true>(p, grid, block, s);
    } else {
      render_variant<kTravBinary, false>(p, grid, block, s);
    }
  }
  return cudaGetLastError();
}

cudaError_t launch_render_steps(const RenderParams &p, uint32_t traversal,
                                uint32_t n_blocks, cudaStream_t s) {
  const dim3 grid(n_blocks), block(p.wd.block_size);
  if (traversal == kTravWide) {
    render_steps_variant<kTravWide>(p, grid, block, s);
  } else {
    render_steps_variant<kTravBinary>(p, grid, block, s);
  }
  return cudaGetLastError();
}

cudaError_t launch_reduce(const ReduceParams &p, cudaStream_t s) {
  dev::k_reduce<<<p.wd.total_blocks(), p.wd.block_size, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_intersect(const RenderParams &p, uint32_t traversal,
                             const float *rays, uint32_t n_rays,
                             const uint32_t *bvh_to_orig, int32_t *idx_out,
                             float *t_out, cudaStream_t s) {
  const uint32_t bs = 128;
  const uint32_t nb = (n_rays + bs - 1) / bs;
  if (nb == 0) {
    return cudaSuccess;
  }
  if (traversal == kTravWide) {
    dev::k_intersect<kTravWide><<<nb, bs, 0, s>>>(p, rays, n_rays, bvh_to_orig,
                                                  idx_out, t_out);
  } else {
    dev::k_intersect<kTravBinary><<<nb, bs, 0, s>>>(p, rays, n_rays, bvh_to_orig,
                                                    idx_out, t_out);
  }
  return cudaGetLastError();
}

cudaError_t launch_pmath(uint32_t fn, const float *x, const float *y,
                         float *out, uint32_t n, cudaStream_t s) {
  const uint32_t bs = 256;
  const uint32_t nb = (n + bs - 1) / bs;
  if (nb == 0) {
    return cudaSuccess;
  }
  dev::k_pmath<<<nb, bs, 0, s>>>(fn, x, y, out, n);
  return cudaGetLastError();
}

} // namespace pg

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

// The megakernel on the 8-wide BVH with warp-cooperative traversal.  Every
// thread keeps its WorkDivision samples and sums their radiance serially in
// sample order, exactly as k_render does, so the image is the same bit for
// bit; but the paths of a warp advance together one BVH node per lane and
// step (idle lanes start their next sample), leaf triangles are tested by
// the whole warp, and the lanes whose rays are done shade together once
// kShadeLanes of them are ready (or no lane is tracing).  Per lane the two
// rays of a vertex are traced in turn: the pending light ray, then the
// extension ray.  On the large-mesh room, 28 ready lanes measured best (8:
// 101, 16: 121, 24: 135, 28: 140, 32: 134 Msamples/s; the per-thread
// kernel 68).  With kSteps (OutputPerStep, rendering_equation.h:61-124) the
// radiance of path step k goes to the thread's step sum k and a path stops
// after P.n_steps steps, as in k_render_steps.
constexpr uint32_t kShadeLanes = 28;

template <bool kCount, bool kUniform, bool kSteps = false>
__global__ void __launch_bounds__(256, 2) k_render_coop(const RenderParams P) {
  const uint32_t block = blockIdx.x + P.start_block;
  const uint32_t tid = threadIdx.x;
  const uint32_t lane = tid & 31;
  __shared__ WarpTriScratch s_tri[8];
  WarpTriScratch &sh = s_tri[tid >> 5];
  const ThreadWork tw = band_work(P, block, tid);
  Counts cnt = {0, 0, 0};
  rgb total = zero_rgb();
  uint32_t smp = tw.start;
  const uint32_t end = tw.exit ? tw.start : tw.end;
  const LightSet L = lights_of(P);
  PathStateT<kUniform> s;
  uint32_t xw[kUniform ? kXorwowWords : 1];
  WideWalk w;
  w.done = true;
  uint32_t st_base[kWideStack];
  uint32_t st_bits[kWideStack];
  Hit lh = no_hit(), nh = no_hit();
  rgb steps[kSteps ? kMaxOutputSteps : 1];
  uint32_t step = 0; // OutputPerStep: the current path's step
  if constexpr (kSteps) {
    for (uint32_t k = 0; k < P.n_steps; ++k) {
      steps[k] = zero_rgb();
    }
  }
  // 0: start the next sample, 1: tracing the light ray, 2: tracing the
  // extension ray, 3: ready to shade, 4: all samples done
  uint32_t phase = 0;
  // the rays of the vertex just shaded (or of the camera sample)
  auto begin_rays = [&]() {
    lh = no_hit();
    nh = no_hit();
    ray r;
    r.o = s.o;
    if (s.has_light) {
      r.d = s.ld;
      wide_begin(P, w, r, light_bound(s.light_target), s.light_target);
      phase = 1;
    } else {
      r.d = s.d;
      wide_begin(P, w, r, PG_INF, -PG_INF);
      phase = 2;
    }
    if (kCount) {
      ++cnt.rays;
    }
  };
  while (true) {
    if (phase == 0) {
      if (smp < end) {
        path_begin(P, smp, tw.x, tw.y, s, xw, 1);
        if (P.initial_idx != nullptr) {
          // InitialIdxAndDir: the first hit is the caller's, at distance 1
          // from the front (initial_ray_sample.h:58-74)
          lh = no_hit();
          nh.t = 1.f;
          nh.idx = P.initial_idx[tw.x];
          nh.ok = true;
          nh.back = false;
          phase = 3;
        } else {
          begin_rays();
        }
      } else {
        phase = 4;
      }
    }
    if (__ballot_sync(kFull, phase != 4) == 0) {
      break;
    }
    const bool tracing = phase == 1 || phase == 2;
    uint32_t tri_base = 0, tmask = 0;
    if (tracing && !w.done) {
      wide_node<kCount>(P, w, st_base, st_bits, cnt, tri_base, tmask);
    }
    warp_triangles_shared<kCount, true>(P, w, tri_base, tmask, lane, cnt, sh);
    if (tracing && w.done) {
      if (phase == 1) {
        lh = w.best;
        if (s.has_next) {
          ray r;
          r.o = s.o;
          r.d = s.d;
          wide_begin(P, w, r, PG_INF, -PG_INF);
          phase = 2;
          if (kCount) {
            ++cnt.rays;
          }
        } else {
          phase = 3;
        }
      } else {
        nh = w.best;
        phase = 3;
      }
    }
    const uint32_t ready = __ballot_sync(kFull, phase == 3);
    const uint32_t busy = __ballot_sync(kFull, phase == 1 || phase == 2);
    if (ready != 0 && (__popc(ready) >= kShadeLanes || busy == 0) && phase == 3) {
      if constexpr (kSteps) {
        const bool cont = path_step(P, L, s, lh, nh);
        steps[step] = steps[step] + s.total;
        s.total = zero_rgb();
        ++step;
        if (cont && step < P.n_steps) {
          begin_rays();
        } else {
          step = 0;
          ++smp;
          phase = 0;
        }
      } else if (path_continues(P, s, path_step(P, L, s, lh, nh))) {
        begin_rays();
      } else {
        total = total + s.total;
        ++smp;
        phase = 0;
      }
    }
  }
  const uint32_t sbs = P.wd.sample_block_size;
  if constexpr (kSteps) {
    // one sub-block reduction per step (mega_kernel/run_impl.h:160-185)
    const uint32_t nsb = P.wd.num_sample_blocks;
    const size_t idx = (block % nsb) + (size_t)nsb * (tw.x + (size_t)tw.y * P.x_dim);
    for (uint32_t k = 0; k < P.n_steps; ++k) {
      rgb sum = sub_block_reduce(steps[k], tid, sbs);
      if (!tw.exit && tid % sbs == 0) {
        if (nsb == 1) {
          sum = sum / (float)P.spp;
        }
        write_pixel(P.out_rgb + k * P.step_stride, nullptr, false, idx, sum);
      }
      __syncthreads(); // the next step reuses the reduction's shared memory
    }
    return;
  }
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

// draws handed out in order (BSDF probe)
struct FixedDraws {
  float v[3];
  uint32_t k;
  __device__ float next() { return v[(k++) % 3]; }
};

// BSDF probe: op 0 continuous_eval, op 1 continuous_sample with the record's
// draws, op 2 the GGX distribution D (records of 9 floats, see
// path_debug_bsdf)
__global__ void k_bsdf(const DevMaterial *mat, uint32_t op, const float *in, uint32_t n,
                       float *out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  const Mat m = load_mat(mat);
  const float *a = in + (size_t)9 * i;
  if (op == 0) {
    rgb f = continuous_eval(m, mk(a[0], a[1], a[2]), mk(a[3], a[4], a[5]), mk(a[6], a[7], a[8]));
    out[3 * i] = f.r;
    out[3 * i + 1] = f.g;
    out[3 * i + 2] = f.b;
  } else if (op == 1) {
    FixedDraws d;
    d.v[0] = a[6];
    d.v[1] = a[7];
    d.v[2] = a[8];
    d.k = 0;
    Sample smp = continuous_sample(m, mk(a[0], a[1], a[2]), mk(a[3], a[4], a[5]), d);
    float *o = out + (size_t)6 * i;
    o[0] = smp.dir.x;
    o[1] = smp.dir.y;
    o[2] = smp.dir.z;
    o[3] = smp.mult.r;
    o[4] = smp.mult.g;
    o[5] = smp.mult.b;
  } else {
    out[i] = ggx_d(a[0], a[1] * a[1]);
  }
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
  if constexpr (kTrav == kTravWide) {
    // the 8-wide traversal runs warp-cooperatively
    if (p.rng_uniform) {
      dev::k_render_coop<kCount, true><<<grid, block, 0, s>>>(p);
    } else {
      dev::k_render_coop<kCount, false><<<grid, block, 0, s>>>(p);
    }
  } else if (p.rng_uniform) {
    dev::k_render<kTrav, kCount, true><<<grid, block, 0, s>>>(p);
  } else {
    dev::k_render<kTrav, kCount, false><<<grid, block, 0, s>>>(p);
  }
}

template <uint32_t kTrav>
void render_steps_variant(const RenderParams &p, dim3 grid, dim3 block, cudaStream_t s) {
  if constexpr (kTrav == kTravWide) {
    if (p.rng_uniform) {
      dev::k_render_coop<false, true, true><<<grid, block, 0, s>>>(p);
    } else {
      dev::k_render_coop<false, false, true><<<grid, block, 0, s>>>(p);
    }
  } else if (p.rng_uniform) {
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

cudaError_t launch_bsdf(const DevMaterial *mat, uint32_t op, const float *in, uint32_t n,
                        float *out, cudaStream_t s) {
  const uint32_t bs = 128;
  const uint32_t nb = (n + bs - 1) / bs;
  if (nb == 0) {
    return cudaSuccess;
  }
  dev::k_bsdf<<<nb, bs, 0, s>>>(mat, op, in, n, out);
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

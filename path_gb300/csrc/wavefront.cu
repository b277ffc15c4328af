// Wavefront ("streaming") render: persistent trace and shade kernels over
// queues, the GB300 form of the reference's streaming::Run
// (include/render/detail/integrate_image/streaming/run_impl.h:159-460).
//
// Path slots hold the state of up to n_slots camera samples between traces
// (PathState in structure-of-arrays form).  One iteration is
//   k_wf_trace : every queued ray (extension or light) of every live slot is
//                traced by a persistent grid, one wide-BVH node per lane and
//                step; idle lanes of a warp take new queue entries together;
//   k_wf_prep  : resets the queue heads for the shade pass;
//   k_wf_shade : every live slot runs one rendering_equation_iteration
//                (path_step, the same code the megakernel runs); slots whose
//                path continues are appended to the next live list and their
//                rays to the ray queue -- compacted per warp with ballots and
//                one atomic per warp and queue -- and finished slots write
//                their sample's radiance and take the next sample index.
// Sample radiance lands in a [samples][3] buffer; k_wf_sum then sums each
// pixel's samples in the reference's order (per WorkDivision thread, then
// the shuffle tree), so the image is bit-identical to the megakernel's.
#include "integrator.cuh"

#include <type_traits>

namespace pg {
namespace dev {

constexpr uint32_t kMissIdx = 0xffffffffu;
constexpr uint32_t kFlagNext = 1u, kFlagLight = 2u, kFlagEmission = 4u;

__device__ __forceinline__ uint2 pack_hit(const Hit &h) {
  uint2 v;
  v.x = __float_as_uint(h.t);
  v.y = h.ok ? (h.idx | (h.back ? 0x80000000u : 0u)) : kMissIdx;
  return v;
}

__device__ __forceinline__ Hit unpack_hit(uint2 v) {
  Hit h;
  h.ok = v.y != kMissIdx;
  h.t = __uint_as_float(v.x);
  h.idx = v.y & 0x7fffffffu;
  h.back = (v.y & 0x80000000u) != 0;
  return h;
}

// the pixel and sample index of a scene-local sample id (pixel-major order)
__device__ __forceinline__ void sample_coords(unsigned long long id, uint32_t spp,
                                              uint32_t x_dim, uint32_t &x, uint32_t &y,
                                              uint32_t &s) {
  unsigned long long pixel = id / spp;
  s = (uint32_t)(id - pixel * spp);
  x = (uint32_t)(pixel % x_dim);
  y = (uint32_t)(pixel / x_dim);
}

// the scene of a global sample id in a batched render: the last scene whose
// first sample is at or below it
__device__ __forceinline__ uint32_t scene_of(const WaveParams &W, unsigned long long id) {
  uint32_t lo = 0, hi = W.n_scenes;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) / 2;
    if (W.scenes[mid].first_sample <= id) {
      lo = mid;
    } else {
      hi = mid;
    }
  }
  return lo;
}

// Slot state: o (xyz, light target), d and ld (xyz, scene root node bits in
// w, read by the trace kernel), multipliers, radiance so far, and
// (id low word, id bits 32-39 | scene << 8, RNG dimension, iters | flags << 24).
// A fresh path (iters 0: no vertex shaded yet) stores only o, d and the
// state word: its light direction, multipliers and radiance are the start
// values (path_begin_cam), which unpack_path restores.  Otherwise a word is
// stored only when something reads it: ld (traced) and the light multiplier
// (added on a visible light hit) only with a pending light ray, the path
// multiplier only with a pending extension ray (path_step reads it only
// after an extension hit, and sets both multipliers afresh each vertex).
template <class S>
__device__ __forceinline__ void store_path(const WaveParams &W, uint32_t slot,
                                           const S &s, unsigned long long id,
                                           uint32_t scene, uint32_t root, bool fresh = false) {
  W.o[slot] = make_float4(s.o.x, s.o.y, s.o.z, s.light_target);
  W.d[slot] = make_float4(s.d.x, s.d.y, s.d.z, __uint_as_float(root));
  if (!fresh) {
    if (s.has_light) {
      W.ld[slot] = make_float4(s.ld.x, s.ld.y, s.ld.z, __uint_as_float(root));
      W.lmult[slot] = make_float4(s.light_mult.r, s.light_mult.g, s.light_mult.b, 0.f);
    }
    if (s.has_next) {
      W.mult[slot] = make_float4(s.multiplier.r, s.multiplier.g, s.multiplier.b, 0.f);
    }
    W.total[slot] = make_float4(s.total.r, s.total.g, s.total.b, 0.f);
  }
  uint32_t flags = (s.has_next ? kFlagNext : 0u) | (s.has_light ? kFlagLight : 0u) |
                   (s.count_emission ? kFlagEmission : 0u);
  uint32_t dim = 0; // a Uniform path's generator state is in W.rng_state
  if constexpr (std::is_same_v<S, PathState>) {
    dim = s.rng.dim;
  }
  W.state[slot] = make_uint4((uint32_t)id, ((uint32_t)(id >> 32) & 0xffu) | (scene << 8),
                             dim, s.iters | (flags << 24));
}

// the lights of a slot's scene
__device__ __forceinline__ LightSet scene_lights(const WaveParams &W, uint32_t scene) {
  if (W.scenes == nullptr) {
    return lights_of(W.P);
  }
  return lights_of(W.P, W.scenes[scene]);
}

// A lane's slot state (and both hits) copied into shared memory by
// asynchronous copies: the shade kernel stages a warp's next batch of slots
// once it has shaded the current one.  The light direction is not staged: a
// vertex's step sets it afresh when it samples a light, and it is read
// only by the trace.
struct SlotStage {
  float4 o, d, mult, lmult, total;
  uint4 state;
  uint2 hit_light, hit_ext;
};

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}

__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// fresh: every slot of the pass is fresh (the first pass after k_wf_init),
// so only o, d, the state word and the extension hit are staged
__device__ __forceinline__ void stage_slot(const WaveParams &W, uint32_t slot, SlotStage &g,
                                           bool fresh) {
  cp_async16(&g.o, W.o + slot);
  cp_async16(&g.d, W.d + slot);
  cp_async16(&g.state, W.state + slot);
  cp_async8(&g.hit_ext, W.hit_ext + slot);
  if (!fresh) {
    cp_async16(&g.mult, W.mult + slot);
    cp_async16(&g.lmult, W.lmult + slot);
    cp_async16(&g.total, W.total + slot);
    cp_async8(&g.hit_light, W.hit_light + slot);
  }
}

// a slot's path state from its staged words
template <bool kUniform>
__device__ __forceinline__ unsigned long long unpack_path(const WaveParams &W, uint32_t slot,
                                                          float4 o, float4 d, float4 m,
                                                          float4 lm, float4 t, uint4 st,
                                                          PathStateT<kUniform> &s,
                                                          uint32_t &scene, uint32_t &root) {
  const RenderParams &P = W.P;
  unsigned long long id = (unsigned long long)st.x | ((unsigned long long)(st.y & 0xffu) << 32);
  scene = st.y >> 8;
  root = __float_as_uint(d.w);
  s.o = mk(o.x, o.y, o.z);
  s.light_target = o.w;
  s.d = mk(d.x, d.y, d.z);
  s.ld = mk(0.f, 0.f, 0.f);
  s.multiplier = mkrgb(m.x, m.y, m.z);
  s.light_mult = mkrgb(lm.x, lm.y, lm.z);
  s.total = mkrgb(t.x, t.y, t.z);
  uint32_t flags = st.w >> 24;
  s.iters = st.w & 0xffffffu;
  s.has_next = (flags & kFlagNext) != 0;
  s.has_light = (flags & kFlagLight) != 0;
  s.count_emission = (flags & kFlagEmission) != 0;
  if (s.iters == 0) {
    // a fresh path: only o, d and this word were stored
    s.multiplier = mkrgb(1.f, 1.f, 1.f);
    s.light_mult = zero_rgb();
    s.total = zero_rgb();
  }
  unsigned long long local = id;
  uint32_t spp = P.spp, offset = P.sample_offset;
  if (W.scenes != nullptr) {
    local = id - W.scenes[scene].first_sample;
    spp = W.scenes[scene].spp;
    offset = W.scenes[scene].sample_offset;
  }
  if constexpr (kUniform) {
    s.rng.w = W.rng_state + slot;
    s.rng.stride = W.n_slots;
  } else {
    const uint32_t smp = (uint32_t)(local % spp);
    s.rng.begin(P, smp + offset);
    s.rng.dim = st.z;
  }
  return id;
}

template <bool kUniform>
__device__ __forceinline__ void begin_sample(const WaveParams &W, uint32_t slot,
                                             unsigned long long id) {
  uint32_t x, y, smp, scene = 0, root = 0;
  PathStateT<kUniform> s;
  if (W.scenes == nullptr) {
    sample_coords(id, W.P.spp, W.P.x_dim, x, y, smp);
    path_begin(W.P, smp, x, y, s, W.rng_state + slot, W.n_slots);
  } else {
    scene = scene_of(W, id);
    const BatchScene &b = W.scenes[scene];
    sample_coords(id - b.first_sample, b.spp, b.x_dim, x, y, smp);
    Camera cam;
    cam.f2w = b.f2w;
    cam.x_dim = b.x_dim;
    cam.y_dim = b.y_dim;
    cam.spp = b.spp;
    cam.sample_offset = b.sample_offset;
    path_begin_cam(W.P, cam, smp, x, y, s, W.rng_state + slot, W.n_slots);
    root = b.root;
  }
  store_path(W, slot, s, id, scene, root, true);
}

// slot i takes sample i; the first ray of each is queued
__global__ void k_wf_init(const WaveParams W, uint32_t n0) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n0) {
    return;
  }
  if (W.P.rng_uniform) {
    begin_sample<true>(W, i, W.first_sample + i);
  } else {
    begin_sample<false>(W, i, W.first_sample + i);
  }
  W.active[0][i] = i;
  W.rays[i] = i << 1;
}

constexpr uint32_t kRayChunk = 64; // queue entries a warp reserves at a time
constexpr int kRefillIdle = 4;     // idle lanes that make a warp take new rays

// Persistent trace: each lane walks one ray through the wide BVH one node
// (and the triangles of its leaf slots) per step; when kRefillIdle of a
// warp's lanes are idle they take new queue entries together from the
// warp's reserved run of entries (one atomic per kRayChunk entries), so
// lanes rarely wait on the longest ray of a batch.
// kStaged: the CTA first copies the BVH's top nodes (W.P.n_staged of them,
// breadth first from the root) into shared memory, where every lane reads
// them from then on.
template <bool kCount, int kMinBlocks, bool kStaged>
__global__ void __launch_bounds__(256, kMinBlocks) k_wf_trace(const WaveParams W) {
  extern __shared__ uint4 s_top[];
  __shared__ WarpTriScratch s_tri[8];
  const uint32_t lane = threadIdx.x & 31;
  WarpTriScratch &sh = s_tri[threadIdx.x >> 5];
  const uint32_t n_top = kStaged ? W.P.n_staged : 0u;
  if constexpr (kStaged) {
    for (uint32_t i = threadIdx.x; i < 5 * n_top; i += blockDim.x) {
      s_top[i] = __ldg(W.P.wide_nodes + i);
    }
    __syncthreads();
  }
  const uint32_t count = W.q->rays;
  Counts cnt = {0, 0, 0};
  WideWalk w;
  w.done = true;
  bool have = false;
  bool drained = false;
  uint32_t entry = 0;
  uint32_t st_base[kWideStack];
  uint32_t st_bits[kWideStack];
  // the warp's reserved run of queue entries [next_i, chunk_end): taken
  // kRayChunk at a time with one atomic (every warp adds to the same
  // cursor), handed out to idle lanes in order
  uint32_t next_i = 0, chunk_end = 0;
  while (true) {
    const uint32_t idle = __ballot_sync(kFull, !have);
    if (!drained && __popc(idle) >= kRefillIdle) {
      const uint32_t need = (uint32_t)__popc(idle);
      const uint32_t avail = chunk_end - next_i;
      uint32_t nb = 0;
      if (need > avail) {
        if (lane == 0) {
          nb = atomicAdd(&W.q->ray_cursor, kRayChunk);
        }
        nb = __shfl_sync(kFull, nb, 0);
      }
      const uint32_t rank = (uint32_t)__popc(idle & ((1u << lane) - 1u));
      const uint32_t i = rank < avail ? next_i + rank : nb + (rank - avail);
      if (need > avail) {
        next_i = nb + (need - avail);
        chunk_end = nb + kRayChunk;
      } else {
        next_i += need;
      }
      drained = next_i >= count;
      if (!have) {
        if (i < count) {
          entry = W.rays[i];
          const uint32_t slot = entry >> 1;
          const bool light = (entry & 1u) != 0;
          const float4 o = W.o[slot];
          const float4 d = light ? W.ld[slot] : W.d[slot];
          sh.o[lane] = o;
          sh.d[lane] = d;
          ray r;
          r.o = mk(o.x, o.y, o.z);
          r.d = mk(d.x, d.y, d.z);
          wide_begin(W.P, w, r, light ? light_bound(o.w) : PG_INF, light ? o.w : -PG_INF,
                     __float_as_uint(d.w));
          have = true;
          if (kCount) {
            ++cnt.rays;
          }
        }
      }
    }
    if (__ballot_sync(kFull, have) == 0) {
      if (drained) {
        break;
      }
      continue;
    }
    uint32_t tri_base = 0, tmask = 0;
    if (have && !w.done) {
      wide_node<kCount, kStaged>(W.P, w, st_base, st_bits, cnt, tri_base, tmask, s_top, n_top);
    }
    warp_triangles_shared<kCount>(W.P, w, tri_base, tmask, lane, cnt, sh);
    if (have && w.done) {
      const uint32_t slot = entry >> 1;
      ((entry & 1u) ? W.hit_light : W.hit_ext)[slot] = pack_hit(w.best);
      have = false;
    }
  }
  if (kCount) {
    atomicAdd(W.P.counters + 0, (unsigned long long)cnt.rays);
    atomicAdd(W.P.counters + 1, (unsigned long long)cnt.nodes);
    atomicAdd(W.P.counters + 2, (unsigned long long)cnt.tris);
  }
}

__global__ void k_wf_prep(const WaveParams W, uint32_t parity) {
  W.q->active[parity ^ 1u] = 0;
  W.q->rays = 0;
  W.q->shade_cursor = 0;
  W.q->ray_cursor = 0;
}

// warp-aggregated append: lanes with pred get consecutive positions
__device__ __forceinline__ uint32_t warp_append(uint32_t *counter, bool pred, uint32_t lane) {
  const uint32_t mask = __ballot_sync(kFull, pred);
  uint32_t base = 0;
  if (lane == 0 && mask != 0) {
    base = atomicAdd(counter, (uint32_t)__popc(mask));
  }
  base = __shfl_sync(kFull, base, 0);
  return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

constexpr uint32_t kNoMaterial = 0xffffffffu;

// Adds v[0..N) to d_params[mat][off..off+N) for every lane's material: lanes
// of one material are summed across the warp first (shuffle butterfly),
// then one FP64 atomic per value.  All 32 lanes call this; kNoMaterial
// lanes add nothing.
template <int N>
__device__ __forceinline__ void warp_grad(double *out, uint32_t mat, const float (&v)[N],
                                          int off, uint32_t lane) {
  uint32_t todo = __ballot_sync(kFull, mat != kNoMaterial);
  while (todo != 0) {
    const uint32_t leader = __ffs(todo) - 1;
    const uint32_t m = __shfl_sync(kFull, mat, leader);
    const bool mine = mat == m && ((todo >> lane) & 1u) != 0;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      float x = mine ? v[k] : 0.f;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        x += __shfl_xor_sync(kFull, x, o);
      }
      if (lane == leader) {
        atomicAdd(out + (size_t)m * 7 + off + k, (double)x);
      }
    }
    todo &= ~__ballot_sync(kFull, mine);
  }
}

// One rendering_equation_iteration per live slot.  With kGrad the same
// iteration is replayed for the adjoint (path replay: same Sobol draws,
// same rays) and its derivative terms are accumulated: the forward
// radiance L of the sample (sample_rgb) minus what has been gathered gives
// the radiance that flowed through each vertex's continuation, which times
// d log f / d(parameter) of that vertex is its parameter gradient; the
// light sample adds its own term, and emission terms are linear.  Sampling
// densities and the light table are held fixed (detached estimator).
// path_step is inlined and the kernel held to 64 registers (4 CTAs of 256
// per SM): the latency of the slot loads is hidden by more resident warps,
// which measured faster than fewer warps without register spills.  kCache
// (paths end into the radiance cache) is a template parameter so that the
// plain kernel carries none of the cache-query code.
// Each warp takes batches of 32 live slots.  Once it has shaded a batch it
// takes the next one and copies each slot's state into shared memory
// (cp.async: all of a lane's words in flight at once, held in no register
// and read where the step uses them); other warps shade while the copies
// land.  The next batch's slot indices are taken only then, so that no
// register holds them through the step (fewer spills under the 64-register
// bound than taking them first).
template <bool kGrad, bool kUniform, bool kCache, uint32_t kFeat = kFeatAll>
__global__ void __launch_bounds__(256, 4) k_wf_shade(const WaveParams W, uint32_t parity) {
  __shared__ SlotStage s_stage[256];
  const uint32_t lane = threadIdx.x & 31;
  SlotStage &g = s_stage[threadIdx.x];
  const uint32_t count = W.q->active[parity];
  const uint32_t *in = W.active[parity];
  uint32_t *out = W.active[parity ^ 1u];
  auto take = [&]() {
    uint32_t b = 0;
    if (lane == 0) {
      b = atomicAdd(&W.q->shade_cursor, 32u);
    }
    return __shfl_sync(kFull, b, 0);
  };
  uint32_t base = take();
  if (base >= count) {
    return;
  }
  bool valid = base + lane < count;
  uint32_t slot = valid ? in[base + lane] : 0u;
  if (valid) {
    stage_slot(W, slot, g, W.pass == kPassFresh);
  }
  cp_async_commit();
  while (true) {
    cp_async_wait_all();
    bool live = false, finished = false, want_next = false, want_light = false;
    uint32_t gm_vertex = kNoMaterial, gm_light = kNoMaterial, gm_emit = kNoMaterial;
    float gv_vertex[4] = {0.f, 0.f, 0.f, 0.f};
    float gv_light[3] = {0.f, 0.f, 0.f}, gv_emit[3] = {0.f, 0.f, 0.f};
    if (valid) {
      PathStateT<kUniform> s;
      uint32_t scene, root;
      unsigned long long id = unpack_path(W, slot, g.o, g.d, g.mult, g.lmult, g.total, g.state,
                                          s, scene, root);
      Hit lh = s.has_light ? unpack_hit(g.hit_light) : no_hit();
      Hit nh = s.has_next ? unpack_hit(g.hit_ext) : no_hit();
      if (!kGrad) {
        StepTrace tr;
        StepTrace *trp = kCache ? &tr : nullptr;
        bool cont = path_continues(
            W.P, s, path_step<kUniform, kFeat>(W.P, scene_lights(W, scene), s, lh, nh, trp));
        if constexpr (!kCache) {
          // the sample id, scene and root read again from the staged words
          // (volatile: no register holds them through the step)
          const volatile uint32_t *vs = reinterpret_cast<const volatile uint32_t *>(&g.state);
          const uint32_t sx = vs[0], sy = vs[1];
          id = (unsigned long long)sx | ((unsigned long long)(sy & 0xffu) << 32);
          scene = sy >> 8;
          root = reinterpret_cast<const volatile uint32_t *>(&g.d)[3];
        }
        if (trp != nullptr && tr.cache_query) {
          // the path ends into the radiance cache: its query and throughput
          const size_t k = (size_t)(id - W.first_sample);
          float *q = W.cache_q + 12 * k;
          const f3 wo = -tr.in;
          // a batch shares one cache: the scene's cell of it
          const f3 cp = W.scenes != nullptr ? batch_cache_position(W.scenes[scene], tr.point)
                                            : tr.point;
          const float vals[12] = {cp.x, cp.y, cp.z, wo.x, wo.y, wo.z,
                                  tr.normal.x, tr.normal.y, tr.normal.z, tr.albedo.r,
                                  tr.albedo.g, tr.albedo.b};
          for (int j = 0; j < 12; ++j) {
            q[j] = vals[j];
          }
          W.cache_beta[3 * k] = s.multiplier.r;
          W.cache_beta[3 * k + 1] = s.multiplier.g;
          W.cache_beta[3 * k + 2] = s.multiplier.b;
        }
        if (cont) {
          store_path(W, slot, s, id, scene, root);
          live = true;
          want_next = s.has_next;
          want_light = s.has_light;
        } else {
          float *dst = W.sample_rgb + 3 * (id - W.first_sample);
          dst[0] = s.total.r;
          dst[1] = s.total.g;
          dst[2] = s.total.b;
          finished = true;
        }
      } else {
        const RenderParams &P = W.P;
        StepTrace tr;
        bool cont = path_continues(
            P, s, path_step<kUniform, kFeat>(P, scene_lights(W, scene), s, lh, nh, &tr));
        // as in the plain branch: id, scene and root, and the vertex's
        // multipliers before the step, from the staged words
        rgb beta, lmult;
        {
          const SlotStage &st = s_stage[threadIdx.x];
          const volatile uint32_t *vs = reinterpret_cast<const volatile uint32_t *>(&st.state);
          const uint32_t sx = vs[0], sy = vs[1], sw = vs[3];
          id = (unsigned long long)sx | ((unsigned long long)(sy & 0xffu) << 32);
          scene = sy >> 8;
          root = reinterpret_cast<const volatile uint32_t *>(&st.d)[3];
          const volatile float *vm = reinterpret_cast<const volatile float *>(&st.mult);
          const volatile float *vl = reinterpret_cast<const volatile float *>(&st.lmult);
          if ((sw & 0xffffffu) == 0) {
            // a fresh path: the start values unpack_path gave it
            beta = mkrgb(1.f, 1.f, 1.f);
            lmult = zero_rgb();
          } else {
            beta = mkrgb(vm[0], vm[1], vm[2]);
            lmult = mkrgb(vl[0], vl[1], vl[2]);
          }
        }
        const float *lf = W.sample_rgb + 3 * (id - W.first_sample);
        const rgb l_sample = mkrgb(lf[0], lf[1], lf[2]);
        const unsigned long long pixel = id / P.spp;
        const float *gp = W.d_image + 3 * pixel;
        const float inv_spp = 1.f / (float)P.spp;
        const rgb g = mkrgb(gp[0] * inv_spp, gp[1] * inv_spp, gp[2] * inv_spp);
        const uint32_t pm = W.pend_mat[slot];
        rgb nee_add = zero_rgb(), emit_add = zero_rgb();
        if (tr.light_added) {
          nee_add = emission_of(P.materials + tr.light_mat) * lmult;
          gm_light = tr.light_mat;
          gv_light[0] = g.r * lmult.r;
          gv_light[1] = g.g * lmult.g;
          gv_light[2] = g.b * lmult.b;
        }
        if (tr.emit_added) {
          emit_add = beta * emission_of(P.materials + tr.mat);
          gm_emit = tr.mat;
          gv_emit[0] = g.r * beta.r;
          gv_emit[1] = g.g * beta.g;
          gv_emit[2] = g.b * beta.b;
        }
        if (pm != kNoMaterial) {
          // radiance through the pending vertex's continuation, and its
          // light sample's contribution (resolved by this step)
          const float4 pr = W.pend_refl[slot], pn = W.pend_nee[slot];
          const rgb rest = l_sample - (s.total - emit_add);
          gm_vertex = pm;
          gv_vertex[0] = g.r * (rest.r * pr.x + nee_add.r * pn.x);
          gv_vertex[1] = g.g * (rest.g * pr.y + nee_add.g * pn.y);
          gv_vertex[2] = g.b * (rest.b * pr.z + nee_add.b * pn.z);
          gv_vertex[3] = (g.r * (rest.r * pr.w + nee_add.r * pn.w) +
                          g.g * (rest.g * pr.w + nee_add.g * pn.w)) +
                         g.b * (rest.b * pr.w + nee_add.b * pn.w);
        }
        uint32_t npm = kNoMaterial;
        if (cont && tr.hit) {
          const Mat mat = load_mat(P.materials + tr.mat);
          rgb r1 = zero_rgb(), r2 = zero_rgb();
          float a1 = 0.f, a2 = 0.f;
          bool any = false;
          if (tr.continuous && s.has_next &&
              bsdf_log_grad(mat, tr.in, tr.next_dir, tr.normal, r1, a1)) {
            any = true;
          }
          if (tr.nee && bsdf_log_grad(mat, tr.in, tr.nee_dir, tr.normal, r2, a2)) {
            any = true;
          }
          if (any) {
            npm = tr.mat;
            W.pend_refl[slot] = make_float4(r1.r, r1.g, r1.b, a1);
            W.pend_nee[slot] = make_float4(r2.r, r2.g, r2.b, a2);
          }
        }
        W.pend_mat[slot] = npm;
        if (cont) {
          store_path(W, slot, s, id, scene, root);
          live = true;
          want_next = s.has_next;
          want_light = s.has_light;
        } else {
          finished = true;
        }
      }
    }
    if (kGrad) {
      warp_grad<4>(W.d_params, gm_vertex, gv_vertex, 0, lane);
      warp_grad<3>(W.d_params, gm_light, gv_light, 4, lane);
      warp_grad<3>(W.d_params, gm_emit, gv_emit, 4, lane);
    }
    __syncwarp();
    // finished slots take the next sample index (one atomic per warp)
    {
      const uint32_t mask = __ballot_sync(kFull, finished);
      unsigned long long first = 0;
      if (lane == 0 && mask != 0) {
        first = atomicAdd(W.next_sample, (unsigned long long)__popc(mask));
      }
      first = __shfl_sync(kFull, first, 0);
      if (finished) {
        unsigned long long id = first + (unsigned long long)__popc(mask & ((1u << lane) - 1u));
        if (id < W.total_samples) {
          begin_sample<kUniform>(W, slot, id);
          if (kGrad) {
            W.pend_mat[slot] = kNoMaterial;
          }
          live = true;
          want_next = true;
          want_light = false;
        }
      }
    }
    const uint32_t pos = warp_append(&W.q->active[parity ^ 1u], live, lane);
    if (live) {
      out[pos] = slot;
    }
    // the warp's extension rays, then its light rays, with one atomic
    {
      const uint32_t mn = __ballot_sync(kFull, want_next);
      const uint32_t ml = __ballot_sync(kFull, want_light);
      const uint32_t below = (1u << lane) - 1u;
      uint32_t rb = 0;
      if (lane == 0 && (mn | ml) != 0) {
        rb = atomicAdd(&W.q->rays, (uint32_t)(__popc(mn) + __popc(ml)));
      }
      rb = __shfl_sync(kFull, rb, 0);
      if (want_next) {
        W.rays[rb + __popc(mn & below)] = slot << 1;
      }
      if (want_light) {
        W.rays[rb + __popc(mn) + __popc(ml & below)] = (slot << 1) | 1u;
      }
    }
    // the next batch's slots, staged before it is shaded
    const uint32_t next_base = take();
    if (next_base >= count) {
      break;
    }
    const bool next_valid = next_base + lane < count;
    const uint32_t next_slot = next_valid ? in[next_base + lane] : 0u;
    if (next_valid) {
      stage_slot(W, next_slot, g, W.pass == kPassFresh);
    }
    cp_async_commit();
    slot = next_slot;
    valid = next_valid;
  }
}

// The shade pass when no live path has an extension ray left, only the
// light ray of its last vertex: under NIters{N} with every sample in flight
// from the first pass, the pass after the (N + 1)-th shaded vertex.  Each
// live slot adds its light ray's emission when the ray reached the light
// point (the first lines of path_step, the same arithmetic) and writes its
// sample's radiance: four words of slot state read instead of the shade
// kernel's staged seven, and none of its code.  A slot with an extension
// ray pending means the host counted the passes wrong: the slot sets
// kStatusPassCount rather than dropping its path without a word.
__global__ void __launch_bounds__(256) k_wf_finish(const WaveParams W, uint32_t parity) {
  const RenderParams &P = W.P;
  const uint32_t count = W.q->active[parity];
  const uint32_t *in = W.active[parity];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += gridDim.x * blockDim.x) {
    const uint32_t slot = in[i];
    const uint4 st = W.state[slot];
    const uint32_t flags = st.w >> 24;
    if ((flags & kFlagNext) != 0) {
      set_status(P.status, kStatusPassCount);
      continue;
    }
    const unsigned long long id =
        (unsigned long long)st.x | ((unsigned long long)(st.y & 0xffu) << 32);
    const float4 t4 = W.total[slot];
    rgb total = mkrgb(t4.x, t4.y, t4.z);
    if ((flags & kFlagLight) != 0) {
      const Hit lh = unpack_hit(W.hit_light[slot]);
      if (lh.ok && pm::fabs(W.o[slot].w - lh.t) <= 1e-6f && (P.back_cull == 0 || !lh.back)) {
        const float4 lm = W.lmult[slot];
        const float4 c = __ldg(P.tri_data + 3 * lh.idx + 2);
        total = total + emission_of(P.materials + __float_as_uint(c.w)) * mkrgb(lm.x, lm.y, lm.z);
      }
    }
    float *dst = W.sample_rgb + 3 * (id - W.first_sample);
    dst[0] = total.r;
    dst[1] = total.g;
    dst[2] = total.b;
  }
}

// each WorkDivision thread sums its samples in order, then the shuffle tree
// (the same summation as k_render, from the per-sample buffer)
__global__ void __launch_bounds__(256) k_wf_sum(const RenderParams P, const float *sample_rgb) {
  const uint32_t block = blockIdx.x + P.start_block;
  const uint32_t tid = threadIdx.x;
  const ThreadWork tw = band_work(P, block, tid);
  rgb total = zero_rgb();
  if (!tw.exit) {
    // sample_rgb starts at the band's first pixel
    const size_t pixel = tw.x + (size_t)(tw.y - P.row_lo) * P.x_dim;
    const float *v = sample_rgb + 3 * (pixel * P.spp + tw.start);
    const uint32_t n = tw.end - tw.start;
    uint32_t s = 0;
    if ((reinterpret_cast<uintptr_t>(v) & 15u) == 0) {
      // four samples from three 16-byte loads, added in the same order: a
      // lane reads whole lines instead of one 12-byte sample per load
      const float4 *v4 = reinterpret_cast<const float4 *>(v);
      for (; s + 4 <= n; s += 4, v4 += 3) {
        const float4 a = __ldg(v4), b = __ldg(v4 + 1), c = __ldg(v4 + 2);
        total = total + mkrgb(a.x, a.y, a.z);
        total = total + mkrgb(a.w, b.x, b.y);
        total = total + mkrgb(b.z, b.w, c.x);
        total = total + mkrgb(c.y, c.z, c.w);
      }
    }
    for (; s < n; ++s) {
      total = total + mkrgb(v[3 * s], v[3 * s + 1], v[3 * s + 2]);
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
}

} // namespace dev

cudaError_t launch_wavefront_init(const WaveParams &w, uint32_t n0, cudaStream_t s) {
  if (n0 == 0) {
    return cudaSuccess;
  }
  dev::k_wf_init<<<(n0 + 255) / 256, 256, 0, s>>>(w, n0);
  return cudaGetLastError();
}

namespace {
template <bool kCount>
void *trace_kernel(uint32_t min_blocks, bool staged) {
  switch (min_blocks) {
  case 3:
    return (void *)dev::k_wf_trace<kCount, 3, false>;
  case 5:
    return (void *)dev::k_wf_trace<kCount, 5, false>;
  case 6:
    return (void *)dev::k_wf_trace<kCount, 6, false>;
  default:
    return staged ? (void *)dev::k_wf_trace<kCount, 4, true>
                  : (void *)dev::k_wf_trace<kCount, 4, false>;
  }
}

size_t staged_bytes(uint32_t n_staged) { return (size_t)n_staged * sizeof(WideNode); }

// the staged nodes and the static per-warp scratch together can pass the
// default 48 KB of shared memory per CTA
cudaError_t allow_staged(void *k, uint32_t n_staged) {
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)staged_bytes(n_staged));
}
} // namespace

int wavefront_trace_blocks_per_sm(uint32_t min_blocks, bool counting, uint32_t n_staged) {
  int n = 0;
  const bool staged = n_staged > 0 && (min_blocks == 0 || min_blocks == 4);
  void *k = counting ? trace_kernel<true>(min_blocks, staged)
                     : trace_kernel<false>(min_blocks, staged);
  if ((staged && allow_staged(k, n_staged) != cudaSuccess) ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 256,
                                                    staged ? staged_bytes(n_staged) : 0) !=
          cudaSuccess ||
      n < 1) {
    n = 1;
  }
  return n;
}

cudaError_t launch_wavefront_trace(const WaveParams &w, uint32_t trace_grid,
                                   uint32_t min_blocks, bool counting, cudaStream_t s) {
  const bool staged = w.P.n_staged > 0 && (min_blocks == 0 || min_blocks == 4);
  void *k = counting ? trace_kernel<true>(min_blocks, staged)
                     : trace_kernel<false>(min_blocks, staged);
  void *args[] = {const_cast<WaveParams *>(&w)};
  if (staged) {
    const cudaError_t e = allow_staged(k, w.P.n_staged);
    if (e != cudaSuccess) {
      return e;
    }
  }
  return cudaLaunchKernel(k, dim3(trace_grid), dim3(256), args,
                          staged ? staged_bytes(w.P.n_staged) : 0, s);
}

cudaError_t launch_wavefront_shade(const WaveParams &w, uint32_t parity, uint32_t shade_grid,
                                   cudaStream_t s, bool grad) {
  dev::k_wf_prep<<<1, 1, 0, s>>>(w, parity);
  if (w.pass == kPassLightOnly && !grad) {
    dev::k_wf_finish<<<shade_grid, 256, 0, s>>>(w, parity);
    return cudaGetLastError();
  }
  const bool u = w.P.rng_uniform != 0;
  const bool cache = w.cache_q != nullptr;
  if (grad) {
    if (u) {
      dev::k_wf_shade<true, true, false><<<shade_grid, 256, 0, s>>>(w, parity);
    } else if (feat_covers(kFeatPlain, w.feat)) {
      dev::k_wf_shade<true, false, false, kFeatPlain><<<shade_grid, 256, 0, s>>>(w, parity);
    } else {
      dev::k_wf_shade<true, false, false><<<shade_grid, 256, 0, s>>>(w, parity);
    }
  } else if (cache) {
    if (u) {
      dev::k_wf_shade<false, true, true><<<shade_grid, 256, 0, s>>>(w, parity);
    } else if (feat_covers(kFeatPlain, w.feat)) {
      dev::k_wf_shade<false, false, true, kFeatPlain><<<shade_grid, 256, 0, s>>>(w, parity);
    } else {
      dev::k_wf_shade<false, false, true><<<shade_grid, 256, 0, s>>>(w, parity);
    }
  } else if (u) {
    dev::k_wf_shade<false, true, false><<<shade_grid, 256, 0, s>>>(w, parity);
  } else if (feat_covers(kFeatPlain, w.feat)) {
    dev::k_wf_shade<false, false, false, kFeatPlain><<<shade_grid, 256, 0, s>>>(w, parity);
  } else {
    dev::k_wf_shade<false, false, false><<<shade_grid, 256, 0, s>>>(w, parity);
  }
  return cudaGetLastError();
}

cudaError_t launch_wavefront_sum(const RenderParams &p, const float *sample_rgb,
                                 uint32_t n_blocks, cudaStream_t s) {
  if (n_blocks == 0) {
    return cudaSuccess;
  }
  dev::k_wf_sum<<<n_blocks, p.wd.block_size, 0, s>>>(p, sample_rgb);
  return cudaGetLastError();
}

} // namespace pg

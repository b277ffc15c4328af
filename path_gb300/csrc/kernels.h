// Launch interface between the host orchestration and the CUDA kernels.
#pragma once

#include "devtypes.h"
#include "workdiv.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace pg {

struct RenderParams {
  // geometry (device pointers)
  const float4 *tris;       // BVH order, 3 float4 per triangle
  const float4 *tri_data;   // normals + material, 3 float4 per triangle
  const uint4 *bin_nodes;   // 2 uint4 per binary node
  const uint32_t *extra_idxs;
  const uint4 *wide_nodes;  // 5 uint4 per wide node
  const float4 *wide_tris;  // 3 float4 per wide-leaf triangle
  uint32_t n_tris, n_bin_nodes, n_wide_nodes;
  const DevMaterial *materials;
  const float4 *light_tris; // 3 float4 per light triangle: v0, e0, e1
  const float *light_cdf;
  uint32_t n_lights;
  // rng: Sobol table [spp][dim_bound], and the direction vectors
  // [dim_bound][32] followed by the scramble constants [dim_bound]
  const float *sobol;
  const uint32_t *sobol_vec;
  uint32_t dim_bound, init_dim_bound;
  // integrator settings
  uint32_t light_sampler, dir_sampler, term_prob, term_iters;
  float term_prob_prob, term_exp, term_min_prob;
  uint32_t back_cull, target_objects;
  // camera: film_to_world, or caller rays [x_dim][6] (InitialRays and
  // InitialIdxAndDir specs)
  const float *initial_rays;
  // InitialIdxAndDir: BVH-order triangle hit at distance 1 per location
  const uint32_t *initial_idx;
  // OutputPerStep: n_steps > 0 writes step k's partial sums at
  // out_rgb + k * step_stride (floats)
  uint32_t n_steps;
  size_t step_stride;
  float f2w[12];
  uint32_t x_dim, y_dim, spp;
  WorkDiv wd;
  // outputs
  float *out_rgb;     // [nsb * x_dim * y_dim][3]
  uint8_t *out_bgra;  // [x_dim * y_dim][4] when output_bgra and nsb == 1
  uint32_t output_bgra;
  uint32_t *status;   // first in-kernel error code
  unsigned long long *counters; // [3] rays, nodes, triangles (counting runs)
  uint32_t start_block;
  // image rows [row_lo, row_hi) are rendered; threads of other rows exit
  uint32_t row_lo, row_hi;
  // Sobol row of sample s is s + sample_offset
  uint32_t sample_offset;
  // radiance cache: paths end into the cache at this vertex (0 = off)
  uint32_t cache_depth;
  // Uniform RNG (cuRAND XORWOW per path) instead of the Sobol table
  uint32_t rng_uniform;
  // streaming trace: wide nodes [0, n_staged) (the breadth-first top of the
  // BVH) are read from a copy in shared memory
  uint32_t n_staged;
};

enum Traversal : uint32_t { kTravBinary = 0, kTravWide = 1 };

// 32-bit words of one Uniform-RNG path state (a curandStateXORWOW)
constexpr uint32_t kRngStateWords = 12;

// queue heads of the wavefront render
struct WaveQueues {
  uint32_t active[2];   // live-slot counts of the two live lists
  uint32_t rays;        // entries in the ray queue
  uint32_t ray_cursor;  // next ray entry to trace
  uint32_t shade_cursor;
  uint32_t pad[3];
};

// the root of a batch scene without triangles: its rays meet nothing
constexpr uint32_t kEmptyRoot = 0xffffffffu;

// one scene of a batched render: its camera, samples and place in the
// concatenated geometry (wide nodes, triangles, materials, lights)
struct BatchScene {
  float f2w[12];
  uint32_t x_dim, y_dim, spp;
  uint32_t root;               // wide-node index of the scene's root (kEmptyRoot: no triangles)
  uint32_t light_off, n_lights; // its emissive triangles in the light table
  // radiance-cache coordinates of a batch with one cache: a position p of
  // this scene is (p - cache_lo) * cache_inv (its box onto [0, 1]^3) plus
  // twice the cell (cache_cell % 16, cache_cell / 16 % 16, cache_cell / 256)
  float cache_lo[3], cache_inv[3];
  uint32_t cache_cell;
  uint32_t sample_offset;          // Sobol row of its sample s: s + sample_offset
  unsigned long long first_sample; // global id of its first sample
};

// a batch item's radiance-cache cell: up to 16^3
constexpr uint32_t kCacheCellsPerAxis = 16;
constexpr uint32_t kMaxCacheCells = kCacheCellsPerAxis * kCacheCellsPerAxis * kCacheCellsPerAxis;

// wavefront render state (device pointers); slot arrays hold PathState
struct WaveParams {
  RenderParams P;
  float4 *o;      // vertex xyz, light target distance in w
  float4 *d;      // next extension direction
  float4 *ld;     // light ray direction
  float4 *mult;   // path multiplier
  float4 *lmult;  // light sample multiplier
  float4 *total;  // radiance gathered so far
  uint4 *state;   // sample id (2 words), RNG dimension, iters | flags << 24
  uint2 *hit_ext, *hit_light;
  uint32_t *active[2]; // live slot lists
  uint32_t *rays;      // ray queue: slot << 1 | (1 for the light ray)
  WaveQueues *q;
  unsigned long long *next_sample;
  unsigned long long first_sample; // first sample id of the rendered rows
  unsigned long long total_samples; // one past the last sample id
  float *sample_rgb;   // [total_samples - first_sample][3]
  uint32_t n_slots;
  // batched render: sample ids run over the scenes in order (nullptr: the
  // single scene of P)
  const BatchScene *scenes;
  uint32_t n_scenes;
  // adjoint replay (gradient shading only).  sample_rgb then holds the
  // forward render's per-sample radiance and is only read.
  const float *d_image;  // dLoss / d(pixel radiance), [x_dim * y_dim][3]
  float4 *pend_refl;     // pending vertex: d log f / d(reflectance rgb, roughness)
                         // along its continuation
  float4 *pend_nee;      // ... along its light sample
  uint32_t *pend_mat;    // its material, 0xffffffff when none
  double *d_params;      // [materials][7]: reflectance rgb, roughness, emission rgb
  // radiance cache (P.cache_depth > 0): per sample the query of the vertex
  // where its path ended into the cache ([12] floats) and the path
  // throughput there (zero when the path ended before it)
  float *cache_q;
  float *cache_beta;
  // Uniform RNG: the XORWOW state words of slot i at rng_state[k * n_slots + i]
  uint32_t *rng_state;
  // features of the work (kFeat* in devtypes.h: the BSDF types of the
  // scenes' materials and the fixed setting choices), for the choice of a
  // specialised shade kernel
  uint32_t feat;
  // what the host knows of the pass's live slots (kPass*)
  uint32_t pass;
};

// kPassFresh: every live slot is fresh (the first pass after k_wf_init);
// kPassLightOnly: no live slot has an extension ray pending, only the light
// ray of its last vertex (k_wf_finish shades the pass)
constexpr uint32_t kPassGeneral = 0, kPassFresh = 1, kPassLightOnly = 2;

// the features (kFeat*) of rendering a scene whose materials have the BSDF
// types mat_types (bit per type) with the settings in p
inline uint32_t work_features(uint32_t mat_types, const RenderParams &p) {
  return (mat_types & kFeatAllMats) | (p.term_prob == 1 ? kFeatNIters : 0u) |
         (p.dir_sampler == 0 ? kFeatBsdfDir : 0u) | (p.light_sampler == 0 ? kFeatLightTri : 0u);
}

cudaError_t launch_wavefront_init(const WaveParams &w, uint32_t n0, cudaStream_t s);
// resident blocks per SM of the trace kernel compiled for min_blocks
int wavefront_trace_blocks_per_sm(uint32_t min_blocks, bool counting, uint32_t n_staged);
// one wavefront iteration: trace the queued rays, then reset the queues
// and shade (launch_wavefront_shade)
cudaError_t launch_wavefront_trace(const WaveParams &w, uint32_t trace_grid,
                                   uint32_t min_blocks, bool counting, cudaStream_t s);
cudaError_t launch_wavefront_shade(const WaveParams &w, uint32_t parity, uint32_t shade_grid,
                                   cudaStream_t s, bool grad = false);
// per-pixel sums of the sample buffer into p.out_rgb / p.out_bgra
cudaError_t launch_wavefront_sum(const RenderParams &p, const float *sample_rgb,
                                 uint32_t n_blocks, cudaStream_t s);

// training records for the radiance cache: n full-length paths from random
// pixels, each its vertex at `depth` (or its last) ([n][16]: query,
// radiance, pad)
cudaError_t launch_nrc_paths(const RenderParams &p, uint32_t n, uint32_t frame, uint32_t depth,
                             float *records, cudaStream_t s);
// the same over a batch: each path takes a random scene of scenes[0..n_scenes)
// (its camera, root and lights) and records its position in the scene's
// cache cell
cudaError_t launch_nrc_paths_batch(const RenderParams &p, const BatchScene *scenes,
                                   uint32_t n_scenes, uint32_t n, uint32_t frame,
                                   uint32_t depth, float *records, cudaStream_t s);
// sample_rgb[i] += beta[i] * max(pred[i], 0) for the n samples
cudaError_t launch_nrc_apply(float *sample_rgb, const float *beta, const float *pred,
                             size_t n, cudaStream_t s);

// integration megakernel over blocks [start_block, start_block + n_blocks)
cudaError_t launch_render(const RenderParams &p, uint32_t traversal,
                          uint32_t n_blocks, bool counting, cudaStream_t s);
// the mega kernel with OutputPerStep output (p.n_steps > 0)
cudaError_t launch_render_steps(const RenderParams &p, uint32_t traversal,
                                uint32_t n_blocks, cudaStream_t s);

// one ReduceFloatRGB pass (reduce_float_rgb_impl.h:17-63)
struct ReduceParams {
  const float *in;
  float *out;
  uint8_t *out_bgra;
  uint32_t reduction_factor;
  uint32_t spp;
  uint32_t output_bgra;
  WorkDiv wd;
};
cudaError_t launch_reduce(const ReduceParams &p, cudaStream_t s);

// closest hit for a batch of rays: idx = original triangle index or -1
cudaError_t launch_intersect(const RenderParams &p, uint32_t traversal,
                             const float *rays, uint32_t n_rays,
                             const uint32_t *bvh_to_orig, int32_t *idx_out,
                             float *t_out, cudaStream_t s);

// Sobol table from direction vectors [dim][32] and scrambles [dim]
cudaError_t launch_sobol_table(const uint32_t *dirs, const uint32_t *scramble,
                               uint32_t dimension_bound, uint32_t count,
                               float *out, cudaStream_t s);
cudaError_t launch_sobol_curand(const uint32_t *dirs, const uint32_t *scramble,
                                uint32_t dimension_bound, uint32_t count,
                                float *out, cudaStream_t s);

cudaError_t launch_pmath(uint32_t fn, const float *x, const float *y,
                         float *out, uint32_t n, cudaStream_t s);
// Sobol draw cost: mode 0 table reads, 1 direction vectors XOR-ed in
// registers (vectors through L1), 2 the same with the vectors in shared
// memory; out[p] = the sum of path p's draws
cudaError_t launch_sobol_draws(int mode, const float *table, const uint32_t *dirs,
                               const uint32_t *scramble, uint32_t dim_bound, uint32_t spp,
                               uint32_t n_paths, uint32_t draws, uint32_t grid, float *out,
                               cudaStream_t s);
// BSDF probe over n records of 9 floats (ops as path_debug_bsdf)
cudaError_t launch_bsdf(const DevMaterial *mat, uint32_t op, const float *in, uint32_t n,
                        float *out, cudaStream_t s);

// tensor-core self-test: D [128][n] = A [128][k] . B [n][k]^T (BF16 in, FP32
// out), one CTA; err set when the MMA did not complete within wait_limit
// polls (0: the kernels' limit); issue false: no MMA is issued, so the wait
// runs out
cudaError_t launch_tc_gemm(const void *a, const void *b, float *d, uint32_t k_dim,
                           uint32_t n_dim, uint32_t *err, cudaStream_t s,
                           uint32_t wait_limit = 0, bool issue = true);

} // namespace pg

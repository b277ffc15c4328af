/*
 * CPU oracle for the render hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, on the CPU, the reference's algorithm for the path
 * tracer's render hot path (SBVH build, BVH traversal, Moller-Trumbore
 * triangle test, the next-event-estimation integrator, BSDFs, the
 * RandomTriangle light sampler, the table-driven Sobol RNG, WorkDivision,
 * the per-pixel reducer and the output stage).  It is the checker that the
 * CUDA kernels are compared against: only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline leg may load it, and nothing in the product links
 * or calls it.
 *
 * Every function cites the reference file:line it follows.  Arithmetic is
 * IEEE single precision in the reference's evaluation order with no fused
 * multiply-add (built with -ffp-contract=off); transcendental functions come
 * from path_gb300/csrc/pmath.h so that the oracle and the kernels agree bit
 * for bit (the reference's own -Ofast build is not reproducible at the ulp
 * level, see CMakeLists.txt:35-40).  A second build, liboracle_libm.so
 * (-DORACLE_LIBM), calls the C library's sinf / cosf / asinf / acosf / powf
 * where the reference calls the std:: functions instead: the distance
 * between the two builds' images is how far the shared polynomials move an
 * image from the C library's arithmetic.
 *
 * Parity pins: closest-hit ids against the reference's brute-force LoopAll
 * rule and hand-written rays (tests/src/intersection.cu:120-177), clipped
 * triangle boxes (tests/src/clipped_triangle.cpp:26-118), rotation
 * (tests/src/projection.cpp:5-34), WorkDivision coverage
 * (tests/src/work_division.cpp:24-110), reducer sums (tests/src/reduce.cu),
 * node packing (tests/src/node.cpp).  Sobol values are pinned against cuRAND
 * itself on the GPU.  The integrator as a whole has no golden image in the
 * reference (no test renders an image), so image-level parity is pinned only
 * through these component pins.
 */
#pragma once

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Material record, 64 bytes; same field meaning as the C-ABI path_material. */
typedef struct {
  uint32_t type; /* 0 Diffuse, 1 Glossy, 2 DiffuseGlossy, 3 DiffuseMirror,
                    4 Mirror, 5 DielectricRefractive, 6 GGX */
  float diffuse[3];
  float specular[3];
  float shininess;
  float ior;
  float diffuse_weight;
  float glossy_weight;
  float roughness;
  float emission[3];
  float pad;
} oracle_material;

/* Scene in the reference's scene::Scene form (include/scene/scene.h:29-130) */
typedef struct {
  const float *triangles;   /* [n_triangles][3][3] object space */
  const float *normals;     /* [n_triangles][3][3] vertex normals */
  const uint32_t *tri_material;
  uint32_t n_triangles;
  const uint32_t *mesh_ends; /* [n_meshes] */
  const uint32_t *cluster_ends_per_mesh; /* [n_meshes] */
  uint32_t n_meshes;
  const float *instance_xforms; /* [n_instances][3][4] object to world */
  const uint32_t *instance_mesh; /* [n_instances] */
  uint32_t n_instances;
  const uint32_t *clusters; /* [n_clusters][3] material, start, end */
  uint32_t n_clusters;
  const oracle_material *materials;
  uint32_t n_materials;
} oracle_scene;

typedef struct {
  uint32_t block_size;
  uint32_t target_x_block_size;
  uint32_t force_target_samples;
  uint32_t forced_target_samples_per_thread;
  uint32_t base_num_threads;
  float samples_per_thread_scaling_power;
  uint32_t max_samples_per_thread;
} oracle_work_division_settings;

typedef struct {
  oracle_work_division_settings render_wd;
  oracle_work_division_settings reduce_wd;
  uint32_t max_blocks_per_launch;
  float overlap_threshold;
  uint32_t use_spatial_splits;
  float traversal_per_intersect_cost;
  uint32_t target_objects;
  uint32_t light_sampler; /* 0 RandomTriangle, 1 NoLightSampling */
  uint32_t dir_sampler;   /* 0 BSDF, 1 Uniform */
  uint32_t term_prob;     /* 0 Constant, 1 NIters, 2 MultiplierFunc, 3 Normalize */
  float term_prob_prob;   /* Constant */
  uint32_t term_prob_iters; /* NIters */
  float term_prob_exp;    /* MultiplierFunc */
  float term_prob_min_prob; /* MultiplierFunc, Normalize */
  uint32_t max_sample_size; /* Sobol dimension bound */
  uint32_t back_cull_emission;
  uint32_t reduce_order; /* 0: CPU lane order, 1: GPU shuffle-tree order */
  uint32_t n_threads;    /* OpenMP threads, 0 = default */
  uint32_t rng;          /* 0 Sobel, 1 Uniform (std::mt19937) */
  uint32_t tie_rule;     /* closest hit at equal distance: 0 the reference's
                            (a later candidate wins, optional_min.h), 1 the
                            GPU 8-wide traversal's (smallest BVH-order index,
                            independent of the visit order) */
} oracle_settings;

typedef struct {
  uint32_t block_size, base_samples_per_thread, n_threads_per_unit_extra,
      sample_block_size, x_block_size, y_block_size, num_sample_blocks,
      num_x_blocks, num_y_blocks, x_dim, y_dim;
} oracle_work_division;

/* pmath functions: fn 0 sin, 1 cos, 2 asin, 3 acos, 4 pow(x, y) */
void oracle_pmath(int fn, const float *x, const float *y, float *out, size_t n);

/* Moller-Trumbore on each (triangle, ray) pair; t = NaN when no hit */
void oracle_triangle_intersect(const float *tris, const float *rays, size_t n,
                               float *t_out, int32_t *is_back_out);

/* brute force closest hit (LoopAll): idx = -1 when no hit */
void oracle_loop_all(const float *tris, uint32_t n_tris, const float *rays,
                     size_t n_rays, int32_t *idx_out, float *t_out);

/* SBVH build over world-space triangles */
void *oracle_sbvh_build(const float *tris, uint32_t n_tris,
                        float overlap_threshold, uint32_t use_spatial_splits,
                        float traversal_per_intersect_cost,
                        uint32_t target_objects);
void oracle_sbvh_free(void *h);
/* sizes: [n_nodes, n_extra, n_perm] */
void oracle_sbvh_sizes(void *h, uint32_t *sizes);
/* nodes as [n][2] packed words (node.h layout) + [n][6] aabb */
void oracle_sbvh_export(void *h, uint32_t *node_words, float *node_aabbs,
                        uint32_t *extra_idxs, uint32_t *permutation);
/* closest hit through the BVH; idx is the ORIGINAL triangle index */
void oracle_bvh_intersect(void *h, const float *rays, size_t n_rays,
                          int32_t *idx_out, float *t_out);
float oracle_sah_cost(void *h, float traversal_per_intersect_cost);

/* ClippedTriangle::new_bounds */
void oracle_clipped_new_bounds(const float *tri, const float *bounds,
                               float left, float right, uint32_t axis,
                               float *out);

/* find_rotate_vector_to_vector applied to inp */
void oracle_rotate_to(const float *inp, const float *target, float *out);
void oracle_find_relative_vec(const float *vec, float phi, float theta,
                              float *out);

int oracle_work_division_make(const oracle_work_division_settings *s,
                              uint32_t samples_per, uint32_t x_dim,
                              uint32_t y_dim, oracle_work_division *out);
/* thread info: out = [start, end, x, y, exit] */
void oracle_work_division_thread_info(const oracle_work_division *wd,
                                      uint32_t block_idx, uint32_t thread_idx,
                                      uint32_t *out);

/* sub_block_reduce emulation: sums [n_blocks*block_size] values in groups of
 * sub_block_size, either in CPU lane order (order 0) or GPU tree order (1) */
void oracle_sub_block_reduce(const float *vals, uint32_t n_blocks,
                             uint32_t block_size, uint32_t sub_block_size,
                             uint32_t order, float *out);

/* Sobol table vals[i * dimension_bound + d] (src/rng/sobel/sobel.cu:21-93),
 * direction vectors and scramble constants fetched from cuRAND's host API */
int oracle_sobol_table(uint32_t dimension_bound, uint32_t count, float *out);

/* full render of a square image; out = [y_dim * x_dim][3] FloatRGB.
 * rows [row_start, row_end) only (others left untouched); returns 0 on
 * success.  seconds = wall time of the integration + reduction. */
int oracle_render(const oracle_scene *scene, const oracle_settings *settings,
                  uint32_t samples_per, uint32_t x_dim, uint32_t y_dim,
                  const float *film_to_world, uint32_t row_start,
                  uint32_t row_end, float *out, double *seconds);

/* scene::get_camera_transform (src/scene/camera.cpp:4-27): 3x4 row-major
 * film_to_world */
void oracle_camera_transform(const float *look, const float *up, const float *pos,
                             float height_angle_deg, float width_height_ratio, float *out);

/* BSDF evaluation for tests, n records of 9 floats in `in`:
 *   op 0: continuous_eval, in = (in dir, out dir, normal), out [n][3];
 *   op 1: continuous_sample with the draws u0, u1, u2 in that order,
 *         in = (in dir, normal, u0, u1, u2), out [n][6] = (dir, multiplier);
 *   op 2: the GGX distribution D, in = (n.h, alpha, -), out [n]. */
int oracle_debug_bsdf(const oracle_material *material, uint32_t op, const float *in,
                      uint32_t n, float *out);

/* Options of a render of a prepared scene. */
typedef struct {
  uint32_t row_start;     /* rows row_start, row_start + row_stride, ... */
  uint32_t row_end;       /* below row_end (0 = y_dim) */
  uint32_t row_stride;    /* 0 or 1 = every row */
  uint32_t sample_offset; /* Sobol row of sample s is s + sample_offset */
  uint32_t mode;          /* 0: FP32 image through WorkDivision and the
                             reducer (the reference's CPU path), out =
                             [y_dim][x_dim][3] floats, selected rows written;
                             1: every sample summed per pixel in double,
                             out_f64 = [y_dim][x_dim][3] mean radiance;
                             2: per-sample radiance, out = [selected rows]
                             [x_dim][samples_per][3] */
} oracle_render_options;

/* The flattened scene and its SBVH, built once (free with
 * oracle_prepared_free) for renders with the same accel settings and light
 * sampler. */
void *oracle_prepare(const oracle_scene *scene, const oracle_settings *settings);
void oracle_prepared_free(void *prepared);
/* returns 0, 1 on invalid arguments, 2 when the settings' accel fields or
 * light sampler differ from the ones the scene was prepared with.  seconds =
 * wall time of the integration (+ reduction in mode 0). */
int oracle_render_prepared(void *prepared, const oracle_settings *settings,
                           uint32_t samples_per, uint32_t x_dim, uint32_t y_dim,
                           const float *film_to_world, const oracle_render_options *opt,
                           float *out, double *out_f64, double *seconds);

/* InitialRays (idxs NULL) or InitialIdxAndDir (idxs = scene-order triangle
 * hit at distance 1 along each ray) sample spec.  out = [n_rays][3]
 * FloatRGB, or [n_steps][n_rays][3] with OutputPerStep (n_steps > 0). */
int oracle_render_rays(const oracle_scene *scene, const oracle_settings *settings,
                       uint32_t samples_per, const float *rays, const uint32_t *idxs,
                       uint32_t n_rays, uint32_t n_steps, float *out);

/* OutputPerStep of a square image: out = [n_steps][y_dim * x_dim][3] */
int oracle_render_steps(const oracle_scene *scene, const oracle_settings *settings,
                        uint32_t samples_per, uint32_t x_dim, uint32_t y_dim,
                        const float *film_to_world, uint32_t n_steps, float *out);

/* render with BGRA32 output: out = [y_dim * x_dim][4] bytes */
int oracle_render_bgra(const oracle_scene *scene,
                       const oracle_settings *settings, uint32_t samples_per,
                       uint32_t x_dim, uint32_t y_dim,
                       const float *film_to_world, uint8_t *out);

/* per-sample radiance of one pixel (debugging): out = [n][3] */
int oracle_render_samples(const oracle_scene *scene,
                          const oracle_settings *settings,
                          uint32_t samples_per, uint32_t x_dim, uint32_t y_dim,
                          const float *film_to_world, uint32_t x, uint32_t y,
                          float *out);

#ifdef __cplusplus
}
#endif

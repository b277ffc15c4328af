/*
 * path_gb300: C ABI of the GB300-native render hot path.
 *
 * The entry points below replace the reference's render API for the path
 * tracer (rgreenblatt/path).  All types are plain C: pointers, sizes and POD
 * structs; no C++ or torch types cross the boundary.  Every function returns
 * a path_status; on failure path_last_error() describes the cause.  Calls on
 * one renderer are synchronous and a renderer is not thread safe (as with
 * render::Renderer); use one renderer per host thread.
 */
#ifndef PATH_GB300_H
#define PATH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PATH_OK = 0,
  PATH_ERR_ARGUMENT = 1,     /* bad pointer, size or setting value */
  PATH_ERR_SCENE_PARSE = 2,  /* XML / OBJ / MTL / YAML could not be read */
  PATH_ERR_OOM = 3,          /* device or host allocation failed */
  PATH_ERR_DEVICE_TIMEOUT = 4, /* a kernel's bounded wait or stack check
                                  gave up; the device status word says where */
  PATH_ERR_UNSUPPORTED = 5,  /* setting combination not built */
  PATH_ERR_CUDA = 6,         /* CUDA runtime error */
  PATH_ERR_IO = 7            /* file could not be opened or written */
} path_status;

/* include/execution_model/execution_model.h:3-6.  This library implements
 * the GPU execution model; PATH_EXEC_CPU is rejected with
 * PATH_ERR_UNSUPPORTED (there is no CPU fallback in the product). */
typedef enum { PATH_EXEC_CPU = 0, PATH_EXEC_GPU = 1 } path_exec_model;

/* include/bsdf/union_bsdf.h:17-24 (+ GGX, which the reference lacks) */
typedef enum {
  PATH_BSDF_DIFFUSE = 0,
  PATH_BSDF_GLOSSY = 1,
  PATH_BSDF_DIFFUSE_GLOSSY = 2,
  PATH_BSDF_DIFFUSE_MIRROR = 3,
  PATH_BSDF_MIRROR = 4,
  PATH_BSDF_DIELECTRIC_REFRACTIVE = 5,
  PATH_BSDF_GGX = 6
} path_bsdf_type;

/* scene::Material = bsdf::Material<UnionBSDF> (include/scene/material.h),
 * 64 bytes.  Field use per type:
 *   DIFFUSE: diffuse.  GLOSSY: specular, shininess.  MIRROR: specular.
 *   DIFFUSE_GLOSSY / DIFFUSE_MIRROR: diffuse, specular, shininess,
 *     diffuse_weight, glossy_weight (include/bsdf/combined.h weights).
 *   DIELECTRIC_REFRACTIVE: specular, ior.  GGX: specular = F0, roughness. */
typedef struct {
  uint32_t type;
  float diffuse[3];
  float specular[3];
  float shininess;
  float ior;
  float diffuse_weight;
  float glossy_weight;
  float roughness;
  float emission[3];
  float pad;
} path_material;

/* kernel::WorkDivisionSettings (include/kernel/work_division_settings.h) */
typedef struct {
  uint32_t block_size;
  uint32_t target_x_block_size;
  uint32_t force_target_samples;
  uint32_t forced_target_samples_per_thread;
  uint32_t base_num_threads;
  float samples_per_thread_scaling_power;
  uint32_t max_samples_per_thread;
} path_work_division_settings;

typedef enum { PATH_KERNEL_MEGA = 0, PATH_KERNEL_STREAMING = 1 } path_kernel_approach;
typedef enum { PATH_LIGHT_RANDOM_TRIANGLE = 0, PATH_LIGHT_NONE = 1 } path_light_sampler;
typedef enum { PATH_DIR_BSDF = 0, PATH_DIR_UNIFORM = 1 } path_dir_sampler;
typedef enum {
  PATH_TERM_CONSTANT = 0,
  PATH_TERM_N_ITERS = 1,
  PATH_TERM_MULTIPLIER_FUNC = 2,
  PATH_TERM_NORMALIZE = 3
} path_term_prob;
/* Sobel: the scrambled Sobol table (rng_from_sequence_gen.h).  Uniform: one
 * cuRAND XORWOW generator per sample, seeded with sample + location x spp and
 * drawn with curand_uniform, 1.0 mapped to 0.0 (include/rng/uniform/
 * uniform.h:18-76, the reference's GPU execution model; its CPU model draws
 * std::mt19937 instead, so the two agree only in expectation). */
typedef enum { PATH_RNG_SOBEL = 0, PATH_RNG_UNIFORM = 1 } path_rng;
typedef enum {
  PATH_TRAVERSAL_BINARY = 0, /* the reference's binary SBVH and traversal order */
  PATH_TRAVERSAL_WIDE8 = 1   /* compressed 8-wide quantised BVH */
} path_traversal;

/* render::Settings (include/render/settings.h:27-70), flattened.  The last
 * block holds the GB300-specific knobs with no reference counterpart. */
typedef struct {
  uint32_t kernel_approach; /* path_kernel_approach */
  uint32_t max_blocks_per_launch_gpu;
  uint32_t max_blocks_per_launch_cpu;
  path_work_division_settings render_work_division;
  path_work_division_settings reduce_work_division;
  /* accel SBVH (include/intersect/accel/sbvh/settings.h) */
  float overlap_threshold;
  uint32_t use_spatial_splits;
  float traversal_per_intersect_cost;
  uint32_t target_objects;
  /* light sampler */
  uint32_t light_sampler;
  uint32_t binary_search_threshold;
  /* direction sampler */
  uint32_t dir_sampler;
  /* termination probability */
  uint32_t term_prob;
  float term_prob_prob;      /* Constant */
  uint32_t term_prob_iters;  /* NIters */
  float term_prob_exp;       /* MultiplierFunc */
  float term_prob_min_prob;  /* MultiplierFunc, Normalize */
  /* rng */
  uint32_t rng;
  uint32_t max_sample_size;
  /* integrate::RenderingEquationSettings */
  uint32_t back_cull_emission;
  /* GB300 knobs */
  uint32_t traversal;        /* path_traversal */
  uint32_t persistent_ctas_per_sm; /* 0 = one launch over all blocks */
  uint32_t count_work;       /* 1: count rays / nodes / triangles (slower) */
  uint32_t upload_scene_every_render; /* 1: re-copy the cached scene arrays
                                         the render reads (triangles, shading
                                         data, its traversal's BVH, materials,
                                         lights) host -> device on every
                                         render */
  uint32_t trace_min_blocks; /* streaming trace kernel: resident 256-thread
                                blocks per SM it is compiled for (3..6, 0 =
                                default 4); fewer registers per thread above 3 */
  uint32_t time_kernels;     /* 1: time the streaming trace launches with CUDA
                                events (path_render_stats.trace_ms) */
  uint32_t gpu_build;        /* build the 8-wide BVH on the GPU: 1 = PLOC
                                clustering of the triangles in Morton order,
                                collapsed to 8-wide; 2 = the same after
                                splitting triangles much smaller than their
                                boxes into clipped references (spatial
                                splits); the wide traversal only, no binary
                                SBVH.  0 = the host SBVH */
  uint32_t wavefront_slots_log2; /* streaming: paths in flight = 2^this
                                    (10..26, 0 = default 26) */
  uint32_t trace_staged_nodes; /* streaming trace kernel: the top nodes of the
                                  8-wide BVH (breadth-first, at most 512)
                                  each CTA keeps in shared memory; 0 = none */
} path_settings;

typedef enum {
  PATH_SAMPLE_SQUARE_IMAGE = 0,
  PATH_SAMPLE_INITIAL_RAYS = 1,
  PATH_SAMPLE_INITIAL_IDX_AND_DIR = 2
} path_sample_spec_type;

/* render::SampleSpec (include/render/renderer.h:19-41).  INITIAL_RAYS and
 * INITIAL_IDX_AND_DIR render one location per entry (x = entry index, one
 * row).  INITIAL_IDX_AND_DIR (render::InitialIdxAndDirSpec, renderer.h:31-35)
 * starts each path at a known hit: triangle idxs[i] (index in scene order:
 * instances in order, each mesh's triangles in order) at distance 1 along
 * rays[i], front side; MegaKernel approach only, as in the reference. */
typedef struct {
  uint32_t type;          /* path_sample_spec_type */
  uint32_t x_dim, y_dim;  /* SQUARE_IMAGE */
  float film_to_world[12]; /* 3x4 row-major affine, SQUARE_IMAGE */
  const float *rays;      /* INITIAL_*: [n_rays][6] origin, unit direction */
  uint32_t n_rays;
  const uint32_t *idxs;   /* INITIAL_IDX_AND_DIR: [n_rays] triangle index */
  /* SQUARE_IMAGE: render only image rows [row_start, row_end) (a band, for
   * sharding one image over several GPUs; both 0 = every row).  A band's
   * pixels are computed exactly as in the whole-image render; output rows
   * outside the band are left untouched.  GB300 addition. */
  uint32_t row_start, row_end;
  /* first Sobol sample index of every pixel (GB300 addition: progressive
   * rendering in frames of samples [sample_offset, sample_offset + spp)) */
  uint32_t sample_offset;
} path_sample_spec;

typedef enum {
  PATH_OUTPUT_BGRA = 0,
  PATH_OUTPUT_FLOAT_RGB = 1,
  PATH_OUTPUT_PER_STEP = 2
} path_output_type;

/* Most path steps one PER_STEP render may ask for. */
#define PATH_MAX_OUTPUT_STEPS 64u

/* render::Output (include/render/renderer.h:13-17,37-38).  data is host
 * memory unless on_device is set, in which case it is a device pointer and
 * the final copy to the host is skipped.  PER_STEP (OutputType::OutputPerStep)
 * writes, for each path step k < n_steps, the mean radiance gathered at that
 * step, and cuts every path after n_steps steps; MegaKernel approach only, as
 * in the reference. */
typedef struct {
  uint32_t type;      /* path_output_type */
  void *data;         /* BGRA: 4 bytes/location (B,G,R,0); FLOAT_RGB: 3
                         floats/location; PER_STEP: [n_steps][locations][3] */
  uint32_t on_device;
  uint32_t n_steps;   /* PER_STEP: 1..PATH_MAX_OUTPUT_STEPS */
} path_output;

typedef struct path_scene path_scene;
typedef struct path_renderer path_renderer;

/* Statistics from the last render (GB300 addition). */
typedef struct {
  double seconds;            /* same span as the reference's returned time */
  double kernel_ms;          /* CUDA-event time of the integration kernels */
  double bvh_build_seconds;  /* host SBVH build (excluded from seconds) */
  uint64_t rays_traced;      /* extension + shadow rays (counting runs only) */
  uint64_t nodes_visited;
  uint64_t triangles_tested;
  uint32_t gpu_launches;     /* kernels this library launched for the render */
  uint32_t device_status;    /* 0, or the first in-kernel error code: 1 traversal
                                stack overflow, 2 object list overflow, 3 bad
                                node, 4 path beyond 4096 vertices, 5 an extension
                                ray in a light-only last pass */
  uint32_t num_bvh_nodes;
  uint32_t num_wide_nodes;
  uint64_t h2d_bytes;        /* host -> device bytes copied by this render */
  uint64_t d2h_bytes;        /* device -> host bytes copied by this render */
  double trace_ms;           /* time_kernels: summed event time of the
                                streaming trace launches */
  uint32_t trace_launches;   /* streaming trace launches of this render */
} path_render_stats;

/* ---- errors ---- */
/* message of the last failed call on this thread (empty string if none) */
const char *path_last_error(void);

/* ---- settings ---- */
/* defaults of render::Settings{} (include/render/settings.h:27-45) */
path_status path_settings_default(path_settings *out);
/* reads a render settings YAML file in the reference's schema
 * (src/render/config_io.cpp:14-35, configs/benchmark.yaml) */
path_status path_settings_load_yaml(const char *path, path_settings *out);

/* ---- scenes ---- */
/* scene::TriangleConstructor (include/scene/triangle_constructor.h:8-19) */
path_status path_scene_create(path_scene **out);
void path_scene_destroy(path_scene *scene);
path_status path_scene_add_material(path_scene *scene,
                                    const path_material *material,
                                    uint32_t *material_idx);
/* replaces material material_idx in place (GB300 addition: parameter
 * updates for differentiation); a renderer holding the scene re-uploads its
 * materials and light table on the next render without rebuilding the BVH */
path_status path_scene_set_material(path_scene *scene, uint32_t material_idx,
                                    const path_material *material);
/* triangles: [n][3][3]; normals: [n][3][3] vertex normals or NULL for the
 * face normal (scenefile_loader.cpp:280-284); material_idx per triangle.
 * Adds one mesh with an identity instance; emissive clusters follow
 * scene::TriangleConstructor::add_triangle. */
path_status path_scene_add_mesh(path_scene *scene, const float *triangles,
                                const float *normals,
                                const uint32_t *material_idx, uint32_t n,
                                const float *object_to_world /* 3x4 or NULL */);
/* ScenefileLoader::load_scene (src/scene/scenefile_compat/scenefile_loader.cpp
 * :23-62): CS123 XML scene + OBJ/MTL meshes.  film_to_world receives the
 * camera transform for the given aspect ratio (3x4 row-major). */
path_status path_scene_load_xml(const char *path, float width_height_ratio,
                                path_scene **out, float *film_to_world);
/* scene::get_camera_transform (src/scene/camera.cpp:4-27) */
path_status path_camera_transform(const float *look, const float *up,
                                  const float *pos, float height_angle_deg,
                                  float width_height_ratio,
                                  float *film_to_world);
/* sizes: [n_triangles, n_meshes, n_instances, n_clusters, n_materials] */
path_status path_scene_sizes(const path_scene *scene, uint32_t *sizes);
/* exports the scene in the reference's scene::Scene arrays (see oracle) */
path_status path_scene_export(const path_scene *scene, float *triangles,
                              float *normals, uint32_t *tri_material,
                              uint32_t *mesh_ends,
                              uint32_t *cluster_ends_per_mesh,
                              float *instance_xforms, uint32_t *instance_mesh,
                              uint32_t *clusters, path_material *materials);

/* ---- renderer ---- */
/* render::Renderer (include/render/renderer.h:43-70) */
path_status path_renderer_create(path_renderer **out);
void path_renderer_destroy(path_renderer *renderer);
/* Renderer::render (include/render/renderer.h:51-54).  seconds receives the
 * time from after scene / accel setup through the output copy
 * (include/render/detail/general_render_impl.h:174-241). */
path_status path_render(path_renderer *renderer, uint32_t exec_model,
                        const path_sample_spec *sample_spec,
                        const path_output *output, const path_scene *scene,
                        uint32_t samples_per, const path_settings *settings,
                        uint32_t show_progress, double *seconds);
path_status path_renderer_stats(const path_renderer *renderer,
                                path_render_stats *out);

/* tensor-core self-test (GB300 addition): d [128][n] = a [128][k] . b [n][k]^T
 * with BF16 a, b (raw 16-bit patterns, row-major) and FP32 d, computed by
 * one tcgen05 MMA tile; k, n multiples of 16 in [16, 128]; host buffers */
path_status path_debug_tc_gemm(const uint16_t *a, const uint16_t *b, uint32_t k, uint32_t n,
                               float *d);
/* The bounded wait of the tensor-core kernels, made to run out: the
 * self-test kernel issues no MMA, so nothing arrives on its mbarrier and
 * its wait gives up after `polls` polls; returns PATH_ERR_DEVICE_TIMEOUT
 * (the status a render or cache call returns when a wait gives up), after
 * which the device is usable as before. */
path_status path_debug_tc_wait_timeout(uint32_t polls);

/* ---- adjoint (GB300 addition; the reference has no derivatives) ---- */
/* Gradients of a loss of the rendered image with respect to each material's
 * parameters, by path replay: a streaming forward render of (spec, scene,
 * samples_per, settings), then the same paths re-run from their Sobol
 * indices, accumulating per vertex the radiance that flowed through it times
 * d log f / d(parameter).  d_image = dLoss/d(FloatRGB image), [y][x][3]
 * floats (device memory if d_image_on_device).  d_params receives, per
 * material, 7 doubles: d/d(reflectance r, g, b) (Diffuse albedo, GGX F0),
 * d/d(GGX roughness), d/d(emission r, g, b).  Sampling densities and the
 * light-selection table are held fixed (the detached estimator); other BSDF
 * types transport light but get zero reflectance / roughness gradients.
 * Square images and the 8-wide BVH only. */
path_status path_render_adjoint(path_renderer *renderer, const path_sample_spec *sample_spec,
                                const path_scene *scene, uint32_t samples_per,
                                const path_settings *settings, const float *d_image,
                                uint32_t d_image_on_device, double *d_params,
                                double *seconds);

/* ---- neural radiance cache (GB300 addition) ----
 * A multiresolution hash-grid encoding of position (16 levels x 2 features,
 * 2^19 entries per level) plus direction, normal and albedo feeds a BF16 MLP
 * (48 -> 64 x5 ReLU -> 3, no biases) run on the tcgen05 tensor cores with
 * FP32 accumulation; trained online with Adam on a relative L2 loss.
 * Query records: [n][12] floats (position, direction, normal, albedo);
 * training records: [n][16] floats (query, target radiance rgb, pad). */
typedef struct path_cache path_cache;
path_status path_cache_create(uint32_t seed, float learning_rate, path_cache **out);
void path_cache_destroy(path_cache *cache);
/* the scene box the hash grid covers */
path_status path_cache_set_bounds(path_cache *cache, const float *lo, const float *hi);
/* positions in batch-cell coordinates, as path_render_batch_cached sets them:
 * a position p of item i is (p - lo_i) / (hi_i - lo_i) (its scene's vertex
 * box onto [0, 1]^3) plus 2 * (i % 16, i / 16 % 16, i / 256); every cell has
 * grid vertices of its own.  path_cache_set_bounds returns to one scene box. */
path_status path_cache_use_batch_cells(path_cache *cache);
/* Inference (queries, cached renders) on an exponential moving average of
 * the weights and table, avg = decay avg + (1 - decay) param after every
 * Adam step, starting from the current parameters; decay in [0, 1), 0 (the
 * default) uses the parameters themselves. */
path_status path_cache_set_ema(path_cache *cache, float decay);
/* radiance [n][3] of n queries (host buffers) */
path_status path_cache_query(path_cache *cache, const float *queries, uint32_t n, float *out);
/* one training step on n records (host buffer): with apply_update 0 only the
 * gradients are computed (path_cache_access reads them); loss = mean
 * relative L2 loss before the step */
path_status path_cache_train(path_cache *cache, const float *records, uint32_t n,
                             uint32_t apply_update, float *loss);
/* copies weights [20480], table [16][2^19][2], and their gradients to the
 * host (set = 0) or weights and table from the host (set = 1); NULL skips */
path_status path_cache_access(path_cache *cache, float *weights, float *table,
                              float *grad_weights, float *grad_table, uint32_t set);

/* One frame of the render with the radiance cache: a streaming render whose
 * paths end into the cache at vertex cache_depth (the cache's prediction of
 * the radiance leaving that vertex, times the path throughput, replaces the
 * rest of the path), then train_steps Adam steps on train_paths records from
 * full-length training paths (each its vertex at cache_depth: its query and
 * the radiance the rest of its path carried back).  Square images, streaming
 * approach, 8-wide BVH. */
path_status path_render_cached(path_renderer *renderer, path_cache *cache,
                               const path_sample_spec *sample_spec, const path_output *output,
                               const path_scene *scene, uint32_t samples_per,
                               const path_settings *settings, uint32_t cache_depth,
                               uint32_t train_paths, uint32_t train_steps, double *seconds);

/* The queries of the last path_render_cached frame (for judging the cache's
 * bias): of every stride-th sample of the frame, those whose path ended into
 * the cache, at most max_n, in sample order -- queries [n][12] (position,
 * direction towards the previous vertex, shading normal, albedo: the
 * network's input record) and the path throughput there [n][3]; n_out
 * receives n.  Host buffers. */
path_status path_cache_frame_queries(const path_renderer *renderer, uint32_t max_n,
                                     uint32_t stride, float *queries, float *throughput,
                                     uint32_t *n_out);

/* ---- batched render (GB300 addition; the reference renders one scene per
 * call) ---- */
/* One image of a batch: a scene, its square-image camera, samples per pixel
 * and where the image goes (FLOAT_RGB or BGRA, host or device memory);
 * sample_offset: the image takes Sobol samples [sample_offset, sample_offset
 * + samples_per), as path_sample_spec.sample_offset (progressive frames). */
typedef struct {
  const path_scene *scene;
  uint32_t x_dim, y_dim;
  float film_to_world[12];
  uint32_t samples_per;
  path_output output;
  uint32_t sample_offset;
} path_batch_item;

/* Launch shape of a batched render.  Every choice gives the same images
 * (bit for bit); they only change speed.  Zero fields take the defaults in
 * brackets. */
typedef struct {
  uint32_t slots_log2;          /* paths in flight = 2^slots_log2, 10..26 [26] */
  uint32_t trace_min_blocks;    /* trace kernel variant, 3..6 [4] */
  uint32_t shade_ctas_per_sm;   /* shade grid = SMs x this [4] */
  uint32_t iterations_per_graph; /* trace/shade iterations per CUDA-graph
                                    launch between live-path checks [4] */
} path_batch_tuning;

/* Renders every item: all scenes' geometry in one device arena, all their
 * samples through one persistent wavefront (one trace and one shade launch
 * per iteration for the whole batch, replayed as a CUDA graph), then each
 * image summed per pixel in the reference's order, so each image equals the
 * single-scene streaming render of the same item.  Uses the streaming
 * approach and the 8-wide BVH whatever settings->kernel_approach says;
 * tuning may be NULL (defaults).  The scenes' BVHs are cached until a
 * scene's contents or the batch's scene list change. */
path_status path_render_batch(path_renderer *renderer, const path_batch_item *items,
                              uint32_t n_items, const path_settings *settings,
                              const path_batch_tuning *tuning, double *seconds);
/* One frame of every item with one radiance cache for the whole batch (the
 * cached form of path_render_batch; at most 4096 items): item i's positions
 * take cell i of the cache (path_cache_use_batch_cells), paths end into the
 * cache at vertex cache_depth as in path_render_cached, and train_steps Adam
 * steps follow on train_paths records, each traced from a random item. */
path_status path_render_batch_cached(path_renderer *renderer, path_cache *cache,
                                     const path_batch_item *items, uint32_t n_items,
                                     const path_settings *settings,
                                     const path_batch_tuning *tuning, uint32_t cache_depth,
                                     uint32_t train_paths, uint32_t train_steps,
                                     double *seconds);
/* Times candidate launch shapes on the batch's first samples (at most
 * sample_budget of them, 0 = 2^27; no image output) and returns the
 * fastest. */
path_status path_batch_autotune(path_renderer *renderer, const path_batch_item *items,
                                uint32_t n_items, const path_settings *settings,
                                uint64_t sample_budget, path_batch_tuning *out);

/* ---- accel / intersection (TriangleAccel concept,
 * include/intersect/accel/accel.h:35-77) ---- */
/* builds the SBVH of a world-space triangle soup (Generator::gen,
 * src/intersect/accel/sbvh/detail/generator.cu:17-66).  sizes receives
 * [n_nodes, n_extra_idxs]; the arrays may be NULL to query sizes. */
path_status path_sbvh_build(const float *triangles, uint32_t n,
                            const path_settings *settings, uint32_t *sizes,
                            uint32_t *node_words, float *node_aabbs,
                            uint32_t *extra_idxs, uint32_t *permutation);
/* The compressed 8-wide BVH the GPU traverses, collapsed from the SBVH the
 * same settings build (GB300 addition, no counterpart in the reference;
 * for inspection and tests).  sizes receives [n_nodes, n_leaf_refs, depth];
 * nodes = n_nodes records of 80 bytes (quantised child boxes, see
 * path_gb300/csrc/devtypes.h WideNode); leaf_refs = BVH-order triangle index
 * of every wide-leaf entry; permutation = BVH order -> input order.  The
 * arrays may be NULL to query sizes. */
path_status path_wide_build(const float *triangles, uint32_t n,
                            const path_settings *settings, uint32_t *sizes,
                            void *nodes, uint32_t *leaf_refs, uint32_t *permutation);
/* closest hit of each ray against the triangle soup on the GPU
 * (AccelRef::intersect_objects with Triangle::intersect): idx = original
 * triangle index or -1, t = distance (NaN when none).  rays/idx/t are host
 * pointers. */
path_status path_intersect(path_renderer *renderer, const float *triangles,
                           uint32_t n_triangles, const float *rays,
                           uint32_t n_rays, const path_settings *settings,
                           int32_t *idx_out, float *t_out);

/* ---- RNG ---- */
/* Sobol table vals[i * dimension_bound + d] on the GPU
 * (SobelSequenceGen::gen, src/rng/sobel/sobel.cu:21-93); out is host. */
path_status path_sobol_table(uint32_t dimension_bound, uint32_t count,
                             float *out);
/* the same table produced by cuRAND's own device generator
 * (curand_init + curand_uniform on curandStateScrambledSobol32), used to
 * pin the register-XOR generator bit for bit. */
path_status path_sobol_table_curand(uint32_t dimension_bound, uint32_t count,
                                    float *out);

/* ---- diagnostics ---- */
/* evaluates the kernels' transcendental functions on the GPU:
 * fn 0 sin, 1 cos, 2 asin, 3 acos, 4 pow(x, y); host arrays of n */
path_status path_debug_pmath(uint32_t fn, const float *x, const float *y,
                             float *out, uint32_t n);
/* Fault injection for the out-of-memory paths (GB300 addition; the
 * reference exits on a CUDA error, include/lib/cuda/utils.h:18-26): once the
 * device memory the library's renderers hold would exceed `bytes`, further
 * device allocations fail as a full device makes them fail, and the call
 * that needed them returns PATH_ERR_OOM with its message; the renderer stays
 * usable.  0 removes the cap.  Process-wide; for tests. */
void path_debug_set_device_alloc_cap(uint64_t bytes);

/* evaluates the kernels' BSDF code on the GPU for one material (GB300
 * addition, for tests): n records of 9 floats in `in` (host arrays);
 *   op 0: continuous_eval (bsdf::BSDF::continuous_eval, include/bsdf/bsdf.h
 *         :10-46), record = (incoming dir, outgoing dir, normal), out [n][3];
 *   op 1: continuous_sample (bsdf.h) drawing u0, u1, u2 in turn, record =
 *         (incoming dir, normal, u0, u1, u2), out [n][6] = (dir, multiplier);
 *   op 2: the GGX normal distribution D, record = (n.h, alpha, unused),
 *         out [n]. */
path_status path_debug_bsdf(const path_material *material, uint32_t op, const float *in,
                            uint32_t n, float *out);
/* The cost of the render's Sobol draws (GB300 addition, a measurement):
 * n_paths paths of `draws` consecutive dimensions each (sample index p mod
 * spp, first dimension as a pixel's, 256 dimensions), summed per path;
 * mode 0 reads the values from the table the integrator uses
 * (rng_from_sequence_gen.h:45-54), mode 1 forms each from the direction
 * vectors XOR-ed in a register (vectors read through L1), mode 2 the same
 * with the vectors in shared memory.  ms receives the kernel time of one
 * launch (mean of 3 after a warm-up), checksum a hash of the sums, equal
 * across the modes. */
path_status path_debug_sobol_draws(uint32_t mode, uint32_t n_paths, uint32_t spp,
                                   uint32_t draws, float *ms, uint32_t *checksum);
/* kernel::WorkDivision (src/kernel/work_division.cpp:12-69): out receives
 * [block_size, base_samples_per_thread, n_threads_per_unit_extra,
 *  sample_block_size, x_block_size, y_block_size, num_sample_blocks,
 *  num_x_blocks, num_y_blocks, x_dim, y_dim] */
path_status path_work_division(const path_work_division_settings *settings,
                               uint32_t samples_per, uint32_t x_dim,
                               uint32_t y_dim, uint32_t *out);
/* number of GPUs visible and the library's build string */
const char *path_version(void);

/* ---- render without device allocation (no counterpart in the reference) ----
 * Some callers cannot call cudaMalloc: a host framework that owns all device
 * memory through its own allocator and forbids raw allocations, or a real-time
 * loop that must not allocate after start-up because cudaMalloc / cudaFree can
 * synchronise the whole device.  path_render_noalloc renders like path_render
 * but allocates nothing: its scratch (the status word, work counters and the
 * per-sample-block partial sums with their reduction buffer) lives in one
 * file-scope device array of PATH_NOALLOC_SCRATCH_BYTES that every GPU loading
 * the library holds until the process exits.  Requirements:
 *   - the scene is already resident on this renderer: an earlier path_render
 *     with the same scene, SBVH settings, max_sample_size and samples_per;
 *   - output->on_device is set (the image is written to caller device memory);
 *   - partial sums that do not fit the array are rejected with
 *     PATH_ERR_ARGUMENT (the message gives the bytes needed).
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture
 * begins.  All calls share the one array: calls whose GPU work overlaps in
 * time race on it, so issue them one after another. */
#define PATH_NOALLOC_SCRATCH_BYTES (32u << 20)
path_status path_render_noalloc(path_renderer *renderer,
                                const path_sample_spec *sample_spec,
                                const path_output *output,
                                const path_scene *scene, uint32_t samples_per,
                                const path_settings *settings, double *seconds);

#ifdef __cplusplus
}
#endif

#endif /* PATH_GB300_H */

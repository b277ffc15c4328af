// render::Renderer for the GPU execution model (host side).
//
// Owns a CUDA stream and device buffers, and caches the uploaded scene
// (flattened triangles, SBVH, wide BVH, materials, light table) and the
// Sobol table across calls, as Renderer::Impl caches its generators and
// vectors (include/render/detail/renderer_impl.h:42-96).
#pragma once

#include "kernels.h"
#include "scene.h"
#include "sbvh.h"
#include "wide.h"

#include <cuda_runtime.h>

#include <array>
#include <string>
#include <utility>
#include <vector>

namespace pg {

// Fault injection for the out-of-memory paths (path_debug_set_device_alloc_cap):
// once the device memory DeviceBuffers hold would exceed `bytes` (0 = no cap),
// further allocations fail as cudaMalloc does when the device is full.
void set_device_alloc_cap(uint64_t bytes);

class DeviceBuffer {
public:
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  ~DeviceBuffer() { release(); }
  cudaError_t ensure(size_t bytes);
  cudaError_t upload(const void *src, size_t bytes, cudaStream_t s);
  void release();
  void swap(DeviceBuffer &o) {
    std::swap(ptr_, o.ptr_);
    std::swap(size_, o.size_);
  }
  void *get() const { return ptr_; }
  template <typename T> T *as() const { return static_cast<T *>(ptr_); }
  size_t size() const { return size_; }

private:
  void *ptr_ = nullptr;
  size_t size_ = 0;
};

// page-locked host staging buffer (fast host -> device copies)
class PinnedBuffer {
public:
  PinnedBuffer() = default;
  PinnedBuffer(const PinnedBuffer &) = delete;
  PinnedBuffer &operator=(const PinnedBuffer &) = delete;
  ~PinnedBuffer() { release(); }
  cudaError_t ensure(size_t bytes);
  void release();
  void *get() const { return ptr_; }
  template <typename T> T *as() const { return static_cast<T *>(ptr_); }
  size_t bytes = 0; // bytes in use

private:
  void *ptr_ = nullptr;
  size_t cap_ = 0;
};

struct Status {
  path_status code = PATH_OK;
  std::string message;
  static Status ok() { return {}; }
  static Status err(path_status c, std::string m) { return {c, std::move(m)}; }
  bool good() const { return code == PATH_OK; }
};

Status cuda_status(cudaError_t e, const char *what);

// host copies of the scene's device arrays (kept for tests and reuse)
struct PreparedScene {
  uint64_t scene_id = 0, scene_version = 0, material_version = 0;
  SBVHSettings sbvh;
  bool valid = false;
  BinaryBVH bvh;
  WideBVH wide;
  std::vector<uint32_t> orig_to_bvh; // inverse of bvh.permutation
  uint32_t gpu_built = 0;            // wide BVH from the GPU builder (path_settings.gpu_build
                                     // mode; no binary BVH), 0 = host SBVH
  uint32_t n_wide_nodes = 0;
  float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f}; // scene box
  uint32_t n_tris = 0, n_lights = 0;
  double build_seconds = 0.0;
};

// device form of a material (UnionBSDF parameters + precomputed values)
DevMaterial to_dev(const path_material &m);
// triangle as (v0, e1 = v1 - v0, e2 = v2 - v0) in 12 floats; extra_bits in
// float 10
void put_tri(float *dst, f3 v0, f3 v1, f3 v2, uint32_t extra_bits);
// settings every render accepts (enum ranges, supported RNG, bounds)
Status check_settings(const path_settings &s);

// box of all vertices of a flattened scene
void scene_box(const FlatScene &flat, float *lo, float *hi);

// one image of a batched render (path_batch_item)
struct BatchItem {
  const Scene *scene;
  uint32_t x_dim, y_dim, spp;
  uint32_t sample_offset = 0; // Sobol samples [sample_offset, sample_offset + spp)
  float f2w[12];
  path_output output;
};

// geometry of a batch's scenes, concatenated on the device
struct PreparedBatch {
  bool valid = false;
  std::vector<std::array<uint64_t, 3>> key; // (scene id, version, material version)
  SBVHSettings sbvh;
  uint32_t gpu_build = 0;
  std::vector<uint32_t> root, light_off, n_lights, n_tris;
  std::vector<std::array<float, 6>> box; // per item: its scene's vertex box (lo, hi)
  uint32_t n_wide_nodes = 0;
  uint64_t total_tris = 0;
  double build_seconds = 0.0;
};

class Renderer {
public:
  Renderer();
  ~Renderer();

  Status render(const path_sample_spec &spec, const path_output &output,
                const Scene &scene, uint32_t spp, const path_settings &settings,
                double *seconds);
  Status intersect(const float *tris, uint32_t n_tris, const float *rays,
                   uint32_t n_rays, const path_settings &settings, int32_t *idx,
                   float *t);
  const path_render_stats &stats() const { return stats_; }
  // adjoint of the streaming render: parameter gradients for dLoss/dImage
  Status render_adjoint(const path_sample_spec &spec, const Scene &scene, uint32_t spp,
                        const path_settings &settings, const float *d_image,
                        bool d_image_on_device, double *d_params, double *seconds);
  // one frame with the radiance cache (render, then train it)
  Status render_cached(const path_sample_spec &spec, const path_output &output,
                       const Scene &scene, uint32_t spp, const path_settings &settings,
                       class RadianceCache &cache, uint32_t cache_depth, uint32_t train_paths,
                       uint32_t train_steps, double *seconds);
  // every stride-th sample of the last cached frame whose path ended into
  // the cache: its query [12] and throughput [3] (at most max_n of them)
  Status cached_frame_queries(uint32_t max_n, uint32_t stride, float *queries,
                              float *throughput, uint32_t *n_out) const;
  // batched render and its launch-shape autotuner (defined in batch.cpp)
  Status render_batch(const std::vector<BatchItem> &items, const path_settings &settings,
                      const path_batch_tuning *tuning, double *seconds);
  Status autotune_batch(const std::vector<BatchItem> &items, const path_settings &settings,
                        uint64_t sample_budget, path_batch_tuning *out);
  // one frame of every item with one radiance cache for the whole batch
  // (item i in cell i of it), then train_steps Adam steps on train_paths
  // records traced from random items
  Status render_batch_cached(const std::vector<BatchItem> &items, const path_settings &settings,
                             const path_batch_tuning *tuning, class RadianceCache &cache,
                             uint32_t cache_depth, uint32_t train_paths, uint32_t train_steps,
                             double *seconds);
  // render that allocates nothing; scratch is device memory the caller owns
  // (defined in noalloc.cu)
  Status render_noalloc(const path_sample_spec &spec, const path_output &output,
                        const Scene &scene, uint32_t spp, const path_settings &settings,
                        void *scratch, size_t scratch_bytes, double *seconds);

private:
  Status init();
  Status prepare_scene(const FlatScene &flat, uint64_t id, uint64_t version,
                       const SBVHSettings &sbvh, bool force);
  Status upload_geometry(const FlatScene &flat, const std::vector<path_material> &mats);
  Status copy_staged(uint64_t *bytes, bool all, uint32_t traversal);
  void stage_materials(const FlatScene &flat, const std::vector<path_material> &mats);
  Status refresh_materials(const Scene &scene, uint64_t *bytes);
  Status prepare_scene_gpu(const FlatScene &flat, uint64_t id, uint64_t version,
                           const std::vector<path_material> &mats, uint32_t mode);
  Status prepare_sobol(uint32_t dim_bound, uint32_t count);
  void fill_params(RenderParams &p) const;
  Status traversal_fits(const path_settings &st) const;

  bool initialised_ = false;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev_start_ = nullptr, ev_stop_ = nullptr;
  std::vector<cudaEvent_t> trace_ev_; // event pairs around streaming trace launches
  uint32_t trace_timed_ = 0, trace_launches_ = 0;
  PreparedScene prep_;
  DeviceBuffer tris_, tri_data_, bin_nodes_, extra_, wide_nodes_, wide_tris_,
      materials_, light_tris_, light_cdf_, perm_;
  // pinned host copies of the device arrays above, in the same order
  PinnedBuffer st_tris_, st_data_, st_nodes_, st_extra_, st_wnodes_, st_wtris_, st_mats_,
      st_lights_, st_cdf_, st_perm_;
  DeviceBuffer sobol_dirs_, sobol_table_; // dirs: vectors, then scramble constants
  uint32_t sobol_bound_ = 0, sobol_count_ = 0;
  DeviceBuffer out_a_, out_b_, bgra_, status_, counters_, rays_, idxs_;
  // wavefront state
  struct AdjointState {
    const float *d_image;
    double *d_params;
  };
  Status run_wavefront(const RenderParams &p, uint32_t n_blocks, bool counting,
                       uint32_t min_blocks, bool time_trace, uint32_t *launches,
                       const AdjointState *adj = nullptr);
  RenderParams last_params_{};
  uint32_t slots_log2_ = 21; // paths in flight of the streaming render, log2
  uint32_t mat_types_ = kFeatAllMats; // BSDF types of the resident scene (bit per type)
  uint32_t b_mat_types_ = kFeatAllMats; // ... of the resident batch
  class RadianceCache *cache_ = nullptr; // set during a cached render
  uint32_t cache_depth_ = 0;
  uint32_t frame_counter_ = 0;
  uint64_t cached_samples_ = 0; // samples of the last cached frame (cache_q_, cache_beta_)
  // cached render: training paths traced on a side stream while the frame
  // renders (cache_train_paths_ > 0 asks render() to launch them)
  uint32_t cache_train_paths_ = 0;
  cudaStream_t side_stream_ = nullptr;
  cudaEvent_t side_done_ = nullptr;
  DeviceBuffer cache_q_, cache_beta_, cache_pred_, cache_records_;
  uint32_t last_blocks_ = 0;
  DeviceBuffer adj_image_, adj_dimage_, adj_params_, adj_pend_;
  cudaEvent_t trace_event(size_t i);
  DeviceBuffer wf_slots_, wf_queues_, wf_samples_, wf_rng_;
  PinnedBuffer wf_host_;
  int num_sms_ = 0;
  path_render_stats stats_{};
  // batched render
  Status check_batch(const std::vector<BatchItem> &items, const path_settings &st) const;
  Status prepare_batch(const std::vector<BatchItem> &items, const SBVHSettings &sb,
                       uint32_t gpu_build);
  Status run_batch(const std::vector<BatchItem> &items, const path_settings &st,
                   const path_batch_tuning &tu, uint64_t sample_limit, bool with_images,
                   float *kernel_ms, uint32_t *launches);
  PreparedBatch batch_;
  DeviceBuffer b_wnodes_, b_wtris_, b_tris_, b_data_, b_mats_, b_lights_, b_cdf_, b_scenes_,
      b_part_a_, b_part_b_, b_bgra_;
};

} // namespace pg

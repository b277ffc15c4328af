// Render entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: a host framework that owns all device
// memory through its own allocator and forbids raw allocations, or a
// real-time loop that must not allocate after start-up because cudaMalloc /
// cudaFree can synchronise the whole device.  path_render_noalloc serves
// them: the scene must already be resident on the renderer (an earlier
// path_render with the same scene and settings uploaded it), the caller
// passes the output as device memory, and every scratch buffer the render
// needs -- the device status word, the work counters, the per-sample-block
// partial sums and the reduction's second buffer -- is carved out of the
// file-scope array below.
//
// The array is PATH_NOALLOC_SCRATCH_BYTES (32 MiB) on every GPU that loads
// the library, held until the process exits.  Its device address is looked
// up once per device, with that device current, by the first call made on
// that device (cudaGetSymbolAddress); that first call should come before
// any stream capture begins.  The cached address belongs to the device's
// current context: like the renderer's own device buffers and stream it
// does not survive cudaDeviceReset, so a process that resets a device must
// not call this entry point on that device afterwards.  All calls share the
// array and it keeps the last call's contents: the status word and counters
// are cleared by every call, and calls whose GPU work overlaps in time race
// on the array.
#include "kernels.h"
#include "renderer.h"

#include <cuda_runtime.h>

#include <chrono>
#include <cstring>
#include <mutex>

namespace pg {

path_status record_status(const Status &s);
Renderer &renderer_of(path_renderer *r);
const Scene &scene_of(const path_scene *s);

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[PATH_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void *g_scratch_addr[kMaxDevices] = {};

// device address of the scratch array on the current device
Status scratch_address(void **out) {
  int dev = 0;
  Status st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
  if (!st.good()) {
    return st;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    return Status::err(PATH_ERR_UNSUPPORTED, "device ordinal beyond 64");
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_addr[dev] == nullptr) {
    void *p = nullptr;
    st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                     "cudaGetSymbolAddress(no-allocation scratch)");
    if (!st.good()) {
      return st;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return Status::ok();
}

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

} // namespace

Status Renderer::render_noalloc(const path_sample_spec &spec, const path_output &output,
                                const Scene &scene, uint32_t spp, const path_settings &st,
                                void *scratch, size_t scratch_bytes, double *seconds) {
  if (spec.type != PATH_SAMPLE_SQUARE_IMAGE || spec.row_start != 0 || spec.row_end != 0 ||
      spec.x_dim == 0 || spec.y_dim == 0 ||
      spp == 0) {
    return Status::err(PATH_ERR_ARGUMENT, "a square image with positive size and spp is needed");
  }
  if (output.data == nullptr || !output.on_device ||
      (output.type != PATH_OUTPUT_BGRA && output.type != PATH_OUTPUT_FLOAT_RGB)) {
    return Status::err(PATH_ERR_ARGUMENT, "the output must be device memory (on_device = 1)");
  }
  if (st.rng > PATH_RNG_UNIFORM || st.traversal > PATH_TRAVERSAL_WIDE8 ||
      st.target_objects == 0 || st.target_objects > 10) {
    return Status::err(PATH_ERR_ARGUMENT, "unsupported settings");
  }
  if (!initialised_ || !prep_.valid || prep_.scene_id != scene.id ||
      prep_.scene_version != scene.version ||
      prep_.material_version != scene.material_version ||
      prep_.sbvh.overlap_threshold != st.overlap_threshold ||
      prep_.sbvh.use_spatial_splits != (st.use_spatial_splits != 0) ||
      prep_.sbvh.traversal_per_intersect_cost != st.traversal_per_intersect_cost ||
      prep_.sbvh.target_objects != st.target_objects ||
      prep_.gpu_built != st.gpu_build) {
    return Status::err(PATH_ERR_ARGUMENT,
                       "scene not resident on this renderer: render it once with path_render");
  }
  if (st.rng == PATH_RNG_SOBEL &&
      (sobol_bound_ != st.max_sample_size ||
       sobol_count_ < (uint64_t)spec.sample_offset + spp || !sobol_table_.get())) {
    return Status::err(PATH_ERR_ARGUMENT,
                       "Sobol table for this max_sample_size / sample_offset + samples_per "
                       "not resident: render once with path_render");
  }
  Status sf = traversal_fits(st);
  if (!sf.good()) {
    return sf;
  }
  WorkDiv wd;
  if (!make_workdiv(st.render_work_division, spp, spec.x_dim, spec.y_dim, wd) ||
      wd.block_size > 256) {
    return Status::err(PATH_ERR_ARGUMENT, "invalid render work division settings");
  }
  const size_t n_pix = (size_t)spec.x_dim * spec.y_dim;
  const bool bgra = output.type == PATH_OUTPUT_BGRA;
  const uint32_t nsb = wd.num_sample_blocks;
  // scratch layout: [status | counters] [partials A] [partials B]
  const size_t head = 256;
  const size_t part = (bgra || nsb > 1) ? align256((size_t)nsb * n_pix * 12) : 0;
  const size_t need = head + part + (nsb > 1 ? part : 0);
  if (need > scratch_bytes) {
    return Status::err(PATH_ERR_ARGUMENT,
                       "render needs " + std::to_string(need) + " bytes of scratch, above the " +
                           std::to_string(scratch_bytes) + "-byte no-allocation array");
  }
  unsigned char *base = static_cast<unsigned char *>(scratch);
  uint32_t *status = reinterpret_cast<uint32_t *>(base);
  unsigned long long *counters = reinterpret_cast<unsigned long long *>(base + 64);
  float *part_a = reinterpret_cast<float *>(base + head);
  float *part_b = reinterpret_cast<float *>(base + head + part);
  cudaError_t e = cudaMemsetAsync(base, 0, head, stream_);
  if (e != cudaSuccess) {
    return cuda_status(e, "scratch clear");
  }

  RenderParams p;
  fill_params(p);
  p.status = status;
  p.counters = counters;
  p.sobol = sobol_table_.as<const float>();
  p.sobol_vec = sobol_dirs_.as<const uint32_t>();
  p.dim_bound = st.max_sample_size;
  p.init_dim_bound = std::min(64u, st.max_sample_size);
  p.light_sampler = st.light_sampler;
  p.dir_sampler = st.dir_sampler;
  p.term_prob = st.term_prob;
  p.term_iters = st.term_prob_iters;
  p.term_prob_prob = st.term_prob_prob;
  p.term_exp = st.term_prob_exp;
  p.term_min_prob = st.term_prob_min_prob;
  p.back_cull = st.back_cull_emission;
  p.target_objects = st.target_objects;
  p.rng_uniform = st.rng == PATH_RNG_UNIFORM ? 1u : 0u;
  std::memcpy(p.f2w, spec.film_to_world, sizeof(p.f2w));
  p.x_dim = spec.x_dim;
  p.y_dim = spec.y_dim;
  p.spp = spp;
  p.sample_offset = spec.sample_offset;
  p.wd = wd;
  const bool direct = !bgra && nsb == 1;
  p.out_rgb = direct ? static_cast<float *>(output.data) : part_a;
  p.out_bgra = bgra ? static_cast<uint8_t *>(output.data) : nullptr;
  p.output_bgra = bgra ? 1 : 0;
  p.start_block = 0;
  p.row_lo = 0;
  p.row_hi = spec.y_dim;

  auto t0 = std::chrono::steady_clock::now();
  uint32_t launches = 0;
  if ((e = cudaEventRecord(ev_start_, stream_)) != cudaSuccess ||
      (e = launch_render(p, st.traversal, wd.total_blocks(), st.count_work != 0, stream_)) !=
          cudaSuccess) {
    return cuda_status(e, "render kernel");
  }
  ++launches;
  uint32_t factor = nsb;
  float *in = p.out_rgb, *other = part_b;
  size_t elems = (size_t)nsb * n_pix;
  while (factor != 1) {
    ReduceParams rp;
    std::memset(&rp, 0, sizeof(rp));
    uint32_t xd = (uint32_t)(elems / factor);
    if (!make_workdiv(st.reduce_work_division, factor, xd, 1, rp.wd)) {
      return Status::err(PATH_ERR_ARGUMENT, "invalid reduce work division settings");
    }
    rp.in = in;
    rp.out = other;
    rp.reduction_factor = factor;
    rp.spp = spp;
    rp.output_bgra = bgra ? 1 : 0;
    rp.out_bgra = p.out_bgra;
    if ((e = launch_reduce(rp, stream_)) != cudaSuccess) {
      return cuda_status(e, "reduce kernel");
    }
    ++launches;
    factor = rp.wd.num_sample_blocks;
    elems = (size_t)xd * factor;
    std::swap(in, other);
  }
  if ((e = cudaEventRecord(ev_stop_, stream_)) != cudaSuccess) {
    return cuda_status(e, "event");
  }
  if (!bgra && in != output.data &&
      (e = cudaMemcpyAsync(output.data, in, n_pix * 12, cudaMemcpyDeviceToDevice, stream_)) !=
          cudaSuccess) {
    return cuda_status(e, "output copy");
  }
  uint32_t dev_status = 0;
  unsigned long long counts[3] = {0, 0, 0};
  if ((e = cudaMemcpyAsync(&dev_status, status, 4, cudaMemcpyDeviceToHost, stream_)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(counts, counters, 24, cudaMemcpyDeviceToHost, stream_)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(stream_)) != cudaSuccess) {
    return cuda_status(e, "status read");
  }
  auto t1 = std::chrono::steady_clock::now();
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev_start_, ev_stop_);
  stats_ = path_render_stats{};
  stats_.seconds = std::chrono::duration<double>(t1 - t0).count();
  stats_.kernel_ms = ms;
  stats_.bvh_build_seconds = prep_.build_seconds;
  stats_.rays_traced = counts[0];
  stats_.nodes_visited = counts[1];
  stats_.triangles_tested = counts[2];
  stats_.gpu_launches = launches;
  stats_.device_status = dev_status;
  stats_.num_bvh_nodes = (uint32_t)prep_.bvh.nodes.size();
  stats_.num_wide_nodes = prep_.n_wide_nodes;
  if (seconds) {
    *seconds = stats_.seconds;
  }
  if (dev_status != 0) {
    return Status::err(PATH_ERR_DEVICE_TIMEOUT,
                       "kernel reported device status " + std::to_string(dev_status));
  }
  return Status::ok();
}

} // namespace pg

extern "C" path_status path_render_noalloc(path_renderer *renderer,
                                           const path_sample_spec *sample_spec,
                                           const path_output *output, const path_scene *scene,
                                           uint32_t samples_per, const path_settings *settings,
                                           double *seconds) {
  if (!renderer || !sample_spec || !output || !scene || !settings) {
    return pg::record_status(pg::Status::err(PATH_ERR_ARGUMENT, "null argument"));
  }
  void *scratch = nullptr;
  pg::Status st = pg::scratch_address(&scratch);
  if (st.good()) {
    st = pg::renderer_of(renderer).render_noalloc(*sample_spec, *output, pg::scene_of(scene),
                                                  samples_per, *settings, scratch,
                                                  PATH_NOALLOC_SCRATCH_BYTES, seconds);
  }
  return pg::record_status(st);
}

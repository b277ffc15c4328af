// render::Renderer for the GPU execution model (see renderer.h).
#include "renderer.h"
#include "cache_host.h"
#include "gpu_build.h"

#include <curand.h>

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>

namespace pg {

namespace {
// allocation cap for fault injection (path_debug_set_device_alloc_cap): the
// bytes every DeviceBuffer holds, and the cap (0 = none)
std::atomic<uint64_t> g_device_bytes{0};
std::atomic<uint64_t> g_device_cap{0};
} // namespace

void set_device_alloc_cap(uint64_t bytes) { g_device_cap.store(bytes); }

cudaError_t DeviceBuffer::ensure(size_t bytes) {
  if (bytes <= size_ && ptr_ != nullptr) {
    return cudaSuccess;
  }
  release();
  if (bytes == 0) {
    return cudaSuccess;
  }
  const uint64_t cap = g_device_cap.load();
  if (cap != 0 && g_device_bytes.load() + bytes > cap) {
    // the allocation a capped device would refuse, refused on the host
    return cudaErrorMemoryAllocation;
  }
  cudaError_t e = cudaMalloc(&ptr_, bytes);
  if (e != cudaSuccess) {
    ptr_ = nullptr;
    size_ = 0;
    return e;
  }
  size_ = bytes;
  g_device_bytes.fetch_add(bytes);
  return cudaSuccess;
}

cudaError_t DeviceBuffer::upload(const void *src, size_t bytes, cudaStream_t s) {
  cudaError_t e = ensure(bytes);
  if (e != cudaSuccess || bytes == 0) {
    return e;
  }
  return cudaMemcpyAsync(ptr_, src, bytes, cudaMemcpyHostToDevice, s);
}

void DeviceBuffer::release() {
  if (ptr_ != nullptr) {
    cudaFree(ptr_);
    g_device_bytes.fetch_sub(size_);
  }
  ptr_ = nullptr;
  size_ = 0;
}

cudaError_t PinnedBuffer::ensure(size_t n) {
  bytes = n;
  if (n <= cap_ && ptr_ != nullptr) {
    return cudaSuccess;
  }
  release();
  bytes = n;
  if (n == 0) {
    return cudaSuccess;
  }
  cudaError_t e = cudaMallocHost(&ptr_, n);
  if (e != cudaSuccess) {
    ptr_ = nullptr;
    cap_ = 0;
    bytes = 0;
    return e;
  }
  cap_ = n;
  return cudaSuccess;
}

void PinnedBuffer::release() {
  if (ptr_ != nullptr) {
    cudaFreeHost(ptr_);
  }
  ptr_ = nullptr;
  cap_ = 0;
  bytes = 0;
}

Status cuda_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) {
    return Status::ok();
  }
  path_status code = e == cudaErrorMemoryAllocation ? PATH_ERR_OOM : PATH_ERR_CUDA;
  return Status::err(code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define PG_TRY_CUDA(expr, what)                                                \
  do {                                                                         \
    Status st_ = cuda_status((expr), what);                                    \
    if (!st_.good()) {                                                         \
      return st_;                                                              \
    }                                                                          \
  } while (0)

Renderer::Renderer() = default;

Renderer::~Renderer() {
  if (initialised_) {
    cudaStreamSynchronize(stream_);
    cudaEventDestroy(ev_start_);
    cudaEventDestroy(ev_stop_);
    for (cudaEvent_t e : trace_ev_) {
      cudaEventDestroy(e);
    }
    cudaStreamDestroy(stream_);
    if (side_stream_ != nullptr) {
      cudaStreamSynchronize(side_stream_);
      cudaEventDestroy(side_done_);
      cudaStreamDestroy(side_stream_);
    }
  }
}

Status Renderer::init() {
  if (initialised_) {
    return Status::ok();
  }
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    return Status::err(PATH_ERR_CUDA, std::string("no CUDA device available: ") +
                                          cudaGetErrorString(e));
  }
  PG_TRY_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
  PG_TRY_CUDA(cudaEventCreate(&ev_start_), "event");
  PG_TRY_CUDA(cudaEventCreate(&ev_stop_), "event");
  initialised_ = true;
  return Status::ok();
}

DevMaterial to_dev(const path_material &m) {
  DevMaterial d;
  std::memset(&d, 0, sizeof(d));
  d.type = m.type;
  for (int i = 0; i < 3; ++i) {
    d.diffuse[i] = m.diffuse[i];
    d.specular[i] = m.specular[i];
    d.emission[i] = m.emission[i];
  }
  d.shininess = m.shininess;
  d.ior = m.ior;
  d.w_d = m.diffuse_weight;
  d.w_g = m.glossy_weight;
  d.roughness = m.roughness;
  d.glossy_norm = (m.shininess + 2.f) / (2.f * (float)M_PI);
  d.inv_shininess_p1 = 1.f / (m.shininess + 1.f);
  float r0 = (m.ior - 1) / (m.ior + 1);
  d.r0 = r0 * r0;
  d.cont_inclusive0 = m.diffuse_weight / (m.diffuse_weight + m.glossy_weight);
  return d;
}

void put_tri(float *dst, f3 v0, f3 v1, f3 v2, uint32_t extra_bits) {
  f3 e1 = v1 - v0, e2 = v2 - v0;
  float vals[12] = {v0.x, v0.y, v0.z, e1.x, e1.y, e1.z, e2.x, e2.y, e2.z, 0.f, 0.f, 0.f};
  std::memcpy(&vals[10], &extra_bits, sizeof(extra_bits));
  std::memcpy(dst, vals, sizeof(vals));
}

Status Renderer::upload_geometry(const FlatScene &flat,
                                 const std::vector<path_material> &mats) {
  const BinaryBVH &bvh = prep_.bvh;
  const WideBVH &wide = prep_.wide;
  const size_t n = flat.v0.size();
  PG_TRY_CUDA(st_tris_.ensure(n * 48), "staging");
  PG_TRY_CUDA(st_data_.ensure(n * 48), "staging");
  PG_TRY_CUDA(st_nodes_.ensure(bvh.nodes.size() * 32), "staging");
  PG_TRY_CUDA(st_extra_.ensure(bvh.extra_idxs.size() * 4), "staging");
  PG_TRY_CUDA(st_wnodes_.ensure(wide.nodes.size() * sizeof(WideNode)), "staging");
  PG_TRY_CUDA(st_wtris_.ensure(wide.tri_index.size() * 48), "staging");
  PG_TRY_CUDA(st_mats_.ensure(mats.size() * sizeof(DevMaterial)), "staging");
  PG_TRY_CUDA(st_lights_.ensure(flat.light_v0.size() * 48), "staging");
  PG_TRY_CUDA(st_cdf_.ensure(flat.light_cdf.size() * 4), "staging");
  PG_TRY_CUDA(st_perm_.ensure(bvh.permutation.size() * 4), "staging");
  float *tris = st_tris_.as<float>();
  float *data = st_data_.as<float>();
  for (size_t i = 0; i < n; ++i) {
    uint32_t o = bvh.permutation[i];
    put_tri(&tris[12 * i], flat.v0[o], flat.v1[o], flat.v2[o], 0);
    float d[12] = {flat.n0[o].x, flat.n0[o].y, flat.n0[o].z, flat.n1[o].x,
                   flat.n1[o].y, flat.n1[o].z, flat.n2[o].x, flat.n2[o].y,
                   flat.n2[o].z, 0.f, 0.f, 0.f};
    std::memcpy(&d[11], &flat.material[o], sizeof(uint32_t));
    std::memcpy(&data[12 * i], d, sizeof(d));
  }
  uint32_t *nodes = st_nodes_.as<uint32_t>();
  for (size_t i = 0; i < bvh.nodes.size(); ++i) {
    const BinaryNode &b = bvh.nodes[i];
    float bx[6] = {b.aabb.lo.x, b.aabb.lo.y, b.aabb.lo.z,
                   b.aabb.hi.x, b.aabb.hi.y, b.aabb.hi.z};
    nodes[8 * i] = b.w0;
    nodes[8 * i + 1] = b.w1;
    std::memcpy(&nodes[8 * i + 2], bx, sizeof(bx));
  }
  if (!bvh.extra_idxs.empty()) {
    std::memcpy(st_extra_.get(), bvh.extra_idxs.data(), bvh.extra_idxs.size() * 4);
  }
  if (!wide.nodes.empty()) {
    std::memcpy(st_wnodes_.get(), wide.nodes.data(), wide.nodes.size() * sizeof(WideNode));
  }
  float *wtris = st_wtris_.as<float>();
  for (size_t k = 0; k < wide.tri_index.size(); ++k) {
    uint32_t b = wide.tri_index[k];
    uint32_t o = bvh.permutation[b];
    put_tri(&wtris[12 * k], flat.v0[o], flat.v1[o], flat.v2[o], 0);
    std::memcpy(&wtris[12 * k + 9], &b, sizeof(b));
  }
  stage_materials(flat, mats);
  if (!bvh.permutation.empty()) {
    std::memcpy(st_perm_.get(), bvh.permutation.data(), bvh.permutation.size() * 4);
  }
  uint64_t bytes = 0;
  Status sc = copy_staged(&bytes, true, PATH_TRAVERSAL_WIDE8);
  if (!sc.good()) {
    return sc;
  }
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "upload sync");
  prep_.n_tris = (uint32_t)n;
  prep_.n_lights = (uint32_t)flat.light_v0.size();
  return Status::ok();
}

// box of all vertices (the radiance cache and the GPU builder use it)
void scene_box(const FlatScene &flat, float *lo, float *hi) {
  box b = empty_box();
  for (size_t i = 0; i < flat.v0.size(); ++i) {
    b = grow(grow(grow(b, flat.v0[i]), flat.v1[i]), flat.v2[i]);
  }
  if (flat.v0.empty()) {
    b.lo = mk(0.f, 0.f, 0.f);
    b.hi = mk(0.f, 0.f, 0.f);
  }
  lo[0] = b.lo.x;
  lo[1] = b.lo.y;
  lo[2] = b.lo.z;
  hi[0] = b.hi.x;
  hi[1] = b.hi.y;
  hi[2] = b.hi.z;
}

// The 8-wide BVH from the GPU builder; the BVH-order triangle and shading
// arrays are gathered on the host with its permutation, as for the SBVH.
Status Renderer::prepare_scene_gpu(const FlatScene &flat, uint64_t id, uint64_t version,
                                   const std::vector<path_material> &mats, uint32_t mode) {
  prep_.valid = false;
  auto t0 = std::chrono::steady_clock::now();
  const size_t n = flat.v0.size();
  scene_box(flat, prep_.lo, prep_.hi);
  std::vector<float> t9(n * 9);
  for (size_t i = 0; i < n; ++i) {
    const f3 v[3] = {flat.v0[i], flat.v1[i], flat.v2[i]};
    for (int k = 0; k < 3; ++k) {
      t9[9 * i + 3 * k] = v[k].x;
      t9[9 * i + 3 * k + 1] = v[k].y;
      t9[9 * i + 3 * k + 2] = v[k].z;
    }
  }
  DeviceBuffer d9;
  PG_TRY_CUDA(d9.upload(t9.data(), t9.size() * 4, stream_), "gpu build upload");
  GpuWideBVH g;
  Status sb = gpu_build_wide(d9.as<float>(), (uint32_t)n, prep_.lo, prep_.hi, mode == 2, stream_,
                             g);
  if (!sb.good()) {
    return sb;
  }
  prep_.bvh = BinaryBVH{};
  prep_.bvh.permutation.resize(n);
  if (n > 0) {
    PG_TRY_CUDA(cudaMemcpyAsync(prep_.bvh.permutation.data(), g.perm.get(), n * 4,
                                cudaMemcpyDeviceToHost, stream_),
                "gpu build permutation");
  }
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "gpu build");
  prep_.wide = WideBVH{};
  prep_.wide.depth = g.depth;
  prep_.n_wide_nodes = g.n_nodes;
  wide_nodes_.swap(g.nodes);
  wide_tris_.swap(g.wide_tris);
  prep_.orig_to_bvh.assign(n, 0u);
  for (size_t i = 0; i < n; ++i) {
    prep_.orig_to_bvh[prep_.bvh.permutation[i]] = (uint32_t)i;
  }
  prep_.build_seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  prep_.scene_id = id;
  prep_.scene_version = version;
  prep_.gpu_built = mode;
  // BVH-order triangles and shading data; materials and lights
  PG_TRY_CUDA(st_tris_.ensure(n * 48), "staging");
  PG_TRY_CUDA(st_data_.ensure(n * 48), "staging");
  PG_TRY_CUDA(st_mats_.ensure(mats.size() * sizeof(DevMaterial)), "staging");
  PG_TRY_CUDA(st_lights_.ensure(flat.light_v0.size() * 48), "staging");
  PG_TRY_CUDA(st_cdf_.ensure(flat.light_cdf.size() * 4), "staging");
  PG_TRY_CUDA(st_perm_.ensure(n * 4), "staging");
  for (PinnedBuffer *b : {&st_nodes_, &st_extra_, &st_wnodes_, &st_wtris_}) {
    PG_TRY_CUDA(b->ensure(0), "staging");
  }
  float *tris = st_tris_.as<float>();
  float *data = st_data_.as<float>();
  for (size_t i = 0; i < n; ++i) {
    const uint32_t o = prep_.bvh.permutation[i];
    put_tri(&tris[12 * i], flat.v0[o], flat.v1[o], flat.v2[o], 0);
    float d[12] = {flat.n0[o].x, flat.n0[o].y, flat.n0[o].z, flat.n1[o].x,
                   flat.n1[o].y, flat.n1[o].z, flat.n2[o].x, flat.n2[o].y,
                   flat.n2[o].z, 0.f, 0.f, 0.f};
    std::memcpy(&d[11], &flat.material[o], sizeof(uint32_t));
    std::memcpy(&data[12 * i], d, sizeof(d));
  }
  stage_materials(flat, mats);
  if (n > 0) {
    std::memcpy(st_perm_.get(), prep_.bvh.permutation.data(), n * 4);
  }
  struct Pair {
    DeviceBuffer *dev;
    PinnedBuffer *host;
  };
  Pair pairs[] = {{&tris_, &st_tris_},         {&tri_data_, &st_data_},
                  {&materials_, &st_mats_},    {&light_tris_, &st_lights_},
                  {&light_cdf_, &st_cdf_},     {&perm_, &st_perm_}};
  for (const Pair &pr : pairs) {
    PG_TRY_CUDA(pr.dev->upload(pr.host->get(), pr.host->bytes, stream_), "scene upload");
  }
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "upload sync");
  prep_.n_tris = (uint32_t)n;
  prep_.n_lights = (uint32_t)flat.light_v0.size();
  return Status::ok();
}

// materials and the light table (which depends on emission) into staging
void Renderer::stage_materials(const FlatScene &flat, const std::vector<path_material> &mats) {
  DevMaterial *dm = st_mats_.as<DevMaterial>();
  mat_types_ = 0;
  for (size_t i = 0; i < mats.size(); ++i) {
    dm[i] = to_dev(mats[i]);
    mat_types_ |= 1u << (mats[i].type & 31u);
  }
  float *lt = st_lights_.as<float>();
  for (size_t i = 0; i < flat.light_v0.size(); ++i) {
    put_tri(&lt[12 * i], flat.light_v0[i], flat.light_v1[i], flat.light_v2[i], 0);
  }
  if (!flat.light_cdf.empty()) {
    std::memcpy(st_cdf_.get(), flat.light_cdf.data(), flat.light_cdf.size() * 4);
  }
}

// after an in-place material edit: new materials and light table, same BVH
Status Renderer::refresh_materials(const Scene &scene, uint64_t *bytes) {
  FlatScene flat = flatten(scene);
  PG_TRY_CUDA(st_mats_.ensure(scene.materials.size() * sizeof(DevMaterial)), "staging");
  PG_TRY_CUDA(st_lights_.ensure(flat.light_v0.size() * 48), "staging");
  PG_TRY_CUDA(st_cdf_.ensure(flat.light_cdf.size() * 4), "staging");
  stage_materials(flat, scene.materials);
  PG_TRY_CUDA(materials_.upload(st_mats_.get(), st_mats_.bytes, stream_), "material upload");
  PG_TRY_CUDA(light_tris_.upload(st_lights_.get(), st_lights_.bytes, stream_), "light upload");
  PG_TRY_CUDA(light_cdf_.upload(st_cdf_.get(), st_cdf_.bytes, stream_), "light upload");
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "upload sync");
  *bytes += st_mats_.bytes + st_lights_.bytes + st_cdf_.bytes;
  prep_.n_lights = (uint32_t)flat.light_v0.size();
  prep_.material_version = scene.material_version;
  return Status::ok();
}

// host -> device copies of every staged scene array (asynchronous)
// The resident scene copied from its pinned staging copies: every array
// (all), or only those a render with this traversal reads (the binary or
// the 8-wide BVH, not both; the permutation serves path_intersect only).
Status Renderer::copy_staged(uint64_t *bytes, bool all, uint32_t traversal) {
  struct Pair {
    DeviceBuffer *dev;
    PinnedBuffer *host;
    bool used;
  };
  const bool wide = traversal == PATH_TRAVERSAL_WIDE8;
  const Pair pairs[] = {{&tris_, &st_tris_, true},          {&tri_data_, &st_data_, true},
                        {&bin_nodes_, &st_nodes_, !wide},    {&extra_, &st_extra_, !wide},
                        {&wide_nodes_, &st_wnodes_, wide},   {&wide_tris_, &st_wtris_, wide},
                        {&materials_, &st_mats_, true},      {&light_tris_, &st_lights_, true},
                        {&light_cdf_, &st_cdf_, true},       {&perm_, &st_perm_, false}};
  uint64_t total = 0;
  for (const Pair &p : pairs) {
    if (!all && !p.used) {
      continue;
    }
    PG_TRY_CUDA(p.dev->upload(p.host->get(), p.host->bytes, stream_), "scene upload");
    total += p.host->bytes;
  }
  *bytes = total;
  return Status::ok();
}

Status Renderer::prepare_scene(const FlatScene &flat, uint64_t id, uint64_t version,
                               const SBVHSettings &sbvh, bool force) {
  if (!force && prep_.valid && prep_.scene_id == id && prep_.scene_version == version &&
      prep_.sbvh.overlap_threshold == sbvh.overlap_threshold &&
      prep_.sbvh.use_spatial_splits == sbvh.use_spatial_splits &&
      prep_.sbvh.traversal_per_intersect_cost == sbvh.traversal_per_intersect_cost &&
      prep_.sbvh.target_objects == sbvh.target_objects) {
    return Status::ok();
  }
  prep_.valid = false;
  prep_.gpu_built = 0;
  auto t0 = std::chrono::steady_clock::now();
  prep_.bvh = build_sbvh(flat.v0.data(), flat.v1.data(), flat.v2.data(), flat.v0.size(), sbvh);
  prep_.wide = build_wide(prep_.bvh);
  prep_.n_wide_nodes = (uint32_t)prep_.wide.nodes.size();
  scene_box(flat, prep_.lo, prep_.hi);
  prep_.orig_to_bvh.assign(prep_.bvh.permutation.size(), 0u);
  for (size_t i = 0; i < prep_.bvh.permutation.size(); ++i) {
    prep_.orig_to_bvh[prep_.bvh.permutation[i]] = (uint32_t)i;
  }
  auto t1 = std::chrono::steady_clock::now();
  prep_.build_seconds = std::chrono::duration<double>(t1 - t0).count();
  prep_.scene_id = id;
  prep_.scene_version = version;
  prep_.sbvh = sbvh;
  return Status::ok();
}

Status Renderer::prepare_sobol(uint32_t dim_bound, uint32_t count) {
  // row s of the table is the s-th Sobol point whatever the table's size, so
  // a table with at least `count` rows serves; grow in powers of two
  if (sobol_bound_ == dim_bound && sobol_count_ >= count && sobol_table_.get()) {
    return Status::ok();
  }
  uint32_t rows = 1;
  while (rows < count) {
    rows <<= 1;
  }
  count = rows;
  curandDirectionVectors32_t *vecs = nullptr;
  unsigned *scr = nullptr;
  if (curandGetDirectionVectors32(&vecs, CURAND_SCRAMBLED_DIRECTION_VECTORS_32_JOEKUO6) !=
          CURAND_STATUS_SUCCESS ||
      curandGetScrambleConstants32(&scr) != CURAND_STATUS_SUCCESS) {
    return Status::err(PATH_ERR_CUDA, "cuRAND direction vectors unavailable");
  }
  if (dim_bound > 20000) {
    return Status::err(PATH_ERR_ARGUMENT, "max_sample_size above the 20000 Sobol dimensions");
  }
  // direction vectors [dim_bound][32], then the scramble constants
  PG_TRY_CUDA(sobol_dirs_.ensure((size_t)dim_bound * 33 * 4), "sobol dirs");
  PG_TRY_CUDA(cudaMemcpyAsync(sobol_dirs_.get(), vecs, (size_t)dim_bound * 32 * 4,
                              cudaMemcpyHostToDevice, stream_),
              "sobol dirs");
  PG_TRY_CUDA(cudaMemcpyAsync(sobol_dirs_.as<uint32_t>() + (size_t)dim_bound * 32, scr,
                              (size_t)dim_bound * 4, cudaMemcpyHostToDevice, stream_),
              "sobol scramble");
  PG_TRY_CUDA(sobol_table_.ensure((size_t)dim_bound * count * 4), "sobol table");
  PG_TRY_CUDA(launch_sobol_table(sobol_dirs_.as<uint32_t>(),
                                 sobol_dirs_.as<uint32_t>() + (size_t)dim_bound * 32, dim_bound,
                                 count, sobol_table_.as<float>(), stream_),
              "sobol kernel");
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "sobol sync");
  sobol_bound_ = dim_bound;
  sobol_count_ = count;
  return Status::ok();
}

void Renderer::fill_params(RenderParams &p) const {
  std::memset(&p, 0, sizeof(p));
  p.tris = tris_.as<const float4>();
  p.tri_data = tri_data_.as<const float4>();
  p.bin_nodes = bin_nodes_.as<const uint4>();
  p.extra_idxs = extra_.as<const uint32_t>();
  p.wide_nodes = wide_nodes_.as<const uint4>();
  p.wide_tris = wide_tris_.as<const float4>();
  p.n_tris = prep_.n_tris;
  p.n_bin_nodes = (uint32_t)prep_.bvh.nodes.size();
  p.n_wide_nodes = prep_.n_wide_nodes;
  p.materials = materials_.as<const DevMaterial>();
  p.light_tris = light_tris_.as<const float4>();
  p.light_cdf = light_cdf_.as<const float>();
  p.n_lights = prep_.n_lights;
  p.status = status_.as<uint32_t>();
  p.counters = counters_.as<unsigned long long>();
}

static_assert(kMaxOutputSteps == PATH_MAX_OUTPUT_STEPS, "step bound");

// i-th event of the trace-timing pool (created on first use)
cudaEvent_t Renderer::trace_event(size_t i) {
  while (trace_ev_.size() <= i) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
      return nullptr;
    }
    trace_ev_.push_back(e);
  }
  return trace_ev_[i];
}

// the resident BVH within the traversal kernels' fixed stacks
Status Renderer::traversal_fits(const path_settings &st) const {
  if (st.traversal == PATH_TRAVERSAL_WIDE8 && prep_.wide.depth + 1 > kWideStackDepth) {
    return Status::err(PATH_ERR_UNSUPPORTED, "wide BVH deeper than the traversal stack");
  }
  if (st.traversal == PATH_TRAVERSAL_BINARY && prep_.gpu_built) {
    return Status::err(PATH_ERR_UNSUPPORTED, "the resident BVH came from the GPU builder, "
                                             "which makes no binary BVH");
  }
  if (st.traversal == PATH_TRAVERSAL_BINARY) {
    if (prep_.bvh.depth + 2 > 64) {
      return Status::err(PATH_ERR_UNSUPPORTED, "SBVH deeper than the 64-entry traversal stack");
    }
    if (st.target_objects + prep_.bvh.max_leaf_size - 1 > 10) {
      return Status::err(PATH_ERR_UNSUPPORTED,
                         "target_objects + max leaf size - 1 exceeds the 10 candidates");
    }
  }
  return Status::ok();
}

Status check_settings(const path_settings &s) {
  if (s.kernel_approach != PATH_KERNEL_MEGA && s.kernel_approach != PATH_KERNEL_STREAMING) {
    return Status::err(PATH_ERR_ARGUMENT, "unknown kernel_approach");
  }
  if (s.rng != PATH_RNG_SOBEL && s.rng != PATH_RNG_UNIFORM) {
    return Status::err(PATH_ERR_ARGUMENT, "unknown rng value");
  }
  if (s.light_sampler > PATH_LIGHT_NONE || s.dir_sampler > PATH_DIR_UNIFORM ||
      s.term_prob > PATH_TERM_NORMALIZE || s.traversal > PATH_TRAVERSAL_WIDE8) {
    return Status::err(PATH_ERR_ARGUMENT, "unknown sampler / term_prob / traversal value");
  }
  if (s.max_sample_size == 0) {
    return Status::err(PATH_ERR_ARGUMENT, "max_sample_size must be positive");
  }
  if (s.target_objects == 0 || s.target_objects > 10) {
    return Status::err(PATH_ERR_ARGUMENT, "target_objects must be in [1, 10]");
  }
  if (s.wavefront_slots_log2 != 0 && (s.wavefront_slots_log2 < 10 || s.wavefront_slots_log2 > 26)) {
    return Status::err(PATH_ERR_ARGUMENT, "wavefront_slots_log2 must be 0 or in [10, 26]");
  }
  if (s.gpu_build > 2) {
    return Status::err(PATH_ERR_ARGUMENT, "gpu_build must be 0, 1 or 2");
  }
  if (s.trace_staged_nodes > kMaxStagedNodes) {
    return Status::err(PATH_ERR_ARGUMENT, "trace_staged_nodes must be at most 512");
  }
  return Status::ok();
}

Status Renderer::render(const path_sample_spec &spec, const path_output &output,
                        const Scene &scene, uint32_t spp, const path_settings &st,
                        double *seconds) {
  Status sc = check_settings(st);
  if (!sc.good()) {
    return sc;
  }
  if (spec.type != PATH_SAMPLE_SQUARE_IMAGE && spec.type != PATH_SAMPLE_INITIAL_RAYS &&
      spec.type != PATH_SAMPLE_INITIAL_IDX_AND_DIR) {
    return Status::err(PATH_ERR_UNSUPPORTED, "unknown sample spec type");
  }
  const bool idx_spec = spec.type == PATH_SAMPLE_INITIAL_IDX_AND_DIR;
  const bool rays_spec = spec.type == PATH_SAMPLE_INITIAL_RAYS || idx_spec;
  if (rays_spec && (spec.rays == nullptr || spec.n_rays == 0)) {
    return Status::err(PATH_ERR_ARGUMENT, "InitialRays / InitialIdxAndDir spec without rays");
  }
  if (idx_spec && spec.idxs == nullptr) {
    return Status::err(PATH_ERR_ARGUMENT, "InitialIdxAndDir spec without triangle indices");
  }
  const bool per_step = output.type == PATH_OUTPUT_PER_STEP;
  if (per_step && (output.n_steps == 0 || output.n_steps > PATH_MAX_OUTPUT_STEPS)) {
    return Status::err(PATH_ERR_ARGUMENT, "OutputPerStep needs 1.." +
                                              std::to_string(PATH_MAX_OUTPUT_STEPS) + " steps");
  }
  if ((idx_spec || per_step) && st.kernel_approach != PATH_KERNEL_MEGA) {
    // streaming/run_impl.h:65 and :455 leave both unimplemented
    return Status::err(PATH_ERR_UNSUPPORTED,
                       "InitialIdxAndDir and OutputPerStep need the MegaKernel approach");
  }
  // InitialRays / InitialIdxAndDir render one "pixel" per entry
  // (mega_kernel/run_impl.h:56-67)
  const uint32_t x_dim = rays_spec ? spec.n_rays : spec.x_dim;
  const uint32_t y_dim = rays_spec ? 1u : spec.y_dim;
  if (x_dim == 0 || y_dim == 0 || spp == 0) {
    return Status::err(PATH_ERR_ARGUMENT, "image size and samples_per must be positive");
  }
  // the band of rows this call renders (the whole image by default)
  uint32_t row_lo = 0, row_hi = y_dim;
  if (!rays_spec && (spec.row_start != 0 || spec.row_end != 0)) {
    if (spec.row_start >= spec.row_end || spec.row_end > y_dim) {
      return Status::err(PATH_ERR_ARGUMENT, "row band must satisfy start < end <= y_dim");
    }
    row_lo = spec.row_start;
    row_hi = spec.row_end;
  }
  if (output.data == nullptr ||
      (output.type != PATH_OUTPUT_BGRA && output.type != PATH_OUTPUT_FLOAT_RGB && !per_step)) {
    return Status::err(PATH_ERR_ARGUMENT, "output buffer missing or unknown output type");
  }
  for (size_t i = 0; i < scene.tri_material.size(); ++i) {
    if (scene.tri_material[i] >= scene.materials.size()) {
      return Status::err(PATH_ERR_ARGUMENT, "triangle material index out of range");
    }
  }
  Status s0 = init();
  if (!s0.good()) {
    return s0;
  }
  SBVHSettings sb;
  sb.overlap_threshold = st.overlap_threshold;
  sb.use_spatial_splits = st.use_spatial_splits != 0;
  sb.traversal_per_intersect_cost = st.traversal_per_intersect_cost;
  sb.target_objects = st.target_objects;
  const uint32_t gpu_build = st.gpu_build;
  if (gpu_build != 0 && st.traversal != PATH_TRAVERSAL_WIDE8) {
    return Status::err(PATH_ERR_UNSUPPORTED, "the GPU builder makes the 8-wide BVH only");
  }
  bool rebuilt = !(prep_.valid && prep_.scene_id == scene.id &&
                   prep_.gpu_built == gpu_build && prep_.scene_version == scene.version &&
                   prep_.sbvh.overlap_threshold == sb.overlap_threshold &&
                   prep_.sbvh.use_spatial_splits == sb.use_spatial_splits &&
                   prep_.sbvh.traversal_per_intersect_cost == sb.traversal_per_intersect_cost &&
                   prep_.sbvh.target_objects == sb.target_objects);
  if (rebuilt && gpu_build != 0) {
    FlatScene flat = flatten(scene);
    Status sp = prepare_scene_gpu(flat, scene.id, scene.version, scene.materials, gpu_build);
    if (!sp.good()) {
      return sp;
    }
    prep_.sbvh = sb;
    prep_.material_version = scene.material_version;
    prep_.valid = true;
  } else if (rebuilt) {
    FlatScene flat = flatten(scene);
    Status sp = prepare_scene(flat, scene.id, scene.version, sb, true);
    if (!sp.good()) {
      return sp;
    }
    Status su = upload_geometry(flat, scene.materials);
    if (!su.good()) {
      return su;
    }
    prep_.material_version = scene.material_version;
    prep_.valid = true;
  }
  uint64_t h2d = 0;
  if (!rebuilt && prep_.material_version != scene.material_version) {
    Status sm = refresh_materials(scene, &h2d);
    if (!sm.good()) {
      return sm;
    }
  }
  if (st.kernel_approach == PATH_KERNEL_STREAMING && st.traversal != PATH_TRAVERSAL_WIDE8) {
    return Status::err(PATH_ERR_UNSUPPORTED, "the streaming approach traces the 8-wide BVH only");
  }
  Status sf = traversal_fits(st);
  if (!sf.good()) {
    return sf;
  }
  if (!rebuilt && st.upload_scene_every_render) {
    Status sr = copy_staged(&h2d, false, st.traversal);
    if (!sr.good()) {
      return sr;
    }
  }
  if (st.rng == PATH_RNG_SOBEL) {
    Status ss = prepare_sobol(st.max_sample_size, spec.sample_offset + spp);
    if (!ss.good()) {
      return ss;
    }
  }
  WorkDiv wd;
  if (!make_workdiv(st.render_work_division, spp, x_dim, y_dim, wd)) {
    return Status::err(PATH_ERR_ARGUMENT, "invalid render work division settings");
  }
  if (wd.block_size > 256) {
    return Status::err(PATH_ERR_UNSUPPORTED, "render block_size above 256");
  }
  const size_t n_pix = (size_t)x_dim * y_dim;
  uint64_t spec_h2d = 0;
  if (rays_spec) {
    PG_TRY_CUDA(rays_.upload(spec.rays, n_pix * 24, stream_), "ray upload");
    spec_h2d = n_pix * 24;
  }
  if (idx_spec) {
    // scene-order triangle index -> BVH order (the device arrays' order)
    std::vector<uint32_t> bvh_idx(n_pix);
    for (size_t i = 0; i < n_pix; ++i) {
      if (spec.idxs[i] >= prep_.orig_to_bvh.size()) {
        return Status::err(PATH_ERR_ARGUMENT, "InitialIdxAndDir triangle index out of range");
      }
      bvh_idx[i] = prep_.orig_to_bvh[spec.idxs[i]];
    }
    PG_TRY_CUDA(idxs_.upload(bvh_idx.data(), n_pix * 4, stream_), "index upload");
    spec_h2d += n_pix * 4;
  }
  const bool bgra = output.type == PATH_OUTPUT_BGRA;
  const uint32_t nsb = wd.num_sample_blocks;
  const uint32_t n_steps = per_step ? output.n_steps : 1u;
  // one (partial-sum) image per output step, step_floats apart
  const size_t step_floats = (size_t)nsb * n_pix * 3;
  float *direct_rgb = nullptr;
  if (!bgra && nsb == 1 && output.on_device) {
    direct_rgb = static_cast<float *>(output.data);
  } else {
    PG_TRY_CUDA(out_a_.ensure(n_steps * step_floats * 4), "output buffer");
  }
  if (nsb > 1) {
    PG_TRY_CUDA(out_b_.ensure(n_steps * step_floats * 4), "reduce buffer");
  }
  if (bgra && !output.on_device) {
    PG_TRY_CUDA(bgra_.ensure(n_pix * 4), "bgra buffer");
  }
  PG_TRY_CUDA(status_.ensure(4), "status word");
  PG_TRY_CUDA(counters_.ensure(3 * 8), "counters");
  PG_TRY_CUDA(cudaMemsetAsync(status_.get(), 0, 4, stream_), "status reset");
  PG_TRY_CUDA(cudaMemsetAsync(counters_.get(), 0, 24, stream_), "counter reset");

  RenderParams p;
  fill_params(p);
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
  std::memcpy(p.f2w, spec.film_to_world, sizeof(p.f2w));
  p.initial_rays = rays_spec ? rays_.as<const float>() : nullptr;
  p.initial_idx = idx_spec ? idxs_.as<const uint32_t>() : nullptr;
  p.n_steps = per_step ? n_steps : 0u;
  p.step_stride = step_floats;
  p.x_dim = x_dim;
  p.y_dim = y_dim;
  p.spp = spp;
  p.wd = wd;
  p.out_rgb = direct_rgb ? direct_rgb : out_a_.as<float>();
  uint8_t *bgra_dev = bgra ? (output.on_device ? static_cast<uint8_t *>(output.data)
                                               : bgra_.as<uint8_t>())
                           : nullptr;
  p.out_bgra = bgra_dev;
  p.output_bgra = bgra ? 1 : 0;
  // blocks are ordered (sample block, x block, y block): a band of rows is
  // the contiguous block range of the y blocks it touches
  const uint32_t blocks_per_yblock = wd.num_sample_blocks * wd.num_x_blocks;
  const uint32_t yb0 = row_lo / wd.y_block_size;
  const uint32_t yb1 = (row_hi + wd.y_block_size - 1) / wd.y_block_size;
  const uint32_t n_blocks = (yb1 - yb0) * blocks_per_yblock;
  p.start_block = yb0 * blocks_per_yblock;
  p.row_lo = row_lo;
  p.sample_offset = spec.sample_offset;
  p.cache_depth = cache_ != nullptr ? cache_depth_ : 0u;
  if (cache_ != nullptr) {
    // the frame's queries are evaluated over this scene's box (also after
    // the cache served a batch in its cell coordinates)
    cache_->set_bounds(prep_.lo, prep_.hi);
  }
  p.rng_uniform = st.rng == PATH_RNG_UNIFORM ? 1u : 0u;
  p.row_hi = row_hi;
  // the streaming trace kernel's shared-memory copy of the BVH's top (host
  // builds lay the top levels out breadth first; the default trace variant)
  p.n_staged = st.traversal == PATH_TRAVERSAL_WIDE8 && !prep_.gpu_built &&
                       (st.trace_min_blocks == 0 || st.trace_min_blocks == 4)
                   ? std::min(st.trace_staged_nodes, prep_.wide.n_top)
                   : 0u;
  const size_t pix0 = (size_t)row_lo * x_dim;           // first band pixel
  const size_t n_band = (size_t)(row_hi - row_lo) * x_dim;

  last_params_ = p;
  last_blocks_ = n_blocks;
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "pre-render sync");
  auto t0 = std::chrono::steady_clock::now();
  uint32_t launches = 0;
  PG_TRY_CUDA(cudaEventRecord(ev_start_, stream_), "event");
  if (cache_ != nullptr && cache_train_paths_ > 0) {
    // the cache's training paths are independent of the frame: trace them on
    // a side stream while the frame renders (the scene is uploaded already)
    if (side_stream_ == nullptr) {
      PG_TRY_CUDA(cudaStreamCreateWithFlags(&side_stream_, cudaStreamNonBlocking), "stream");
      PG_TRY_CUDA(cudaEventCreateWithFlags(&side_done_, cudaEventDisableTiming), "event");
    }
    RenderParams tp = p;
    tp.cache_depth = 0;
    PG_TRY_CUDA(cache_records_.ensure((size_t)cache_train_paths_ * 64), "cache records");
    PG_TRY_CUDA(launch_nrc_paths(tp, cache_train_paths_, frame_counter_++, p.cache_depth,
                                 cache_records_.as<float>(), side_stream_),
                "cache training paths");
    PG_TRY_CUDA(cudaEventRecord(side_done_, side_stream_), "event");
    ++launches;
  }
  if (st.kernel_approach == PATH_KERNEL_STREAMING) {
    // paths in flight: up to 2^26 (144 bytes each, 9.7 GB at the most), so
    // that a render of up to 67 M samples has all of them in flight at once
    slots_log2_ = st.wavefront_slots_log2 ? st.wavefront_slots_log2 : 26u;
    Status sw = run_wavefront(p, n_blocks, st.count_work != 0, st.trace_min_blocks,
                              st.time_kernels != 0, &launches);
    if (!sw.good()) {
      return sw;
    }
  } else if (per_step) {
    PG_TRY_CUDA(launch_render_steps(p, st.traversal, n_blocks, stream_),
                "render kernel");
    ++launches;
  } else {
    PG_TRY_CUDA(launch_render(p, st.traversal, n_blocks, st.count_work != 0, stream_),
                "render kernel");
    ++launches;
  }
  // ReduceFloatRGB passes over the band's pixels: with `factor` partial sums
  // per pixel, pixel j's sums start at float (pix0 + j) * factor * 3
  uint32_t factor = nsb;
  float *in = p.out_rgb;
  float *other = out_b_.as<float>();
  size_t elems = (size_t)nsb * n_band;
  while (factor != 1) {
    ReduceParams rp;
    std::memset(&rp, 0, sizeof(rp));
    uint32_t xd = (uint32_t)(elems / factor);
    if (!make_workdiv(st.reduce_work_division, factor, xd, 1, rp.wd)) {
      return Status::err(PATH_ERR_ARGUMENT, "invalid reduce work division settings");
    }
    rp.reduction_factor = factor;
    rp.spp = spp;
    rp.output_bgra = bgra ? 1 : 0;
    rp.out_bgra = bgra_dev ? bgra_dev + pix0 * 4 : nullptr;
    const uint32_t next_factor = rp.wd.num_sample_blocks;
    for (uint32_t k = 0; k < n_steps; ++k) {
      rp.in = in + k * step_floats + pix0 * factor * 3;
      rp.out = other + k * step_floats + pix0 * next_factor * 3;
      PG_TRY_CUDA(launch_reduce(rp, stream_), "reduce kernel");
      ++launches;
    }
    factor = rp.wd.num_sample_blocks;
    elems = (size_t)xd * factor;
    std::swap(in, other);
  }
  PG_TRY_CUDA(cudaEventRecord(ev_stop_, stream_), "event");
  if (bgra) {
    if (!output.on_device) {
      PG_TRY_CUDA(cudaMemcpyAsync(static_cast<uint8_t *>(output.data) + pix0 * 4,
                                  bgra_dev + pix0 * 4, n_band * 4, cudaMemcpyDeviceToHost,
                                  stream_),
                  "output copy");
    }
  } else if (in != output.data) {
    for (uint32_t k = 0; k < n_steps; ++k) {
      PG_TRY_CUDA(cudaMemcpyAsync(static_cast<float *>(output.data) + k * n_pix * 3 + pix0 * 3,
                                  in + k * step_floats + pix0 * 3, n_band * 12,
                                  output.on_device ? cudaMemcpyDeviceToDevice
                                                   : cudaMemcpyDeviceToHost,
                                  stream_),
                  "output copy");
    }
  }
  uint64_t d2h = 0;
  if (!output.on_device) {
    d2h = bgra ? n_band * 4 : n_steps * n_band * 12;
  }
  uint32_t status = 0;
  unsigned long long counts[3] = {0, 0, 0};
  PG_TRY_CUDA(cudaMemcpyAsync(&status, status_.get(), 4, cudaMemcpyDeviceToHost, stream_),
              "status copy");
  if (st.count_work) {
    PG_TRY_CUDA(cudaMemcpyAsync(counts, counters_.get(), 24, cudaMemcpyDeviceToHost, stream_),
                "counter copy");
  }
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "render sync");
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
  stats_.device_status = status;
  stats_.num_bvh_nodes = (uint32_t)prep_.bvh.nodes.size();
  stats_.num_wide_nodes = prep_.n_wide_nodes;
  stats_.h2d_bytes = h2d + spec_h2d;
  stats_.d2h_bytes = d2h;
  if (st.kernel_approach == PATH_KERNEL_STREAMING) {
    stats_.trace_launches = trace_launches_;
    double tms = 0.0;
    for (uint32_t i = 0; i < trace_timed_; ++i) {
      float e = 0.f;
      PG_TRY_CUDA(cudaEventElapsedTime(&e, trace_ev_[2 * i], trace_ev_[2 * i + 1]), "event");
      tms += e;
    }
    stats_.trace_ms = tms;
  }
  if (seconds) {
    *seconds = stats_.seconds;
  }
  if (status != 0) {
    return Status::err(PATH_ERR_DEVICE_TIMEOUT,
                       "kernel reported device status " + std::to_string(status) +
                           " (1 stack overflow, 2 candidate overflow, 3 bad node, 4 path too long)");
  }
  return Status::ok();
}

// wavefront render of the whole image into p.out_rgb / p.out_bgra (see
// wavefront.cu); the host checks the live-slot count every few iterations
Status Renderer::run_wavefront(const RenderParams &p, uint32_t n_blocks, bool counting,
                               uint32_t min_blocks, bool time_trace, uint32_t *launches,
                               const AdjointState *adj) {
  const uint32_t slots_log2 = slots_log2_;
  trace_timed_ = 0;
  trace_launches_ = 0;
  if (num_sms_ == 0) {
    int dev = 0;
    PG_TRY_CUDA(cudaGetDevice(&dev), "device");
    PG_TRY_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev), "sm count");
  }
  // sample ids are pixel-major: the band's samples are one contiguous range
  const unsigned long long first = (unsigned long long)p.row_lo * p.x_dim * p.spp;
  const unsigned long long total =
      (unsigned long long)(p.row_hi - p.row_lo) * p.x_dim * p.spp;
  const uint32_t n_slots = (uint32_t)std::min<unsigned long long>(total, 1ull << slots_log2);
  auto a256 = [](size_t n) { return (n + 255) & ~size_t(255); };
  const size_t f4 = a256((size_t)n_slots * 16), u2 = a256((size_t)n_slots * 8),
               u1 = a256((size_t)n_slots * 4);
  PG_TRY_CUDA(wf_slots_.ensure(7 * f4 + 2 * u2 + 2 * u1 + 2 * u1), "wavefront slots");
  PG_TRY_CUDA(wf_queues_.ensure(64), "wavefront queues");
  PG_TRY_CUDA(wf_samples_.ensure((size_t)total * 12), "sample buffer");
  PG_TRY_CUDA(wf_host_.ensure(64), "staging");
  unsigned char *b = wf_slots_.as<unsigned char>();
  WaveParams w;
  std::memset(&w, 0, sizeof(w));
  w.P = p;
  w.o = reinterpret_cast<float4 *>(b);
  w.d = reinterpret_cast<float4 *>(b + f4);
  w.ld = reinterpret_cast<float4 *>(b + 2 * f4);
  w.mult = reinterpret_cast<float4 *>(b + 3 * f4);
  w.lmult = reinterpret_cast<float4 *>(b + 4 * f4);
  w.total = reinterpret_cast<float4 *>(b + 5 * f4);
  w.state = reinterpret_cast<uint4 *>(b + 6 * f4);
  w.hit_ext = reinterpret_cast<uint2 *>(b + 7 * f4);
  w.hit_light = reinterpret_cast<uint2 *>(b + 7 * f4 + u2);
  w.active[0] = reinterpret_cast<uint32_t *>(b + 7 * f4 + 2 * u2);
  w.active[1] = reinterpret_cast<uint32_t *>(b + 7 * f4 + 2 * u2 + u1);
  w.rays = reinterpret_cast<uint32_t *>(b + 7 * f4 + 2 * u2 + 2 * u1);
  w.q = wf_queues_.as<WaveQueues>();
  w.next_sample = reinterpret_cast<unsigned long long *>(wf_queues_.as<unsigned char>() + 32);
  w.first_sample = first;
  w.total_samples = first + total;
  w.sample_rgb = wf_samples_.as<float>();
  w.n_slots = n_slots;
  w.feat = work_features(mat_types_, p);
  if (p.cache_depth != 0 && cache_ != nullptr) {
    if (total >= (1ull << 32)) {
      return Status::err(PATH_ERR_UNSUPPORTED, "more than 2^32 samples with the cache");
    }
    PG_TRY_CUDA(cache_q_.ensure((size_t)total * 48), "cache queries");
    PG_TRY_CUDA(cache_beta_.ensure((size_t)total * 12), "cache queries");
    PG_TRY_CUDA(cudaMemsetAsync(cache_beta_.get(), 0, (size_t)total * 12, stream_),
                "cache queries");
    w.cache_q = cache_q_.as<float>();
    w.cache_beta = cache_beta_.as<float>();
    cached_samples_ = total;
  }
  const bool grad = adj != nullptr;
  if (grad) {
    // replay: the forward pass's per-sample radiance stays in wf_samples_
    PG_TRY_CUDA(adj_pend_.ensure((size_t)n_slots * 36 + 512), "adjoint slots");
    unsigned char *pb = adj_pend_.as<unsigned char>();
    w.d_image = adj->d_image;
    w.pend_refl = reinterpret_cast<float4 *>(pb);
    w.pend_nee = reinterpret_cast<float4 *>(pb + a256((size_t)n_slots * 16));
    w.pend_mat = reinterpret_cast<uint32_t *>(pb + 2 * a256((size_t)n_slots * 16));
    w.d_params = adj->d_params;
    PG_TRY_CUDA(cudaMemsetAsync(w.pend_mat, 0xff, (size_t)n_slots * 4, stream_), "adjoint init");
  }
  if (p.rng_uniform) {
    PG_TRY_CUDA(wf_rng_.ensure((size_t)n_slots * kRngStateWords * 4), "rng states");
    w.rng_state = wf_rng_.as<uint32_t>();
  }
  // queue heads: n_slots live slots, one extension ray each
  uint32_t *h = wf_host_.as<uint32_t>();
  std::memset(h, 0, 64);
  h[0] = n_slots;
  h[2] = n_slots;
  unsigned long long next = first + n_slots;
  std::memcpy(h + 8, &next, sizeof(next));
  PG_TRY_CUDA(cudaMemcpyAsync(wf_queues_.get(), h, 48, cudaMemcpyHostToDevice, stream_),
              "queue init");
  PG_TRY_CUDA(launch_wavefront_init(w, n_slots, stream_), "wavefront init");
  *launches += 1;
  const uint32_t trace_grid =
      (uint32_t)num_sms_ * (uint32_t)wavefront_trace_blocks_per_sm(min_blocks, counting, p.n_staged);
  const uint32_t shade_grid = (uint32_t)num_sms_ * 4;
  uint32_t parity = 0;
  volatile uint32_t *live = h + 12;
  // Iterations before the first live-count check: under NIters{N} a path
  // that starts in the first iteration is shaded at most N + 1 times and its
  // last light ray traced once more, so when every sample is in flight the
  // first check after N + 2 iterations finds no live path; then 4 a round.
  const uint32_t first_round =
      p.term_prob == 1 ? std::min<uint32_t>(std::max<uint32_t>(p.term_iters + 2, 4), 64) : 4;
  for (uint32_t round = 0;; ++round) {
    const uint32_t iters = round == 0 ? first_round : 4;
    for (uint32_t k = 0; k < iters; ++k) {
      if (time_trace) {
        PG_TRY_CUDA(cudaEventRecord(trace_event(2 * trace_timed_), stream_), "event");
      }
      PG_TRY_CUDA(launch_wavefront_trace(w, trace_grid, min_blocks, counting, stream_),
                  "wavefront trace");
      if (time_trace) {
        PG_TRY_CUDA(cudaEventRecord(trace_event(2 * trace_timed_ + 1), stream_), "event");
        ++trace_timed_;
      }
      // what the host knows of the pass's live slots: all fresh in the
      // first pass; none with an extension ray in the pass after the
      // (N + 1)-th vertex when every sample has been in flight from the start
      w.pass = round == 0 && k == 0 ? kPassFresh
               : round == 0 && p.term_prob == 1 && n_slots == total && k == p.term_iters + 1
                   ? kPassLightOnly
                   : kPassGeneral;
      PG_TRY_CUDA(launch_wavefront_shade(w, parity, shade_grid, stream_, grad),
                  "wavefront shade");
      *launches += 3;
      ++trace_launches_;
      parity ^= 1u;
    }
    PG_TRY_CUDA(cudaMemcpyAsync(h + 12, &w.q->active[parity], 4, cudaMemcpyDeviceToHost,
                                stream_),
                "live count");
    PG_TRY_CUDA(cudaStreamSynchronize(stream_), "wavefront sync");
    if (*live == 0) {
      break;
    }
    if (round > 4 * kMaxPathVertices) {
      return Status::err(PATH_ERR_DEVICE_TIMEOUT, "wavefront did not drain");
    }
  }
  if (grad) {
    return Status::ok();
  }
  if (w.cache_q != nullptr) {
    // the radiance cache's prediction at every path's last vertex
    PG_TRY_CUDA(cache_pred_.ensure((size_t)total * 12), "cache predictions");
    // paths that ended before the cache vertex (zero throughput) skip it
    Status sc = cache_->infer(w.cache_q, (uint32_t)total, cache_pred_.as<float>(), stream_,
                              w.cache_beta);
    if (!sc.good()) {
      return sc;
    }
    PG_TRY_CUDA(launch_nrc_apply(w.sample_rgb, w.cache_beta, cache_pred_.as<float>(), total,
                                 stream_),
                "cache apply");
    *launches += 2;
  }
  PG_TRY_CUDA(launch_wavefront_sum(p, w.sample_rgb, n_blocks, stream_), "sample sum");
  *launches += 1;
  return Status::ok();
}

Status Renderer::intersect(const float *tris, uint32_t n_tris, const float *rays,
                           uint32_t n_rays, const path_settings &st, int32_t *idx,
                           float *t) {
  Status s0 = init();
  if (!s0.good()) {
    return s0;
  }
  FlatScene flat;
  for (uint32_t i = 0; i < n_tris; ++i) {
    const float *p = tris + 9 * (size_t)i;
    flat.v0.push_back(mk(p[0], p[1], p[2]));
    flat.v1.push_back(mk(p[3], p[4], p[5]));
    flat.v2.push_back(mk(p[6], p[7], p[8]));
    flat.n0.push_back(mk(0.f, 0.f, 1.f));
    flat.n1.push_back(mk(0.f, 0.f, 1.f));
    flat.n2.push_back(mk(0.f, 0.f, 1.f));
    flat.material.push_back(0);
  }
  SBVHSettings sb;
  sb.overlap_threshold = st.overlap_threshold;
  sb.use_spatial_splits = st.use_spatial_splits != 0;
  sb.traversal_per_intersect_cost = st.traversal_per_intersect_cost;
  sb.target_objects = st.target_objects;
  prep_.valid = false;
  std::vector<path_material> mats(1);
  std::memset(mats.data(), 0, sizeof(path_material));
  if (st.gpu_build) {
    if (st.traversal != PATH_TRAVERSAL_WIDE8) {
      return Status::err(PATH_ERR_UNSUPPORTED, "the GPU builder makes the 8-wide BVH only");
    }
    Status sp = prepare_scene_gpu(flat, 0, 0, mats, st.gpu_build);
    if (!sp.good()) {
      return sp;
    }
  } else {
    Status sp = prepare_scene(flat, 0, 0, sb, true);
    if (!sp.good()) {
      return sp;
    }
    Status su = upload_geometry(flat, mats);
    if (!su.good()) {
      return su;
    }
  }
  Status sf = traversal_fits(st);
  if (!sf.good()) {
    return sf;
  }
  DeviceBuffer d_rays, d_idx, d_t;
  PG_TRY_CUDA(d_rays.upload(rays, (size_t)n_rays * 24, stream_), "rays");
  PG_TRY_CUDA(d_idx.ensure((size_t)n_rays * 4), "idx");
  PG_TRY_CUDA(d_t.ensure((size_t)n_rays * 4), "t");
  PG_TRY_CUDA(status_.ensure(4), "status word");
  PG_TRY_CUDA(counters_.ensure(24), "counters");
  PG_TRY_CUDA(cudaMemsetAsync(status_.get(), 0, 4, stream_), "status reset");
  RenderParams p;
  fill_params(p);
  p.target_objects = st.target_objects;
  PG_TRY_CUDA(launch_intersect(p, st.traversal, d_rays.as<float>(), n_rays,
                               perm_.as<uint32_t>(), d_idx.as<int32_t>(), d_t.as<float>(),
                               stream_),
              "intersect kernel");
  uint32_t status = 0;
  PG_TRY_CUDA(cudaMemcpyAsync(idx, d_idx.get(), (size_t)n_rays * 4, cudaMemcpyDeviceToHost,
                              stream_),
              "idx copy");
  PG_TRY_CUDA(cudaMemcpyAsync(t, d_t.get(), (size_t)n_rays * 4, cudaMemcpyDeviceToHost, stream_),
              "t copy");
  PG_TRY_CUDA(cudaMemcpyAsync(&status, status_.get(), 4, cudaMemcpyDeviceToHost, stream_),
              "status copy");
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "intersect sync");
  if (status != 0) {
    return Status::err(PATH_ERR_DEVICE_TIMEOUT,
                       "kernel reported device status " + std::to_string(status));
  }
  return Status::ok();
}

} // namespace pg

namespace pg {

// Adjoint of the streaming render: a forward render (its per-sample
// radiance stays resident), then a replay of the same paths with gradient
// shading; d_params[materials][7] = dLoss/d(reflectance rgb, roughness,
// emission rgb) for dLoss/d(image) = d_image.
Status Renderer::render_adjoint(const path_sample_spec &spec, const Scene &scene, uint32_t spp,
                                const path_settings &st_in, const float *d_image,
                                bool d_image_on_device, double *d_params, double *seconds) {
  if (spec.type != PATH_SAMPLE_SQUARE_IMAGE || spec.row_start != 0 || spec.row_end != 0) {
    return Status::err(PATH_ERR_UNSUPPORTED, "the adjoint renders whole square images");
  }
  if (d_image == nullptr || d_params == nullptr) {
    return Status::err(PATH_ERR_ARGUMENT, "null adjoint buffer");
  }
  if (st_in.traversal != PATH_TRAVERSAL_WIDE8) {
    return Status::err(PATH_ERR_UNSUPPORTED, "the adjoint replays the streaming render, which "
                                             "traces the 8-wide BVH");
  }
  path_settings st = st_in;
  st.kernel_approach = PATH_KERNEL_STREAMING;
  st.count_work = 0;
  st.time_kernels = 0;
  const size_t n_pix = (size_t)spec.x_dim * spec.y_dim;
  auto t0 = std::chrono::steady_clock::now();
  Status s0 = init();
  if (!s0.good()) {
    return s0;
  }
  PG_TRY_CUDA(adj_image_.ensure(std::max<size_t>(n_pix, 1) * 12), "adjoint image");
  path_output o{};
  o.type = PATH_OUTPUT_FLOAT_RGB;
  o.data = adj_image_.get();
  o.on_device = 1;
  Status sf = render(spec, o, scene, spp, st, nullptr);
  if (!sf.good()) {
    return sf;
  }
  const float fwd_ms = (float)stats_.kernel_ms;
  const size_t n_mat = scene.materials.size();
  PG_TRY_CUDA(adj_params_.ensure(std::max<size_t>(n_mat, 1) * 7 * 8), "adjoint params");
  PG_TRY_CUDA(cudaMemsetAsync(adj_params_.get(), 0, std::max<size_t>(n_mat, 1) * 7 * 8, stream_),
              "adjoint params");
  const float *dimg = d_image;
  if (!d_image_on_device) {
    PG_TRY_CUDA(adj_dimage_.upload(d_image, n_pix * 12, stream_), "adjoint image upload");
    dimg = adj_dimage_.as<const float>();
  }
  AdjointState adj;
  adj.d_image = dimg;
  adj.d_params = adj_params_.as<double>();
  PG_TRY_CUDA(cudaMemsetAsync(status_.get(), 0, 4, stream_), "status reset");
  PG_TRY_CUDA(cudaEventRecord(ev_start_, stream_), "event");
  uint32_t launches = 0;
  Status sr = run_wavefront(last_params_, last_blocks_, false, st.trace_min_blocks, false,
                            &launches, &adj);
  if (!sr.good()) {
    return sr;
  }
  PG_TRY_CUDA(cudaEventRecord(ev_stop_, stream_), "event");
  PG_TRY_CUDA(cudaMemcpyAsync(d_params, adj_params_.get(), n_mat * 7 * 8,
                              cudaMemcpyDeviceToHost, stream_),
              "gradient copy");
  uint32_t status = 0;
  PG_TRY_CUDA(cudaMemcpyAsync(&status, status_.get(), 4, cudaMemcpyDeviceToHost, stream_),
              "status copy");
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "adjoint sync");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev_start_, ev_stop_);
  stats_.kernel_ms = fwd_ms + ms;
  stats_.trace_ms = ms; // the replay alone
  stats_.device_status = status;
  stats_.gpu_launches += launches;
  stats_.seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (seconds) {
    *seconds = stats_.seconds;
  }
  if (status != 0) {
    return Status::err(PATH_ERR_DEVICE_TIMEOUT,
                       "kernel reported device status " + std::to_string(status));
  }
  return Status::ok();
}

} // namespace pg

namespace pg {

Status Renderer::cached_frame_queries(uint32_t max_n, uint32_t stride, float *queries,
                                      float *throughput, uint32_t *n_out) const {
  *n_out = 0;
  if (stride == 0 || cached_samples_ == 0 || cache_q_.get() == nullptr) {
    return Status::err(PATH_ERR_ARGUMENT, "no cached frame (or stride 0)");
  }
  const size_t n = (size_t)((cached_samples_ + stride - 1) / stride);
  std::vector<float> q(n * 12), b(n * 3);
  // every stride-th record, strided copies
  PG_TRY_CUDA(cudaMemcpy2D(q.data(), 48, cache_q_.get(), (size_t)48 * stride, 48, n,
                           cudaMemcpyDeviceToHost),
              "cache queries");
  PG_TRY_CUDA(cudaMemcpy2D(b.data(), 12, cache_beta_.get(), (size_t)12 * stride, 12, n,
                           cudaMemcpyDeviceToHost),
              "cache throughput");
  uint32_t k = 0;
  for (size_t i = 0; i < n && k < max_n; ++i) {
    if (b[3 * i] == 0.f && b[3 * i + 1] == 0.f && b[3 * i + 2] == 0.f) {
      continue; // the path ended before the cache vertex
    }
    std::memcpy(queries + (size_t)12 * k, &q[12 * i], 48);
    std::memcpy(throughput + (size_t)3 * k, &b[3 * i], 12);
    ++k;
  }
  *n_out = k;
  return Status::ok();
}

// One frame with the radiance cache: render (paths end into the cache at
// vertex cache_depth), then train the cache on fresh full-length paths.
Status Renderer::render_cached(const path_sample_spec &spec, const path_output &output,
                               const Scene &scene, uint32_t spp, const path_settings &st_in,
                               RadianceCache &cache, uint32_t cache_depth,
                               uint32_t train_paths, uint32_t train_steps, double *seconds) {
  if (spec.type != PATH_SAMPLE_SQUARE_IMAGE) {
    return Status::err(PATH_ERR_UNSUPPORTED, "the cached render takes square images");
  }
  if (cache_depth == 0 || cache_depth > 64) {
    return Status::err(PATH_ERR_ARGUMENT, "cache_depth must be in [1, 64]");
  }
  if (st_in.traversal != PATH_TRAVERSAL_WIDE8) {
    return Status::err(PATH_ERR_UNSUPPORTED, "the cached render traces the 8-wide BVH");
  }
  path_settings st = st_in;
  st.kernel_approach = PATH_KERNEL_STREAMING;
  st.time_kernels = 0;
  auto t0 = std::chrono::steady_clock::now();
  cache_ = &cache;
  cache_depth_ = cache_depth;
  cache_train_paths_ = train_steps > 0 ? train_paths : 0u;
  Status sr = render(spec, output, scene, spp, st, nullptr);
  const bool side = cache_train_paths_ > 0;
  cache_ = nullptr;
  cache_depth_ = 0;
  cache_train_paths_ = 0;
  if (side && side_done_ != nullptr) {
    // the training paths' records (traced beside the frame)
    PG_TRY_CUDA(cudaEventSynchronize(side_done_), "cache training paths");
    PG_TRY_CUDA(cudaGetLastError(), "cache training paths");
  }
  if (!sr.good()) {
    return sr;
  }
  const double render_ms = stats_.kernel_ms;
  if (train_paths > 0 && train_steps > 0) {
    const uint32_t per = std::max<uint32_t>(train_paths / train_steps, 1);
    for (uint32_t k = 0; k < train_steps; ++k) {
      const uint32_t first = k * per;
      if (first >= train_paths) {
        break;
      }
      const uint32_t cnt = std::min<uint32_t>(per, train_paths - first);
      Status st_train = cache.train(cache_records_.as<float>() + (size_t)first * 16, cnt, nullptr);
      if (!st_train.good()) {
        return st_train;
      }
    }
  }
  auto t1 = std::chrono::steady_clock::now();
  stats_.seconds = std::chrono::duration<double>(t1 - t0).count();
  stats_.kernel_ms = render_ms;
  if (seconds) {
    *seconds = stats_.seconds;
  }
  return Status::ok();
}

} // namespace pg

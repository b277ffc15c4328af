// Batched render: many scenes of uneven size through one persistent
// wavefront.
//
// All scenes' 8-wide BVHs, leaf triangles, BVH-order triangles, shading
// data, materials and light tables are concatenated into one device arena (node, triangle and material
// indices rebased); a BatchScene record per scene holds its camera, sample
// count, root node and light range.  Sample ids run over the scenes in
// order, so the persistent trace and shade kernels of the single-scene
// wavefront serve the whole batch unchanged: a slot carries its scene index
// and root node, and paths of different scenes share every launch.  The
// trace / shade iterations are captured once as a CUDA graph of
// `iterations_per_graph` iterations and replayed until no path is live;
// the per-pixel sums (k_wf_sum + ReduceFloatRGB per scene, in the
// reference's order) are captured as a second graph.  Each image therefore
// equals the single-scene streaming render of the same scene bit for bit,
// whatever the launch shape, which is what lets the autotuner pick shapes
// by time alone.
#include "renderer.h"
#include "gpu_build.h"
#include "cache_host.h"

#include <omp.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cstring>
#include <exception>
#include <mutex>

namespace pg {

namespace {

constexpr uint32_t kDefaultSlotsLog2 = 26;
constexpr uint32_t kDefaultTraceMinBlocks = 4;
constexpr uint32_t kDefaultShadeCtas = 4;
constexpr uint32_t kDefaultItersPerGraph = 4;

path_batch_tuning resolved(const path_batch_tuning *t) {
  path_batch_tuning r{};
  if (t != nullptr) {
    r = *t;
  }
  if (r.slots_log2 == 0) {
    r.slots_log2 = kDefaultSlotsLog2;
  }
  if (r.trace_min_blocks == 0) {
    r.trace_min_blocks = kDefaultTraceMinBlocks;
  }
  if (r.shade_ctas_per_sm == 0) {
    r.shade_ctas_per_sm = kDefaultShadeCtas;
  }
  if (r.iterations_per_graph == 0) {
    r.iterations_per_graph = kDefaultItersPerGraph;
  }
  return r;
}

SBVHSettings sbvh_of(const path_settings &st) {
  SBVHSettings sb;
  sb.overlap_threshold = st.overlap_threshold;
  sb.use_spatial_splits = st.use_spatial_splits != 0;
  sb.traversal_per_intersect_cost = st.traversal_per_intersect_cost;
  sb.target_objects = st.target_objects;
  return sb;
}

bool same_sbvh(const SBVHSettings &a, const SBVHSettings &b) {
  return a.overlap_threshold == b.overlap_threshold &&
         a.use_spatial_splits == b.use_spatial_splits &&
         a.traversal_per_intersect_cost == b.traversal_per_intersect_cost &&
         a.target_objects == b.target_objects;
}

} // namespace

#define PG_TRY_CUDA(expr, what)                                                \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      return cuda_status(e_, what);                                            \
    }                                                                          \
  } while (0)

Status Renderer::check_batch(const std::vector<BatchItem> &items,
                             const path_settings &st) const {
  Status sc = check_settings(st);
  if (!sc.good()) {
    return sc;
  }
  if (items.empty()) {
    return Status::err(PATH_ERR_ARGUMENT, "empty batch");
  }
  if (items.size() >= (1u << 24)) {
    return Status::err(PATH_ERR_UNSUPPORTED, "more than 2^24 - 1 scenes in one batch");
  }
  if (st.traversal != PATH_TRAVERSAL_WIDE8) {
    return Status::err(PATH_ERR_UNSUPPORTED, "a batch is traced through the 8-wide BVH");
  }
  unsigned long long total = 0;
  for (const BatchItem &it : items) {
    if (it.scene == nullptr || it.x_dim == 0 || it.y_dim == 0 || it.spp == 0) {
      return Status::err(PATH_ERR_ARGUMENT, "batch item without scene, size or samples");
    }
    if (it.output.data == nullptr ||
        (it.output.type != PATH_OUTPUT_BGRA && it.output.type != PATH_OUTPUT_FLOAT_RGB)) {
      return Status::err(PATH_ERR_ARGUMENT, "batch item output missing or not BGRA / FloatRGB");
    }
    for (uint32_t m : it.scene->tri_material) {
      if (m >= it.scene->materials.size()) {
        return Status::err(PATH_ERR_ARGUMENT, "triangle material index out of range");
      }
    }
    total += (unsigned long long)it.x_dim * it.y_dim * it.spp;
  }
  if (total >= (1ull << 40)) {
    return Status::err(PATH_ERR_UNSUPPORTED, "more than 2^40 samples in one batch");
  }
  return Status::ok();
}

namespace {

// One scene's 8-wide BVH built on the GPU on stream s (d9 and g: the calling
// thread's buffers, reused from scene to scene), downloaded into w (nodes,
// leaf references) and b (the permutation).
Status build_one_gpu(const FlatScene &f, bool split, cudaStream_t s, DeviceBuffer &d9,
                     GpuWideBVH &g, WideBVH &w, BinaryBVH &b) {
  const size_t nt = f.v0.size();
  std::vector<float> t9(nt * 9);
  for (size_t k = 0; k < nt; ++k) {
    const f3 v[3] = {f.v0[k], f.v1[k], f.v2[k]};
    for (int c = 0; c < 3; ++c) {
      t9[9 * k + 3 * c] = v[c].x;
      t9[9 * k + 3 * c + 1] = v[c].y;
      t9[9 * k + 3 * c + 2] = v[c].z;
    }
  }
  float lo[3], hi[3];
  scene_box(f, lo, hi);
  PG_TRY_CUDA(d9.upload(t9.data(), t9.size() * 4, s), "gpu build upload");
  Status sg = gpu_build_wide(d9.as<float>(), (uint32_t)nt, lo, hi, split, s, g);
  if (!sg.good()) {
    return sg;
  }
  w.nodes.resize(g.n_nodes);
  w.depth = g.depth;
  const size_t nw = g.n_wide_tris;
  std::vector<float> wt(nw * 12);
  b.permutation.resize(nt);
  if (nt > 0) {
    PG_TRY_CUDA(cudaMemcpyAsync(w.nodes.data(), g.nodes.get(), g.n_nodes * sizeof(WideNode),
                                cudaMemcpyDeviceToHost, s),
                "gpu build download");
    PG_TRY_CUDA(cudaMemcpyAsync(wt.data(), g.wide_tris.get(), nw * 48, cudaMemcpyDeviceToHost,
                                s),
                "gpu build download");
    PG_TRY_CUDA(cudaMemcpyAsync(b.permutation.data(), g.perm.get(), nt * 4,
                                cudaMemcpyDeviceToHost, s),
                "gpu build download");
  }
  PG_TRY_CUDA(cudaStreamSynchronize(s), "gpu build download");
  w.tri_index.resize(nw);
  for (size_t k = 0; k < nw; ++k) {
    std::memcpy(&w.tri_index[k], &wt[12 * k + 9], 4);
  }
  return Status::ok();
}

} // namespace

Status Renderer::prepare_batch(const std::vector<BatchItem> &items, const SBVHSettings &sb,
                               uint32_t gpu_build) {
  std::vector<std::array<uint64_t, 3>> key;
  key.reserve(items.size());
  for (const BatchItem &it : items) {
    key.push_back({it.scene->id, it.scene->version, it.scene->material_version});
  }
  if (batch_.valid && batch_.key == key && same_sbvh(batch_.sbvh, sb) &&
      batch_.gpu_build == gpu_build) {
    return Status::ok();
  }
  batch_.valid = false;
  const size_t n = items.size();
  auto t0 = std::chrono::steady_clock::now();
  // one distinct scene may appear in several items: build it once
  std::vector<size_t> first_of(n);
  for (size_t i = 0; i < n; ++i) {
    first_of[i] = i;
    for (size_t j = 0; j < i; ++j) {
      if (key[j] == key[i]) {
        first_of[i] = first_of[j];
        break;
      }
    }
  }
  std::vector<FlatScene> flats(n);
  std::vector<BinaryBVH> bvhs(n);
  std::vector<WideBVH> wides(n);
  std::vector<std::string> errors(n);
#pragma omp parallel for schedule(dynamic, 1)
  for (long long i = 0; i < (long long)n; ++i) {
    if (first_of[(size_t)i] != (size_t)i) {
      continue;
    }
    try {
      FlatScene &f = flats[(size_t)i];
      f = flatten(*items[(size_t)i].scene);
      if (!gpu_build) {
        bvhs[(size_t)i] = build_sbvh(f.v0.data(), f.v1.data(), f.v2.data(), f.v0.size(), sb);
        wides[(size_t)i] = build_wide(bvhs[(size_t)i]);
      }
    } catch (const std::exception &e) {
      errors[(size_t)i] = e.what();
    }
  }
  if (gpu_build) {
    // one GPU build per distinct scene, several at once: host threads with
    // a stream each (the builder's scratch memory is stream-ordered, so the
    // builds overlap); each scene's wide nodes, leaf references and
    // permutation come back for the arena assembly below
    std::vector<size_t> todo;
    size_t max_n = 0;
    for (size_t i = 0; i < n; ++i) {
      if (first_of[i] == i && errors[i].empty()) {
        todo.push_back(i);
        max_n = std::max(max_n, flats[i].v0.size());
      }
    }
    // largest first, so that the threads' buffers are sized by their first scene
    std::sort(todo.begin(), todo.end(),
              [&](size_t a, size_t b) { return flats[a].v0.size() > flats[b].v0.size(); });
    int dev = 0;
    PG_TRY_CUDA(cudaGetDevice(&dev), "device");
    PG_TRY_CUDA(cudaStreamSynchronize(stream_), "gpu build");
    const int n_threads = (int)std::min<size_t>(8, std::max<size_t>(todo.size(), 1));
    std::vector<Status> build_status(n);
    size_t next = 0;
    std::mutex next_mutex;
#pragma omp parallel num_threads(n_threads)
    {
      cudaStream_t bs = nullptr;
      cudaError_t se = cudaSetDevice(dev);
      if (se == cudaSuccess) {
        se = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
      }
      DeviceBuffer d9;
      GpuWideBVH g;
      while (true) {
        size_t k;
        {
          std::lock_guard<std::mutex> lock(next_mutex);
          k = next++;
        }
        if (k >= todo.size()) {
          break;
        }
        const size_t i = todo[k];
        if (se != cudaSuccess) {
          build_status[i] = cuda_status(se, "gpu build stream");
          continue;
        }
        build_status[i] = build_one_gpu(flats[i], gpu_build == 2, bs, d9, g, wides[i], bvhs[i]);
      }
      if (bs != nullptr) {
        cudaStreamSynchronize(bs);
        cudaStreamDestroy(bs);
      }
    }
    for (size_t i : todo) {
      if (!build_status[i].good()) {
        return build_status[i];
      }
    }
  }
  for (size_t i = 0; i < n; ++i) {
    if (!errors[i].empty()) {
      return Status::err(PATH_ERR_OOM, "batch BVH build: " + errors[i]);
    }
    const WideBVH &w = wides[first_of[i]];
    if (w.depth + 1 > kWideStackDepth) {
      return Status::err(PATH_ERR_UNSUPPORTED, "a batch scene's wide BVH is deeper than the "
                                               "traversal stack");
    }
  }
  // arena offsets (an item that repeats a scene shares its first copy)
  std::vector<uint32_t> node_off(n), wtri_off(n), tri_off(n), mat_off(n), light_off(n);
  uint64_t nodes = 0, wtris = 0, tris = 0, mats = 0, lights = 0;
  for (size_t i = 0; i < n; ++i) {
    if (first_of[i] != i) {
      continue;
    }
    node_off[i] = (uint32_t)nodes;
    wtri_off[i] = (uint32_t)wtris;
    tri_off[i] = (uint32_t)tris;
    mat_off[i] = (uint32_t)mats;
    light_off[i] = (uint32_t)lights;
    nodes += wides[i].nodes.size();
    wtris += wides[i].tri_index.size();
    tris += flats[i].v0.size();
    mats += items[i].scene->materials.size();
    lights += flats[i].light_v0.size();
  }
  if (nodes >= (1ull << 31) || wtris >= (1ull << 31) || tris >= (1ull << 31)) {
    return Status::err(PATH_ERR_UNSUPPORTED, "batch arena above 2^31 nodes or triangles");
  }
  std::vector<WideNode> h_nodes((size_t)nodes);
  std::vector<float> h_wtris((size_t)wtris * 12), h_tris((size_t)tris * 12),
      h_data((size_t)tris * 12);
  std::vector<DevMaterial> h_mats((size_t)std::max<uint64_t>(mats, 1));
  std::vector<float> h_lights((size_t)std::max<uint64_t>(lights, 1) * 12),
      h_cdf((size_t)std::max<uint64_t>(lights, 1));
#pragma omp parallel for schedule(dynamic, 1)
  for (long long ii = 0; ii < (long long)n; ++ii) {
    const size_t i = (size_t)ii;
    if (first_of[i] != i) {
      continue;
    }
    const FlatScene &f = flats[i];
    const BinaryBVH &b = bvhs[i];
    const WideBVH &w = wides[i];
    for (size_t k = 0; k < w.nodes.size(); ++k) {
      WideNode wn = w.nodes[k];
      wn.child_base += node_off[i];
      wn.tri_base += wtri_off[i];
      h_nodes[node_off[i] + k] = wn;
    }
    for (size_t k = 0; k < w.tri_index.size(); ++k) {
      const uint32_t bi = w.tri_index[k];
      const uint32_t o = b.permutation[bi];
      put_tri(&h_wtris[12 * ((size_t)wtri_off[i] + k)], f.v0[o], f.v1[o], f.v2[o], 0);
      const uint32_t global = tri_off[i] + bi;
      std::memcpy(&h_wtris[12 * ((size_t)wtri_off[i] + k) + 9], &global, 4);
    }
    for (size_t k = 0; k < f.v0.size(); ++k) {
      const uint32_t o = b.permutation[k];
      // BVH-order triangle (shading needs its vertices for barycentrics)
      put_tri(&h_tris[12 * ((size_t)tri_off[i] + k)], f.v0[o], f.v1[o], f.v2[o], 0);
      float d[12] = {f.n0[o].x, f.n0[o].y, f.n0[o].z, f.n1[o].x, f.n1[o].y, f.n1[o].z,
                     f.n2[o].x, f.n2[o].y, f.n2[o].z, 0.f,       0.f,       0.f};
      const uint32_t m = mat_off[i] + f.material[o];
      std::memcpy(&d[11], &m, 4);
      std::memcpy(&h_data[12 * ((size_t)tri_off[i] + k)], d, sizeof(d));
    }
    const std::vector<path_material> &sm = items[i].scene->materials;
    for (size_t k = 0; k < sm.size(); ++k) {
      h_mats[mat_off[i] + k] = to_dev(sm[k]);
    }
    for (size_t k = 0; k < f.light_v0.size(); ++k) {
      put_tri(&h_lights[12 * ((size_t)light_off[i] + k)], f.light_v0[k], f.light_v1[k],
              f.light_v2[k], 0);
      h_cdf[light_off[i] + k] = f.light_cdf[k];
    }
  }
  PG_TRY_CUDA(b_wnodes_.upload(h_nodes.data(), h_nodes.size() * sizeof(WideNode), stream_),
              "batch upload");
  PG_TRY_CUDA(b_wtris_.upload(h_wtris.data(), h_wtris.size() * 4, stream_), "batch upload");
  PG_TRY_CUDA(b_tris_.upload(h_tris.data(), h_tris.size() * 4, stream_), "batch upload");
  PG_TRY_CUDA(b_data_.upload(h_data.data(), h_data.size() * 4, stream_), "batch upload");
  b_mat_types_ = 0;
  for (const BatchItem &it : items) {
    for (const path_material &m : it.scene->materials) {
      b_mat_types_ |= 1u << (m.type & 31u);
    }
  }
  PG_TRY_CUDA(b_mats_.upload(h_mats.data(), h_mats.size() * sizeof(DevMaterial), stream_),
              "batch upload");
  PG_TRY_CUDA(b_lights_.upload(h_lights.data(), h_lights.size() * 4, stream_), "batch upload");
  PG_TRY_CUDA(b_cdf_.upload(h_cdf.data(), h_cdf.size() * 4, stream_), "batch upload");
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "batch upload");
  batch_.root.assign(n, 0);
  batch_.light_off.assign(n, 0);
  batch_.n_lights.assign(n, 0);
  batch_.n_tris.assign(n, 0);
  batch_.box.assign(n, {0.f, 0.f, 0.f, 0.f, 0.f, 0.f});
  for (size_t i = 0; i < n; ++i) {
    const size_t f = first_of[i];
    scene_box(flats[f], batch_.box[i].data(), batch_.box[i].data() + 3);
    batch_.root[i] = wides[f].nodes.empty() ? kEmptyRoot : node_off[f];
    batch_.light_off[i] = light_off[f];
    batch_.n_lights[i] = (uint32_t)flats[f].light_v0.size();
    batch_.n_tris[i] = (uint32_t)flats[f].v0.size();
  }
  batch_.n_wide_nodes = (uint32_t)nodes;
  batch_.total_tris = tris;
  batch_.key = key;
  batch_.sbvh = sb;
  batch_.gpu_build = gpu_build;
  batch_.build_seconds =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  batch_.valid = true;
  return Status::ok();
}

// Runs the batch's wavefront over sample ids [0, sample_limit) and, with
// images, sums every item's pixels into its output.  kernel_ms: event time
// from the first launch to the last.
Status Renderer::run_batch(const std::vector<BatchItem> &items, const path_settings &st,
                           const path_batch_tuning &tu, uint64_t sample_limit,
                           bool with_images, float *kernel_ms, uint32_t *launches) {
  const size_t n = items.size();
  if (num_sms_ == 0) {
    int dev = 0;
    PG_TRY_CUDA(cudaGetDevice(&dev), "device");
    PG_TRY_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev),
                "sm count");
  }
  if (tu.trace_min_blocks < 3 || tu.trace_min_blocks > 6 || tu.slots_log2 < 10 ||
      tu.slots_log2 > 26 || tu.shade_ctas_per_sm > 64 || tu.iterations_per_graph > 64) {
    return Status::err(PATH_ERR_ARGUMENT, "batch tuning out of range");
  }
  uint32_t max_spp = 0;
  std::vector<BatchScene> scenes(n);
  std::vector<WorkDiv> wds(n);
  std::vector<size_t> part_off(n), bgra_off(n);
  size_t part_floats = 0, bgra_bytes = 0;
  bool any_reduce = false;
  unsigned long long total = 0;
  for (size_t i = 0; i < n; ++i) {
    const BatchItem &it = items[i];
    BatchScene &b = scenes[i];
    std::memset(&b, 0, sizeof(b));
    std::memcpy(b.f2w, it.f2w, sizeof(b.f2w));
    b.x_dim = it.x_dim;
    b.y_dim = it.y_dim;
    b.spp = it.spp;
    b.sample_offset = it.sample_offset;
    b.root = batch_.root[i];
    b.light_off = batch_.light_off[i];
    b.n_lights = st.light_sampler == PATH_LIGHT_RANDOM_TRIANGLE ? batch_.n_lights[i] : 0u;
    for (int a = 0; a < 3; ++a) {
      b.cache_lo[a] = batch_.box[i][a];
      b.cache_inv[a] = 1.f / std::max(batch_.box[i][3 + a] - batch_.box[i][a], 1e-6f);
    }
    b.cache_cell = (uint32_t)i;
    b.first_sample = total;
    total += (unsigned long long)it.x_dim * it.y_dim * it.spp;
    if ((uint64_t)it.sample_offset + it.spp > 0xffffffffull) {
      return Status::err(PATH_ERR_ARGUMENT, "sample_offset + samples_per above 2^32 - 1");
    }
    max_spp = std::max(max_spp, it.sample_offset + it.spp);
    if (!make_workdiv(st.render_work_division, it.spp, it.x_dim, it.y_dim, wds[i])) {
      return Status::err(PATH_ERR_ARGUMENT, "invalid render work division settings");
    }
    if (wds[i].block_size > 256) {
      return Status::err(PATH_ERR_UNSUPPORTED, "render block_size above 256");
    }
    const size_t npix = (size_t)it.x_dim * it.y_dim;
    part_off[i] = part_floats;
    part_floats += (size_t)wds[i].num_sample_blocks * npix * 3;
    any_reduce = any_reduce || wds[i].num_sample_blocks > 1;
    bgra_off[i] = bgra_bytes;
    if (it.output.type == PATH_OUTPUT_BGRA) {
      bgra_bytes += npix * 4;
    }
  }
  const unsigned long long limit = std::min<unsigned long long>(total, sample_limit);
  if (st.rng == PATH_RNG_SOBEL) {
    Status ss = prepare_sobol(st.max_sample_size, max_spp);
    if (!ss.good()) {
      return ss;
    }
  }
  PG_TRY_CUDA(b_scenes_.upload(scenes.data(), n * sizeof(BatchScene), stream_), "scene table");
  // wavefront state for the whole batch
  const uint32_t n_slots =
      (uint32_t)std::min<unsigned long long>(limit, 1ull << tu.slots_log2);
  auto a256 = [](size_t v) { return (v + 255) & ~size_t(255); };
  const size_t f4 = a256((size_t)n_slots * 16), u2 = a256((size_t)n_slots * 8),
               u1 = a256((size_t)n_slots * 4);
  PG_TRY_CUDA(wf_slots_.ensure(7 * f4 + 2 * u2 + 2 * u1 + 2 * u1), "wavefront slots");
  PG_TRY_CUDA(wf_queues_.ensure(64), "wavefront queues");
  PG_TRY_CUDA(wf_samples_.ensure((size_t)limit * 12), "sample buffer");
  PG_TRY_CUDA(wf_host_.ensure(64), "staging");
  PG_TRY_CUDA(status_.ensure(4), "status word");
  PG_TRY_CUDA(counters_.ensure(24), "counters");
  PG_TRY_CUDA(cudaMemsetAsync(status_.get(), 0, 4, stream_), "status reset");
  PG_TRY_CUDA(cudaMemsetAsync(counters_.get(), 0, 24, stream_), "counter reset");
  if (with_images) {
    PG_TRY_CUDA(b_part_a_.ensure(std::max<size_t>(part_floats, 1) * 4), "partial sums");
    if (any_reduce) {
      PG_TRY_CUDA(b_part_b_.ensure(std::max<size_t>(part_floats, 1) * 4), "partial sums");
    }
    if (bgra_bytes > 0) {
      PG_TRY_CUDA(b_bgra_.ensure(bgra_bytes), "bgra buffer");
    }
  }

  RenderParams p;
  std::memset(&p, 0, sizeof(p));
  p.tris = b_tris_.as<const float4>();
  p.tri_data = b_data_.as<const float4>();
  p.wide_nodes = b_wnodes_.as<const uint4>();
  p.wide_tris = b_wtris_.as<const float4>();
  p.n_tris = (uint32_t)batch_.total_tris;
  p.n_wide_nodes = batch_.n_wide_nodes;
  p.materials = b_mats_.as<const DevMaterial>();
  p.light_tris = b_lights_.as<const float4>();
  p.light_cdf = b_cdf_.as<const float>();
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
  p.status = status_.as<uint32_t>();
  p.counters = counters_.as<unsigned long long>();
  const bool cached = cache_ != nullptr && cache_depth_ != 0;
  if (cached) {
    if (limit >= (1ull << 32)) {
      return Status::err(PATH_ERR_UNSUPPORTED, "more than 2^32 samples with the cache");
    }
    PG_TRY_CUDA(cache_q_.ensure((size_t)limit * 48), "cache queries");
    PG_TRY_CUDA(cache_beta_.ensure((size_t)limit * 12), "cache queries");
    PG_TRY_CUDA(cudaMemsetAsync(cache_beta_.get(), 0, (size_t)limit * 12, stream_),
                "cache queries");
    cached_samples_ = limit;
    if (cache_train_paths_ > 0) {
      // the training paths are independent of the frame: traced on a side
      // stream while the frame renders, once the batch's tables are resident
      if (side_stream_ == nullptr) {
        PG_TRY_CUDA(cudaStreamCreateWithFlags(&side_stream_, cudaStreamNonBlocking), "stream");
        PG_TRY_CUDA(cudaEventCreateWithFlags(&side_done_, cudaEventDisableTiming), "event");
      }
      PG_TRY_CUDA(cudaEventRecord(side_done_, stream_), "event");
      PG_TRY_CUDA(cudaStreamWaitEvent(side_stream_, side_done_, 0), "event");
      PG_TRY_CUDA(cache_records_.ensure((size_t)cache_train_paths_ * 64), "cache records");
      PG_TRY_CUDA(launch_nrc_paths_batch(p, b_scenes_.as<const BatchScene>(), (uint32_t)n,
                                         cache_train_paths_, frame_counter_++, cache_depth_,
                                         cache_records_.as<float>(), side_stream_),
                  "cache training paths");
      PG_TRY_CUDA(cudaEventRecord(side_done_, side_stream_), "event");
    }
    p.cache_depth = cache_depth_;
  }

  unsigned char *base = wf_slots_.as<unsigned char>();
  WaveParams w;
  std::memset(&w, 0, sizeof(w));
  w.P = p;
  w.o = reinterpret_cast<float4 *>(base);
  w.d = reinterpret_cast<float4 *>(base + f4);
  w.ld = reinterpret_cast<float4 *>(base + 2 * f4);
  w.mult = reinterpret_cast<float4 *>(base + 3 * f4);
  w.lmult = reinterpret_cast<float4 *>(base + 4 * f4);
  w.total = reinterpret_cast<float4 *>(base + 5 * f4);
  w.state = reinterpret_cast<uint4 *>(base + 6 * f4);
  w.hit_ext = reinterpret_cast<uint2 *>(base + 7 * f4);
  w.hit_light = reinterpret_cast<uint2 *>(base + 7 * f4 + u2);
  w.active[0] = reinterpret_cast<uint32_t *>(base + 7 * f4 + 2 * u2);
  w.active[1] = reinterpret_cast<uint32_t *>(base + 7 * f4 + 2 * u2 + u1);
  w.rays = reinterpret_cast<uint32_t *>(base + 7 * f4 + 2 * u2 + 2 * u1);
  w.q = wf_queues_.as<WaveQueues>();
  w.next_sample = reinterpret_cast<unsigned long long *>(wf_queues_.as<unsigned char>() + 32);
  w.first_sample = 0;
  w.total_samples = limit;
  w.sample_rgb = wf_samples_.as<float>();
  w.n_slots = n_slots;
  if (p.rng_uniform) {
    PG_TRY_CUDA(wf_rng_.ensure((size_t)n_slots * kRngStateWords * 4), "rng states");
    w.rng_state = wf_rng_.as<uint32_t>();
  }
  w.scenes = b_scenes_.as<const BatchScene>();
  w.n_scenes = (uint32_t)n;
  w.feat = work_features(b_mat_types_, p);
  if (cached) {
    w.cache_q = cache_q_.as<float>();
    w.cache_beta = cache_beta_.as<float>();
  }

  uint32_t *h = wf_host_.as<uint32_t>();
  std::memset(h, 0, 64);
  h[0] = n_slots;
  h[2] = n_slots;
  unsigned long long next = n_slots;
  std::memcpy(h + 8, &next, sizeof(next));
  const bool counting = st.count_work != 0;
  const uint32_t trace_grid =
      (uint32_t)num_sms_ *
      (uint32_t)wavefront_trace_blocks_per_sm(tu.trace_min_blocks, counting, 0);
  const uint32_t shade_grid = (uint32_t)num_sms_ * tu.shade_ctas_per_sm;
  const uint32_t k_iters = tu.iterations_per_graph + (tu.iterations_per_graph & 1u);

  // the iteration graph: k_iters x (trace, prep, shade), parity back to 0
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "pre-capture sync");
  PG_TRY_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture");
  cudaError_t ce = cudaSuccess;
  uint32_t parity = 0;
  for (uint32_t k = 0; k < k_iters && ce == cudaSuccess; ++k) {
    ce = launch_wavefront_trace(w, trace_grid, tu.trace_min_blocks, counting, stream_);
    if (ce == cudaSuccess) {
      ce = launch_wavefront_shade(w, parity, shade_grid, stream_);
    }
    parity ^= 1u;
  }
  cudaError_t ee = cudaStreamEndCapture(stream_, &graph);
  if (ce != cudaSuccess || ee != cudaSuccess) {
    if (graph) {
      cudaGraphDestroy(graph);
    }
    return cuda_status(ce != cudaSuccess ? ce : ee, "iteration graph capture");
  }
  ce = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) {
    return cuda_status(ce, "iteration graph instantiate");
  }
  struct ExecGuard {
    cudaGraphExec_t e;
    ~ExecGuard() {
      if (e) {
        cudaGraphExecDestroy(e);
      }
    }
  } guard{exec};

  PG_TRY_CUDA(cudaEventRecord(ev_start_, stream_), "event");
  PG_TRY_CUDA(cudaMemcpyAsync(wf_queues_.get(), h, 48, cudaMemcpyHostToDevice, stream_),
              "queue init");
  PG_TRY_CUDA(launch_wavefront_init(w, n_slots, stream_), "wavefront init");
  uint32_t nl = 1;
  volatile uint32_t *live = h + 12;
  for (uint32_t round = 0;; ++round) {
    PG_TRY_CUDA(cudaGraphLaunch(exec, stream_), "iteration graph");
    nl += 3 * k_iters;
    PG_TRY_CUDA(cudaMemcpyAsync(h + 12, &w.q->active[0], 4, cudaMemcpyDeviceToHost, stream_),
                "live count");
    PG_TRY_CUDA(cudaStreamSynchronize(stream_), "wavefront sync");
    if (*live == 0) {
      break;
    }
    if ((uint64_t)round * k_iters > 4ull * kMaxPathVertices + limit) {
      return Status::err(PATH_ERR_DEVICE_TIMEOUT, "batch wavefront did not drain");
    }
  }
  if (cached) {
    // the cache's prediction at every path's last vertex
    PG_TRY_CUDA(cache_pred_.ensure((size_t)limit * 12), "cache predictions");
    Status sc = cache_->infer(w.cache_q, (uint32_t)limit, cache_pred_.as<float>(), stream_,
                              w.cache_beta);
    if (!sc.good()) {
      return sc;
    }
    PG_TRY_CUDA(launch_nrc_apply(w.sample_rgb, w.cache_beta, cache_pred_.as<float>(), limit,
                                 stream_),
                "cache apply");
    nl += 2;
  }
  if (with_images) {
    // per-item sums + ReduceFloatRGB, captured as one graph
    std::vector<float *> final_rgb(n);
    cudaGraph_t sg = nullptr;
    PG_TRY_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture");
    cudaError_t se = cudaSuccess;
    uint32_t sum_launches = 0;
    for (size_t i = 0; i < n && se == cudaSuccess; ++i) {
      const BatchItem &it = items[i];
      const WorkDiv &wd = wds[i];
      const bool bgra = it.output.type == PATH_OUTPUT_BGRA;
      const size_t npix = (size_t)it.x_dim * it.y_dim;
      RenderParams ps = p;
      ps.x_dim = it.x_dim;
      ps.y_dim = it.y_dim;
      ps.spp = it.spp;
      ps.wd = wd;
      ps.out_rgb = b_part_a_.as<float>() + part_off[i];
      ps.out_bgra = bgra ? b_bgra_.as<uint8_t>() + bgra_off[i] : nullptr;
      ps.output_bgra = bgra ? 1u : 0u;
      ps.start_block = 0;
      ps.row_lo = 0;
      ps.row_hi = it.y_dim;
      se = launch_wavefront_sum(ps, w.sample_rgb + 3 * scenes[i].first_sample,
                                wd.total_blocks(), stream_);
      ++sum_launches;
      float *in = ps.out_rgb;
      float *other = b_part_b_.as<float>() + part_off[i];
      uint32_t factor = wd.num_sample_blocks;
      size_t elems = (size_t)factor * npix;
      while (factor != 1 && se == cudaSuccess) {
        ReduceParams rp;
        std::memset(&rp, 0, sizeof(rp));
        const uint32_t xd = (uint32_t)(elems / factor);
        if (!make_workdiv(st.reduce_work_division, factor, xd, 1, rp.wd)) {
          se = cudaErrorInvalidValue;
          break;
        }
        rp.in = in;
        rp.out = other;
        rp.reduction_factor = factor;
        rp.spp = it.spp;
        rp.output_bgra = bgra ? 1u : 0u;
        rp.out_bgra = ps.out_bgra;
        se = launch_reduce(rp, stream_);
        ++sum_launches;
        factor = rp.wd.num_sample_blocks;
        elems = (size_t)xd * factor;
        std::swap(in, other);
      }
      final_rgb[i] = in;
    }
    cudaError_t se2 = cudaStreamEndCapture(stream_, &sg);
    if (se != cudaSuccess || se2 != cudaSuccess) {
      if (sg) {
        cudaGraphDestroy(sg);
      }
      return cuda_status(se != cudaSuccess ? se : se2, "sum graph capture");
    }
    cudaGraphExec_t sx = nullptr;
    se = cudaGraphInstantiate(&sx, sg, 0);
    cudaGraphDestroy(sg);
    if (se != cudaSuccess) {
      return cuda_status(se, "sum graph instantiate");
    }
    ExecGuard sguard{sx};
    PG_TRY_CUDA(cudaGraphLaunch(sx, stream_), "sum graph");
    nl += sum_launches;
    PG_TRY_CUDA(cudaEventRecord(ev_stop_, stream_), "event");
    uint64_t d2h = 0;
    for (size_t i = 0; i < n; ++i) {
      const BatchItem &it = items[i];
      const size_t npix = (size_t)it.x_dim * it.y_dim;
      const bool bgra = it.output.type == PATH_OUTPUT_BGRA;
      const void *src = bgra ? static_cast<const void *>(b_bgra_.as<uint8_t>() + bgra_off[i])
                             : static_cast<const void *>(final_rgb[i]);
      const size_t bytes = bgra ? npix * 4 : npix * 12;
      PG_TRY_CUDA(cudaMemcpyAsync(it.output.data, src, bytes,
                                  it.output.on_device ? cudaMemcpyDeviceToDevice
                                                      : cudaMemcpyDeviceToHost,
                                  stream_),
                  "output copy");
      if (!it.output.on_device) {
        d2h += bytes;
      }
    }
    stats_.d2h_bytes = d2h;
    PG_TRY_CUDA(cudaStreamSynchronize(stream_), "batch sync");
  } else {
    PG_TRY_CUDA(cudaEventRecord(ev_stop_, stream_), "event");
    PG_TRY_CUDA(cudaStreamSynchronize(stream_), "batch sync");
  }
  float ms = 0.f;
  PG_TRY_CUDA(cudaEventElapsedTime(&ms, ev_start_, ev_stop_), "event");
  *kernel_ms = ms;
  *launches = nl;
  uint32_t status = 0;
  unsigned long long counts[3] = {0, 0, 0};
  PG_TRY_CUDA(cudaMemcpy(&status, status_.get(), 4, cudaMemcpyDeviceToHost), "status copy");
  if (counting) {
    PG_TRY_CUDA(cudaMemcpy(counts, counters_.get(), 24, cudaMemcpyDeviceToHost), "counters");
  }
  stats_.rays_traced = counts[0];
  stats_.nodes_visited = counts[1];
  stats_.triangles_tested = counts[2];
  stats_.device_status = status;
  if (status != 0) {
    return Status::err(PATH_ERR_DEVICE_TIMEOUT,
                       "kernel reported device status " + std::to_string(status));
  }
  return Status::ok();
}

Status Renderer::render_batch(const std::vector<BatchItem> &items, const path_settings &st,
                              const path_batch_tuning *tuning, double *seconds) {
  Status sc = check_batch(items, st);
  if (!sc.good()) {
    return sc;
  }
  Status s0 = init();
  if (!s0.good()) {
    return s0;
  }
  auto t0 = std::chrono::steady_clock::now();
  Status sp = prepare_batch(items, sbvh_of(st), st.gpu_build);
  if (!sp.good()) {
    return sp;
  }
  auto t1 = std::chrono::steady_clock::now();
  stats_ = path_render_stats{};
  float ms = 0.f;
  uint32_t launches = 0;
  Status sr = run_batch(items, st, resolved(tuning), ~0ull, true, &ms, &launches);
  auto t2 = std::chrono::steady_clock::now();
  stats_.seconds = std::chrono::duration<double>(t2 - t1).count();
  stats_.kernel_ms = ms;
  stats_.bvh_build_seconds = batch_.build_seconds;
  stats_.gpu_launches = launches;
  stats_.num_wide_nodes = batch_.n_wide_nodes;
  (void)t0;
  if (seconds) {
    *seconds = stats_.seconds;
  }
  return sr;
}

Status Renderer::render_batch_cached(const std::vector<BatchItem> &items,
                                     const path_settings &st, const path_batch_tuning *tuning,
                                     RadianceCache &cache, uint32_t cache_depth,
                                     uint32_t train_paths, uint32_t train_steps,
                                     double *seconds) {
  if (cache_depth == 0 || cache_depth > 64) {
    return Status::err(PATH_ERR_ARGUMENT, "cache_depth must be in [1, 64]");
  }
  if (items.size() > kMaxCacheCells) {
    return Status::err(PATH_ERR_UNSUPPORTED, "more than 4096 items in a cached batch");
  }
  Status sc = check_batch(items, st);
  if (!sc.good()) {
    return sc;
  }
  Status s0 = init();
  if (!s0.good()) {
    return s0;
  }
  auto t0 = std::chrono::steady_clock::now();
  Status sp = prepare_batch(items, sbvh_of(st), st.gpu_build);
  if (!sp.good()) {
    return sp;
  }
  auto t1 = std::chrono::steady_clock::now();
  // the batch's cache cells: every item's positions in a cell of its own
  cache.set_batch_cells();
  cache_ = &cache;
  cache_depth_ = cache_depth;
  cache_train_paths_ = train_steps > 0 ? train_paths : 0u;
  stats_ = path_render_stats{};
  float ms = 0.f;
  uint32_t launches = 0;
  Status sr = run_batch(items, st, resolved(tuning), ~0ull, true, &ms, &launches);
  const bool side = cache_train_paths_ > 0;
  cache_ = nullptr;
  cache_depth_ = 0;
  cache_train_paths_ = 0;
  if (side && side_done_ != nullptr) {
    PG_TRY_CUDA(cudaEventSynchronize(side_done_), "cache training paths");
    PG_TRY_CUDA(cudaGetLastError(), "cache training paths");
  }
  if (!sr.good()) {
    return sr;
  }
  if (train_paths > 0 && train_steps > 0) {
    const uint32_t per = std::max<uint32_t>(train_paths / train_steps, 1);
    for (uint32_t k = 0; k < train_steps; ++k) {
      const uint32_t first = k * per;
      if (first >= train_paths) {
        break;
      }
      const uint32_t cnt = std::min<uint32_t>(per, train_paths - first);
      Status st_train =
          cache.train(cache_records_.as<float>() + (size_t)first * 16, cnt, nullptr);
      if (!st_train.good()) {
        return st_train;
      }
    }
  }
  auto t2 = std::chrono::steady_clock::now();
  stats_.seconds = std::chrono::duration<double>(t2 - t1).count();
  stats_.kernel_ms = ms;
  stats_.bvh_build_seconds = batch_.build_seconds;
  stats_.gpu_launches = launches + (side ? 1u : 0u);
  stats_.num_wide_nodes = batch_.n_wide_nodes;
  (void)t0;
  if (seconds) {
    *seconds = stats_.seconds;
  }
  return Status::ok();
}

Status Renderer::autotune_batch(const std::vector<BatchItem> &items, const path_settings &st,
                                uint64_t sample_budget, path_batch_tuning *out) {
  Status sc = check_batch(items, st);
  if (!sc.good()) {
    return sc;
  }
  Status s0 = init();
  if (!s0.good()) {
    return s0;
  }
  Status sp = prepare_batch(items, sbvh_of(st), st.gpu_build);
  if (!sp.good()) {
    return sp;
  }
  stats_ = path_render_stats{};
  stats_.bvh_build_seconds = batch_.build_seconds;
  if (sample_budget == 0) {
    // twice the largest candidate's paths in flight, so that every
    // candidate refills its slots
    sample_budget = 1ull << 27;
  }
  path_settings quiet = st;
  quiet.count_work = 0;
  // candidates: paths in flight x trace occupancy x shade grid (trace CTAs
  // per SM other than 4 and shade grids below 4 CTAs per SM never won on
  // the batched workload)
  const uint32_t slots[] = {23, 24, 25, 26};
  const uint32_t mins[] = {4};
  const uint32_t shades[] = {4, 8};
  path_batch_tuning best = resolved(nullptr);
  float best_ms = -1.f;
  for (uint32_t sl : slots) {
    for (uint32_t mb : mins) {
      for (uint32_t sh : shades) {
        path_batch_tuning t = resolved(nullptr);
        t.slots_log2 = sl;
        t.trace_min_blocks = mb;
        t.shade_ctas_per_sm = sh;
        float ms = 0.f;
        uint32_t launches = 0;
        Status sr = run_batch(items, quiet, t, sample_budget, false, &ms, &launches);
        if (!sr.good()) {
          return sr;
        }
        if (best_ms < 0.f || ms < best_ms) {
          best_ms = ms;
          best = t;
        }
      }
    }
  }
  *out = best;
  return Status::ok();
}

} // namespace pg

// C ABI of the render path (include/path_gb300.h).
#include "path_gb300.h"

#include "cache_host.h"
#include "kernels.h"
#include "renderer.h"
#include "scene.h"
#include "sbvh.h"
#include "wide.h"
#include "settings.h"
#include "workdiv.h"

#include <curand.h>

#include <atomic>
#include <cstring>
#include <exception>
#include <new>
#include <string>
#include <vector>

struct path_scene {
  pg::Scene s;
};

struct path_renderer {
  pg::Renderer r;
};

namespace {

thread_local std::string g_last_error;
std::atomic<uint64_t> g_next_scene_id{1};

path_status fail(path_status code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

path_status from(const pg::Status &s) {
  if (s.good()) {
    g_last_error.clear();
    return PATH_OK;
  }
  return fail(s.code, s.message);
}

template <typename F> path_status guarded(F &&f) {
  try {
    return f();
  } catch (const std::bad_alloc &) {
    return fail(PATH_ERR_OOM, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(PATH_ERR_ARGUMENT, e.what());
  } catch (...) {
    return fail(PATH_ERR_ARGUMENT, "unknown error");
  }
}

pg::f3 load3(const float *p) { return pg::mk(p[0], p[1], p[2]); }

} // namespace

namespace pg {
// records the message path_last_error() returns (for entry points defined in
// other translation units)
path_status record_status(const Status &s) { return from(s); }
pg::Renderer &renderer_of(path_renderer *r) { return r->r; }
const pg::Scene &scene_of(const path_scene *s) { return s->s; }
} // namespace pg

extern "C" {

const char *path_last_error(void) { return g_last_error.c_str(); }

const char *path_version(void) {
  return "path_gb300 1.0 (sm_103a)";
}

path_status path_settings_default(path_settings *out) {
  if (!out) {
    return fail(PATH_ERR_ARGUMENT, "null settings");
  }
  pg::default_settings(*out);
  return PATH_OK;
}

path_status path_settings_load_yaml(const char *path, path_settings *out) {
  if (!path || !out) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    std::string err;
    if (!pg::settings_from_yaml_file(path, *out, err)) {
      return fail(err.rfind("cannot open", 0) == 0 ? PATH_ERR_IO : PATH_ERR_SCENE_PARSE, err);
    }
    return PATH_OK;
  });
}

path_status path_scene_create(path_scene **out) {
  if (!out) {
    return fail(PATH_ERR_ARGUMENT, "null output");
  }
  return guarded([&] {
    *out = new path_scene();
    (*out)->s.id = g_next_scene_id++;
    return PATH_OK;
  });
}

void path_scene_destroy(path_scene *scene) { delete scene; }

path_status path_scene_add_material(path_scene *scene, const path_material *m,
                                    uint32_t *material_idx) {
  if (!scene || !m) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  if (m->type > PATH_BSDF_GGX) {
    return fail(PATH_ERR_ARGUMENT, "unknown bsdf type");
  }
  return guarded([&] {
    if (material_idx) {
      *material_idx = (uint32_t)scene->s.materials.size();
    }
    scene->s.materials.push_back(*m);
    ++scene->s.version;
    return PATH_OK;
  });
}

path_status path_scene_set_material(path_scene *scene, uint32_t material_idx,
                                    const path_material *m) {
  if (!scene || !m) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  if (m->type > PATH_BSDF_GGX) {
    return fail(PATH_ERR_ARGUMENT, "unknown bsdf type");
  }
  if (material_idx >= scene->s.materials.size()) {
    return fail(PATH_ERR_ARGUMENT, "material index out of range");
  }
  scene->s.materials[material_idx] = *m;
  ++scene->s.material_version;
  return PATH_OK;
}

// TriangleConstructor::add_triangle (src/scene/triangle_constructor.cpp:14-30):
// face normals when none are given, and one emissive cluster per emissive
// triangle
path_status path_scene_add_mesh(path_scene *scene, const float *triangles,
                                const float *normals, const uint32_t *material_idx,
                                uint32_t n, const float *object_to_world) {
  if (!scene || (n > 0 && (!triangles || !material_idx))) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    pg::Scene &s = scene->s;
    for (uint32_t i = 0; i < n; ++i) {
      if (material_idx[i] >= s.materials.size()) {
        return fail(PATH_ERR_ARGUMENT, "material index out of range");
      }
    }
    uint32_t start = s.n_tris();
    s.tris.insert(s.tris.end(), triangles, triangles + 9 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) {
      if (normals) {
        s.normals.insert(s.normals.end(), normals + 9 * (size_t)i, normals + 9 * (size_t)i + 9);
      } else {
        const float *t = triangles + 9 * (size_t)i;
        pg::f3 nn = pg::normalize(pg::cross(load3(t + 3) - load3(t), load3(t + 6) - load3(t)));
        for (int k = 0; k < 3; ++k) {
          s.normals.push_back(nn.x);
          s.normals.push_back(nn.y);
          s.normals.push_back(nn.z);
        }
      }
      s.tri_material.push_back(material_idx[i]);
      if (pg::is_emissive(s.materials[material_idx[i]])) {
        s.clusters.push_back(material_idx[i]);
        s.clusters.push_back(start + i);
        s.clusters.push_back(start + i + 1);
      }
    }
    s.mesh_ends.push_back(s.n_tris());
    s.cluster_ends_per_mesh.push_back((uint32_t)(s.clusters.size() / 3));
    pg::affine xf = pg::identity_affine();
    if (object_to_world) {
      std::memcpy(xf.m, object_to_world, sizeof(xf.m));
    }
    s.instances.push_back(xf);
    s.instance_mesh.push_back((uint32_t)s.mesh_ends.size() - 1);
    ++s.version;
    return PATH_OK;
  });
}

path_status path_scene_load_xml(const char *path, float width_height_ratio,
                                path_scene **out, float *film_to_world) {
  if (!path || !out) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    auto *sc = new path_scene();
    sc->s.id = g_next_scene_id++;
    pg::affine f2w;
    std::string err;
    if (!pg::load_scene_xml(path, width_height_ratio, sc->s, f2w, err)) {
      delete sc;
      return fail(err.rfind("cannot open", 0) == 0 ? PATH_ERR_IO : PATH_ERR_SCENE_PARSE, err);
    }
    if (film_to_world) {
      std::memcpy(film_to_world, f2w.m, sizeof(f2w.m));
    }
    *out = sc;
    return PATH_OK;
  });
}

path_status path_camera_transform(const float *look, const float *up, const float *pos,
                                  float height_angle_deg, float width_height_ratio,
                                  float *film_to_world) {
  if (!look || !up || !pos || !film_to_world) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  pg::affine a = pg::camera_transform(load3(look), load3(up), load3(pos), height_angle_deg,
                                      width_height_ratio);
  std::memcpy(film_to_world, a.m, sizeof(a.m));
  return PATH_OK;
}

path_status path_scene_sizes(const path_scene *scene, uint32_t *sizes) {
  if (!scene || !sizes) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  const pg::Scene &s = scene->s;
  sizes[0] = s.n_tris();
  sizes[1] = (uint32_t)s.mesh_ends.size();
  sizes[2] = (uint32_t)s.instances.size();
  sizes[3] = (uint32_t)(s.clusters.size() / 3);
  sizes[4] = (uint32_t)s.materials.size();
  return PATH_OK;
}

path_status path_scene_export(const path_scene *scene, float *triangles, float *normals,
                              uint32_t *tri_material, uint32_t *mesh_ends,
                              uint32_t *cluster_ends_per_mesh, float *instance_xforms,
                              uint32_t *instance_mesh, uint32_t *clusters,
                              path_material *materials) {
  if (!scene) {
    return fail(PATH_ERR_ARGUMENT, "null scene");
  }
  const pg::Scene &s = scene->s;
  auto put = [](void *dst, const void *src, size_t bytes) {
    if (dst && bytes) {
      std::memcpy(dst, src, bytes);
    }
  };
  put(triangles, s.tris.data(), s.tris.size() * 4);
  put(normals, s.normals.data(), s.normals.size() * 4);
  put(tri_material, s.tri_material.data(), s.tri_material.size() * 4);
  put(mesh_ends, s.mesh_ends.data(), s.mesh_ends.size() * 4);
  put(cluster_ends_per_mesh, s.cluster_ends_per_mesh.data(), s.cluster_ends_per_mesh.size() * 4);
  for (size_t i = 0; i < s.instances.size() && instance_xforms; ++i) {
    std::memcpy(instance_xforms + 12 * i, s.instances[i].m, 48);
  }
  put(instance_mesh, s.instance_mesh.data(), s.instance_mesh.size() * 4);
  put(clusters, s.clusters.data(), s.clusters.size() * 4);
  put(materials, s.materials.data(), s.materials.size() * sizeof(path_material));
  return PATH_OK;
}

path_status path_renderer_create(path_renderer **out) {
  if (!out) {
    return fail(PATH_ERR_ARGUMENT, "null output");
  }
  return guarded([&] {
    *out = new path_renderer();
    return PATH_OK;
  });
}

void path_renderer_destroy(path_renderer *renderer) { delete renderer; }

path_status path_render(path_renderer *renderer, uint32_t exec_model,
                        const path_sample_spec *sample_spec, const path_output *output,
                        const path_scene *scene, uint32_t samples_per,
                        const path_settings *settings, uint32_t show_progress,
                        double *seconds) {
  (void)show_progress;
  if (!renderer || !sample_spec || !output || !scene || !settings) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  if (exec_model != PATH_EXEC_GPU) {
    return fail(PATH_ERR_UNSUPPORTED,
                "this library implements the GPU execution model only; there is no "
                "CPU fallback");
  }
  return guarded([&] {
    return from(renderer->r.render(*sample_spec, *output, scene->s, samples_per, *settings,
                                   seconds));
  });
}

struct path_cache {
  pg::RadianceCache c;
  pg::DeviceBuffer in, out;
};

path_status path_cache_create(uint32_t seed, float learning_rate, path_cache **out) {
  if (!out) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&]() -> path_status {
    auto *c = new path_cache();
    path_status st = from(c->c.init(seed, learning_rate));
    if (st != PATH_OK) {
      delete c;
      return st;
    }
    *out = c;
    return PATH_OK;
  });
}

void path_cache_destroy(path_cache *cache) { delete cache; }

path_status path_cache_set_bounds(path_cache *cache, const float *lo, const float *hi) {
  if (!cache || !lo || !hi) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  cache->c.set_bounds(lo, hi);
  return PATH_OK;
}

path_status path_cache_set_ema(path_cache *cache, float decay) {
  if (!cache) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] { return from(cache->c.set_ema(decay)); });
}

path_status path_cache_use_batch_cells(path_cache *cache) {
  if (!cache) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  cache->c.set_batch_cells();
  return PATH_OK;
}

path_status path_cache_query(path_cache *cache, const float *queries, uint32_t n, float *out) {
  if (!cache || (n > 0 && (!queries || !out))) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&]() -> path_status {
    cudaStream_t s = cache->c.stream();
    cudaError_t e;
    if ((e = cache->in.upload(queries, (size_t)n * 48, s)) != cudaSuccess ||
        (e = cache->out.ensure((size_t)std::max<uint32_t>(n, 1) * 12)) != cudaSuccess) {
      return from(pg::cuda_status(e, "cache query"));
    }
    path_status st = from(cache->c.infer(cache->in.as<float>(), n, cache->out.as<float>(), s));
    if (st != PATH_OK) {
      return st;
    }
    if ((e = cudaMemcpyAsync(out, cache->out.get(), (size_t)n * 12, cudaMemcpyDeviceToHost,
                             s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
      return from(pg::cuda_status(e, "cache query"));
    }
    return PATH_OK;
  });
}

path_status path_cache_train(path_cache *cache, const float *records, uint32_t n,
                             uint32_t apply_update, float *loss) {
  if (!cache || (n > 0 && !records)) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&]() -> path_status {
    cudaError_t e = cache->in.upload(records, (size_t)n * 64, cache->c.stream());
    if (e != cudaSuccess) {
      return from(pg::cuda_status(e, "cache train"));
    }
    return from(apply_update ? cache->c.train(cache->in.as<float>(), n, loss)
                             : cache->c.gradients(cache->in.as<float>(), n, loss));
  });
}

path_status path_cache_access(path_cache *cache, float *weights, float *table,
                              float *grad_weights, float *grad_table, uint32_t set) {
  if (!cache) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  if (set && (grad_weights || grad_table)) {
    return fail(PATH_ERR_ARGUMENT, "gradients cannot be set");
  }
  return guarded([&] {
    return from(cache->c.access(weights, table, grad_weights, grad_table, set != 0));
  });
}

path_status path_render_cached(path_renderer *renderer, path_cache *cache,
                               const path_sample_spec *sample_spec, const path_output *output,
                               const path_scene *scene, uint32_t samples_per,
                               const path_settings *settings, uint32_t cache_depth,
                               uint32_t train_paths, uint32_t train_steps, double *seconds) {
  if (!renderer || !cache || !sample_spec || !output || !scene || !settings) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    return from(renderer->r.render_cached(*sample_spec, *output, scene->s, samples_per,
                                          *settings, cache->c, cache_depth, train_paths,
                                          train_steps, seconds));
  });
}

path_status path_cache_frame_queries(const path_renderer *renderer, uint32_t max_n,
                                     uint32_t stride, float *queries, float *throughput,
                                     uint32_t *n_out) {
  if (!renderer || !queries || !throughput || !n_out) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    return from(renderer->r.cached_frame_queries(max_n, stride, queries, throughput, n_out));
  });
}

path_status path_debug_tc_gemm(const uint16_t *a, const uint16_t *b, uint32_t k, uint32_t n,
                               float *d) {
  if (!a || !b || !d) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  if (k % 16 != 0 || n % 16 != 0 || k < 16 || n < 16 || k > 128 || n > 128) {
    return fail(PATH_ERR_ARGUMENT, "k and n must be multiples of 16 in [16, 128]");
  }
  return guarded([&]() -> path_status {
    pg::DeviceBuffer da, db, dd, derr;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaSuccess;
    uint32_t err = 0;
    if ((e = da.upload(a, (size_t)128 * k * 2, s)) != cudaSuccess ||
        (e = db.upload(b, (size_t)n * k * 2, s)) != cudaSuccess ||
        (e = dd.ensure((size_t)128 * n * 4)) != cudaSuccess ||
        (e = derr.upload(&err, 4, s)) != cudaSuccess ||
        (e = pg::launch_tc_gemm(da.get(), db.get(), dd.as<float>(), k, n, derr.as<uint32_t>(),
                                s)) != cudaSuccess ||
        (e = cudaMemcpy(d, dd.get(), (size_t)128 * n * 4, cudaMemcpyDeviceToHost)) !=
            cudaSuccess ||
        (e = cudaMemcpy(&err, derr.get(), 4, cudaMemcpyDeviceToHost)) != cudaSuccess) {
      return from(pg::cuda_status(e, "tensor-core test"));
    }
    if (err != 0) {
      return fail(PATH_ERR_DEVICE_TIMEOUT, "tensor-core MMA did not complete");
    }
    return PATH_OK;
  });
}

path_status path_debug_tc_wait_timeout(uint32_t polls) {
  if (polls == 0) {
    return fail(PATH_ERR_ARGUMENT, "polls must be positive");
  }
  return guarded([&]() -> path_status {
    pg::DeviceBuffer da, db, dd, derr;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaSuccess;
    uint32_t err = 0;
    if ((e = da.ensure((size_t)128 * 16 * 2)) != cudaSuccess ||
        (e = db.ensure((size_t)16 * 16 * 2)) != cudaSuccess ||
        (e = cudaMemset(da.get(), 0, (size_t)128 * 16 * 2)) != cudaSuccess ||
        (e = cudaMemset(db.get(), 0, (size_t)16 * 16 * 2)) != cudaSuccess ||
        (e = dd.ensure((size_t)128 * 16 * 4)) != cudaSuccess ||
        (e = derr.upload(&err, 4, s)) != cudaSuccess ||
        (e = pg::launch_tc_gemm(da.get(), db.get(), dd.as<float>(), 16, 16,
                                derr.as<uint32_t>(), s, polls, false)) != cudaSuccess ||
        (e = cudaMemcpy(&err, derr.get(), 4, cudaMemcpyDeviceToHost)) != cudaSuccess) {
      return from(pg::cuda_status(e, "tensor-core wait test"));
    }
    if (err != 0) {
      return fail(PATH_ERR_DEVICE_TIMEOUT, "tensor-core wait gave up");
    }
    return PATH_OK;
  });
}

path_status path_render_adjoint(path_renderer *renderer, const path_sample_spec *sample_spec,
                                const path_scene *scene, uint32_t samples_per,
                                const path_settings *settings, const float *d_image,
                                uint32_t d_image_on_device, double *d_params,
                                double *seconds) {
  if (!renderer || !sample_spec || !scene || !settings || !d_image || !d_params) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    return from(renderer->r.render_adjoint(*sample_spec, scene->s, samples_per, *settings,
                                           d_image, d_image_on_device != 0, d_params,
                                           seconds));
  });
}

static path_status batch_items(const path_batch_item *items, uint32_t n,
                               std::vector<pg::BatchItem> &out) {
  out.resize(n);
  for (uint32_t i = 0; i < n; ++i) {
    if (!items[i].scene) {
      return fail(PATH_ERR_ARGUMENT, "batch item without scene");
    }
    pg::BatchItem &b = out[i];
    b.scene = &items[i].scene->s;
    b.x_dim = items[i].x_dim;
    b.y_dim = items[i].y_dim;
    b.spp = items[i].samples_per;
    b.sample_offset = items[i].sample_offset;
    std::memcpy(b.f2w, items[i].film_to_world, sizeof(b.f2w));
    b.output = items[i].output;
  }
  return PATH_OK;
}

path_status path_render_batch(path_renderer *renderer, const path_batch_item *items,
                              uint32_t n_items, const path_settings *settings,
                              const path_batch_tuning *tuning, double *seconds) {
  if (!renderer || (n_items > 0 && !items) || !settings) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    std::vector<pg::BatchItem> v;
    path_status s = batch_items(items, n_items, v);
    if (s != PATH_OK) {
      return s;
    }
    return from(renderer->r.render_batch(v, *settings, tuning, seconds));
  });
}

path_status path_render_batch_cached(path_renderer *renderer, path_cache *cache,
                                     const path_batch_item *items, uint32_t n_items,
                                     const path_settings *settings,
                                     const path_batch_tuning *tuning, uint32_t cache_depth,
                                     uint32_t train_paths, uint32_t train_steps,
                                     double *seconds) {
  if (!renderer || !cache || (n_items > 0 && !items) || !settings) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    std::vector<pg::BatchItem> v;
    path_status s = batch_items(items, n_items, v);
    if (s != PATH_OK) {
      return s;
    }
    return from(renderer->r.render_batch_cached(v, *settings, tuning, cache->c, cache_depth,
                                                train_paths, train_steps, seconds));
  });
}

path_status path_batch_autotune(path_renderer *renderer, const path_batch_item *items,
                                uint32_t n_items, const path_settings *settings,
                                uint64_t sample_budget, path_batch_tuning *out) {
  if (!renderer || (n_items > 0 && !items) || !settings || !out) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    std::vector<pg::BatchItem> v;
    path_status s = batch_items(items, n_items, v);
    if (s != PATH_OK) {
      return s;
    }
    return from(renderer->r.autotune_batch(v, *settings, sample_budget, out));
  });
}

path_status path_renderer_stats(const path_renderer *renderer, path_render_stats *out) {
  if (!renderer || !out) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  *out = renderer->r.stats();
  return PATH_OK;
}

path_status path_wide_build(const float *triangles, uint32_t n, const path_settings *settings,
                            uint32_t *sizes, void *nodes, uint32_t *leaf_refs,
                            uint32_t *permutation) {
  if ((n > 0 && !triangles) || !settings || !sizes) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    std::vector<pg::f3> a(n), b(n), c(n);
    for (uint32_t i = 0; i < n; ++i) {
      a[i] = load3(triangles + 9 * (size_t)i);
      b[i] = load3(triangles + 9 * (size_t)i + 3);
      c[i] = load3(triangles + 9 * (size_t)i + 6);
    }
    pg::SBVHSettings sb;
    sb.overlap_threshold = settings->overlap_threshold;
    sb.use_spatial_splits = settings->use_spatial_splits != 0;
    sb.traversal_per_intersect_cost = settings->traversal_per_intersect_cost;
    sb.target_objects = settings->target_objects;
    pg::BinaryBVH bvh = pg::build_sbvh(a.data(), b.data(), c.data(), n, sb);
    pg::WideBVH wide = pg::build_wide(bvh);
    sizes[0] = (uint32_t)wide.nodes.size();
    sizes[1] = (uint32_t)wide.tri_index.size();
    sizes[2] = wide.depth;
    if (nodes && !wide.nodes.empty()) {
      std::memcpy(nodes, wide.nodes.data(), wide.nodes.size() * sizeof(pg::WideNode));
    }
    if (leaf_refs && !wide.tri_index.empty()) {
      std::memcpy(leaf_refs, wide.tri_index.data(), wide.tri_index.size() * 4);
    }
    if (permutation && n > 0) {
      std::memcpy(permutation, bvh.permutation.data(), (size_t)n * 4);
    }
    return PATH_OK;
  });
}

path_status path_sbvh_build(const float *triangles, uint32_t n, const path_settings *settings,
                            uint32_t *sizes, uint32_t *node_words, float *node_aabbs,
                            uint32_t *extra_idxs, uint32_t *permutation) {
  if ((n > 0 && !triangles) || !settings || !sizes) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    std::vector<pg::f3> a(n), b(n), c(n);
    for (uint32_t i = 0; i < n; ++i) {
      a[i] = load3(triangles + 9 * (size_t)i);
      b[i] = load3(triangles + 9 * (size_t)i + 3);
      c[i] = load3(triangles + 9 * (size_t)i + 6);
    }
    pg::SBVHSettings sb;
    sb.overlap_threshold = settings->overlap_threshold;
    sb.use_spatial_splits = settings->use_spatial_splits != 0;
    sb.traversal_per_intersect_cost = settings->traversal_per_intersect_cost;
    sb.target_objects = settings->target_objects;
    pg::BinaryBVH bvh = pg::build_sbvh(a.data(), b.data(), c.data(), n, sb);
    sizes[0] = (uint32_t)bvh.nodes.size();
    sizes[1] = (uint32_t)bvh.extra_idxs.size();
    for (size_t i = 0; i < bvh.nodes.size(); ++i) {
      if (node_words) {
        node_words[2 * i] = bvh.nodes[i].w0;
        node_words[2 * i + 1] = bvh.nodes[i].w1;
      }
      if (node_aabbs) {
        const pg::box &x = bvh.nodes[i].aabb;
        float v[6] = {x.lo.x, x.lo.y, x.lo.z, x.hi.x, x.hi.y, x.hi.z};
        std::memcpy(node_aabbs + 6 * i, v, sizeof(v));
      }
    }
    if (extra_idxs && !bvh.extra_idxs.empty()) {
      std::memcpy(extra_idxs, bvh.extra_idxs.data(), bvh.extra_idxs.size() * 4);
    }
    if (permutation && n > 0) {
      std::memcpy(permutation, bvh.permutation.data(), (size_t)n * 4);
    }
    return PATH_OK;
  });
}

path_status path_intersect(path_renderer *renderer, const float *triangles,
                           uint32_t n_triangles, const float *rays, uint32_t n_rays,
                           const path_settings *settings, int32_t *idx_out, float *t_out) {
  if (!renderer || (n_triangles > 0 && !triangles) || (n_rays > 0 && (!rays || !idx_out || !t_out)) ||
      !settings) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    return from(renderer->r.intersect(triangles, n_triangles, rays, n_rays, *settings, idx_out,
                                      t_out));
  });
}

static path_status sobol_common(uint32_t dimension_bound, uint32_t count, float *out,
                                bool use_curand) {
  if (!out || dimension_bound == 0 || dimension_bound > 20000) {
    return fail(PATH_ERR_ARGUMENT, "bad Sobol table arguments");
  }
  return guarded([&] {
    curandDirectionVectors32_t *vecs = nullptr;
    unsigned *scr = nullptr;
    if (curandGetDirectionVectors32(&vecs, CURAND_SCRAMBLED_DIRECTION_VECTORS_32_JOEKUO6) !=
            CURAND_STATUS_SUCCESS ||
        curandGetScrambleConstants32(&scr) != CURAND_STATUS_SUCCESS) {
      return fail(PATH_ERR_CUDA, "cuRAND direction vectors unavailable");
    }
    pg::DeviceBuffer d_dirs, d_scr, d_out;
    size_t n = (size_t)dimension_bound * count;
    pg::Status st = pg::cuda_status(d_dirs.upload(vecs, (size_t)dimension_bound * 128, 0), "dirs");
    if (st.good()) {
      st = pg::cuda_status(d_scr.upload(scr, (size_t)dimension_bound * 4, 0), "scramble");
    }
    if (st.good()) {
      st = pg::cuda_status(d_out.ensure(n * 4), "table");
    }
    if (st.good()) {
      st = pg::cuda_status(
          use_curand ? pg::launch_sobol_curand(d_dirs.as<uint32_t>(), d_scr.as<uint32_t>(),
                                               dimension_bound, count, d_out.as<float>(), 0)
                     : pg::launch_sobol_table(d_dirs.as<uint32_t>(), d_scr.as<uint32_t>(),
                                              dimension_bound, count, d_out.as<float>(), 0),
          "sobol kernel");
    }
    if (st.good() && n > 0) {
      st = pg::cuda_status(cudaMemcpy(out, d_out.get(), n * 4, cudaMemcpyDeviceToHost),
                           "sobol copy");
    }
    return from(st);
  });
}

path_status path_sobol_table(uint32_t dimension_bound, uint32_t count, float *out) {
  return sobol_common(dimension_bound, count, out, false);
}

path_status path_sobol_table_curand(uint32_t dimension_bound, uint32_t count, float *out) {
  return sobol_common(dimension_bound, count, out, true);
}

path_status path_debug_sobol_draws(uint32_t mode, uint32_t n_paths, uint32_t spp,
                                   uint32_t draws, float *ms, uint32_t *checksum) {
  if (!ms || !checksum || mode > 2 || spp == 0 || spp > (1u << 20) || n_paths == 0 ||
      n_paths > (1u << 28) || draws == 0 || draws > 4096) {
    return fail(PATH_ERR_ARGUMENT, "bad Sobol draw arguments");
  }
  return guarded([&] {
    const uint32_t bound = 256;
    curandDirectionVectors32_t *vecs = nullptr;
    unsigned *scr = nullptr;
    if (curandGetDirectionVectors32(&vecs, CURAND_SCRAMBLED_DIRECTION_VECTORS_32_JOEKUO6) !=
            CURAND_STATUS_SUCCESS ||
        curandGetScrambleConstants32(&scr) != CURAND_STATUS_SUCCESS) {
      return fail(PATH_ERR_CUDA, "cuRAND direction vectors unavailable");
    }
    pg::DeviceBuffer d_dirs, d_scr, d_table, d_out;
    pg::Status st = pg::cuda_status(d_dirs.upload(vecs, (size_t)bound * 128, 0), "dirs");
    if (st.good()) {
      st = pg::cuda_status(d_scr.upload(scr, (size_t)bound * 4, 0), "scramble");
    }
    if (st.good()) {
      st = pg::cuda_status(d_table.ensure((size_t)bound * spp * 4), "table");
    }
    if (st.good()) {
      st = pg::cuda_status(d_out.ensure((size_t)n_paths * 4), "out");
    }
    if (st.good()) {
      st = pg::cuda_status(pg::launch_sobol_table(d_dirs.as<uint32_t>(), d_scr.as<uint32_t>(),
                                                  bound, spp, d_table.as<float>(), 0),
                           "sobol table");
    }
    int dev = 0, sms = 0;
    if (st.good()) {
      st = pg::cuda_status(cudaGetDevice(&dev), "device");
    }
    if (st.good()) {
      st = pg::cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                           "sm count");
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (st.good()) {
      st = pg::cuda_status(cudaEventCreate(&e0), "event");
    }
    if (st.good()) {
      st = pg::cuda_status(cudaEventCreate(&e1), "event");
    }
    const int reps = 3;
    for (int r = -1; st.good() && r < reps; ++r) {
      if (r == 0) {
        st = pg::cuda_status(cudaEventRecord(e0, 0), "event");
      }
      if (st.good()) {
        st = pg::cuda_status(pg::launch_sobol_draws((int)mode, d_table.as<float>(),
                                                    d_dirs.as<uint32_t>(),
                                                    d_scr.as<uint32_t>(), bound, spp, n_paths,
                                                    draws, (uint32_t)sms * 8, d_out.as<float>(),
                                                    0),
                             "sobol draws");
      }
    }
    if (st.good()) {
      st = pg::cuda_status(cudaEventRecord(e1, 0), "event");
    }
    if (st.good()) {
      st = pg::cuda_status(cudaEventSynchronize(e1), "event");
    }
    float t = 0.f;
    if (st.good()) {
      cudaEventElapsedTime(&t, e0, e1);
      *ms = t / reps;
      std::vector<uint32_t> h(n_paths);
      st = pg::cuda_status(cudaMemcpy(h.data(), d_out.get(), (size_t)n_paths * 4,
                                      cudaMemcpyDeviceToHost),
                           "copy");
      uint32_t c = 0;
      for (uint32_t v : h) {
        c = c * 31u + v;
      }
      *checksum = c;
    }
    if (e0) {
      cudaEventDestroy(e0);
    }
    if (e1) {
      cudaEventDestroy(e1);
    }
    return from(st);
  });
}

path_status path_debug_pmath(uint32_t fn, const float *x, const float *y, float *out,
                             uint32_t n) {
  if (!x || !out || (fn == 4 && !y)) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  return guarded([&] {
    pg::DeviceBuffer dx, dy, dout;
    pg::Status st = pg::cuda_status(dx.upload(x, (size_t)n * 4, 0), "x");
    if (st.good() && y) {
      st = pg::cuda_status(dy.upload(y, (size_t)n * 4, 0), "y");
    }
    if (st.good()) {
      st = pg::cuda_status(dout.ensure((size_t)n * 4), "out");
    }
    if (st.good()) {
      st = pg::cuda_status(pg::launch_pmath(fn, dx.as<float>(), y ? dy.as<float>() : nullptr,
                                            dout.as<float>(), n, 0),
                           "pmath kernel");
    }
    if (st.good() && n > 0) {
      st = pg::cuda_status(cudaMemcpy(out, dout.get(), (size_t)n * 4, cudaMemcpyDeviceToHost),
                           "copy");
    }
    return from(st);
  });
}

void path_debug_set_device_alloc_cap(uint64_t bytes) { pg::set_device_alloc_cap(bytes); }

path_status path_debug_bsdf(const path_material *material, uint32_t op, const float *in,
                            uint32_t n, float *out) {
  if (!material || !in || !out || op > 2 || material->type > PATH_BSDF_GGX) {
    return fail(PATH_ERR_ARGUMENT, "bad BSDF probe arguments");
  }
  return guarded([&] {
    const size_t out_floats = op == 0 ? 3 : op == 1 ? 6 : 1;
    pg::DevMaterial dm = pg::to_dev(*material);
    pg::DeviceBuffer dmat, din, dout;
    pg::Status st = pg::cuda_status(dmat.upload(&dm, sizeof(dm), 0), "material");
    if (st.good()) {
      st = pg::cuda_status(din.upload(in, (size_t)n * 36, 0), "records");
    }
    if (st.good()) {
      st = pg::cuda_status(dout.ensure((size_t)n * out_floats * 4 + 4), "out");
    }
    if (st.good()) {
      st = pg::cuda_status(pg::launch_bsdf(dmat.as<pg::DevMaterial>(), op, din.as<float>(), n,
                                           dout.as<float>(), 0),
                           "BSDF kernel");
    }
    if (st.good() && n > 0) {
      st = pg::cuda_status(
          cudaMemcpy(out, dout.get(), (size_t)n * out_floats * 4, cudaMemcpyDeviceToHost),
          "copy");
    }
    return from(st);
  });
}

path_status path_work_division(const path_work_division_settings *settings,
                               uint32_t samples_per, uint32_t x_dim, uint32_t y_dim,
                               uint32_t *out) {
  if (!settings || !out) {
    return fail(PATH_ERR_ARGUMENT, "null argument");
  }
  pg::WorkDiv w;
  if (!pg::make_workdiv(*settings, samples_per, x_dim, y_dim, w)) {
    return fail(PATH_ERR_ARGUMENT, "invalid work division settings");
  }
  const uint32_t v[11] = {w.block_size, w.base_samples_per_thread, w.n_threads_per_unit_extra,
                          w.sample_block_size, w.x_block_size, w.y_block_size,
                          w.num_sample_blocks, w.num_x_blocks, w.num_y_blocks, w.x_dim,
                          w.y_dim};
  std::memcpy(out, v, sizeof(v));
  return PATH_OK;
}

} // extern "C"

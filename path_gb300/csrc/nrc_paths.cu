// Training data of the radiance cache: full-length paths traced from random
// pixels with the integrator of the render (8-wide BVH), each contributing
// its vertex at the depth where the render's paths end into the cache: its
// query (position, direction towards the previous vertex, shading normal,
// albedo) and, as the target, the radiance its path gathered after that
// vertex's emission divided by the path throughput at the vertex -- a
// one-sample estimate of exactly what the render asks the cache for there,
// with the bounces a path has left at that depth.  (A vertex at another
// depth has a different number of bounces left, so its target estimates a
// different quantity: mixing depths biased the cache low.)  A path that
// ends before that depth gives its last vertex.  Compiled with --fmad=false
// like the render kernels.
#include "integrator.cuh"

namespace pg {
namespace dev {
namespace {

constexpr uint32_t kMaxRecordVertices = 16;

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  // integer finaliser of MurmurHash3 (Appleby)
  x ^= x >> 16;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  x *= 0xc2b2ae35u;
  x ^= x >> 16;
  return x;
}

// scenes != nullptr: a batch; each path takes a random scene of it and
// records its positions in that scene's cell of the cache
template <bool kUniform>
__global__ void __launch_bounds__(128) k_nrc_paths(const RenderParams P, const BatchScene *scenes,
                                                   uint32_t n_scenes, uint32_t n,
                                                   uint32_t frame, uint32_t depth,
                                                   float *records) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  const uint32_t h0 = mix32(i * 0x9e3779b9u ^ mix32(frame + 0x632be5abu));
  Camera cam = camera_of(P);
  LightSet lights = lights_of(P);
  uint32_t root = 0;
  const BatchScene *scene = nullptr;
  if (scenes != nullptr) {
    scene = scenes + mix32(h0 ^ 0x5bd1e995u) % n_scenes;
    cam.f2w = scene->f2w;
    cam.x_dim = scene->x_dim;
    cam.y_dim = scene->y_dim;
    cam.spp = scene->spp;
    cam.sample_offset = scene->sample_offset;
    lights = lights_of(P, *scene);
    root = scene->root;
  }
  const uint32_t n_pix = cam.x_dim * cam.y_dim;
  const uint32_t pixel = h0 % n_pix;
  const uint32_t x = pixel % cam.x_dim, y = pixel / cam.x_dim;
  const uint32_t smp = mix32(h0) % cam.spp;
  PathStateT<kUniform> s;
  uint32_t xw[kUniform ? kXorwowWords : 1];
  path_begin_cam(P, cam, smp, x, y, s, xw, 1);
  float q[kMaxRecordVertices][12];
  rgb gathered[kMaxRecordVertices], beta[kMaxRecordVertices];
  uint32_t nv = 0;
  Counts cnt = {0, 0, 0};
  while (true) {
    Hit lh, nh;
    step_hits<kTravWide, false>(P, s, false, x, cnt, lh, nh, root);
    const rgb b = s.multiplier;
    StepTrace tr;
    const bool cont = path_continues(P, s, path_step(P, lights, s, lh, nh, &tr));
    if (tr.hit && nv < kMaxRecordVertices) {
      const f3 wo = -tr.in;
      const f3 cp = scene != nullptr ? batch_cache_position(*scene, tr.point) : tr.point;
      const float v[12] = {cp.x, cp.y, cp.z, wo.x, wo.y, wo.z,
                           tr.normal.x, tr.normal.y, tr.normal.z, tr.albedo.r,
                           tr.albedo.g, tr.albedo.b};
      for (int j = 0; j < 12; ++j) {
        q[nv][j] = v[j];
      }
      gathered[nv] = s.total;
      beta[nv] = b;
      ++nv;
    }
    if (!cont) {
      break;
    }
  }
  float *r = records + (size_t)i * 16;
  if (nv == 0) {
    // the camera ray left the scene: a zero-radiance record at its origin
    const f3 cp = scene != nullptr ? batch_cache_position(*scene, s.o) : s.o;
    const float v[16] = {cp.x, cp.y, cp.z, 0.f, 0.f, 1.f, 0.f, 0.f, 1.f,
                         0.f,   0.f,   0.f,   0.f, 0.f, 0.f, 0.f};
    for (int j = 0; j < 16; ++j) {
      r[j] = v[j];
    }
    return;
  }
  const uint32_t k = depth < nv ? depth : nv - 1;
  const rgb total = s.total;
  const rgb rest = total - gathered[k];
  const float t[3] = {beta[k].r > 1e-12f ? rest.r / beta[k].r : 0.f,
                      beta[k].g > 1e-12f ? rest.g / beta[k].g : 0.f,
                      beta[k].b > 1e-12f ? rest.b / beta[k].b : 0.f};
  for (int j = 0; j < 12; ++j) {
    r[j] = q[k][j];
  }
  r[12] = fmaxf(t[0], 0.f);
  r[13] = fmaxf(t[1], 0.f);
  r[14] = fmaxf(t[2], 0.f);
  r[15] = 0.f;
}

__global__ void k_nrc_apply(float *sample_rgb, const float *beta, const float *pred, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  for (int c = 0; c < 3; ++c) {
    const float b = beta[3 * i + c];
    if (b != 0.f) {
      sample_rgb[3 * i + c] += b * fmaxf(pred[3 * i + c], 0.f);
    }
  }
}

} // namespace
} // namespace dev

cudaError_t launch_nrc_paths(const RenderParams &p, uint32_t n, uint32_t frame, uint32_t depth,
                             float *records,
                             cudaStream_t s) {
  if (n == 0) {
    return cudaSuccess;
  }
  if (p.rng_uniform) {
    dev::k_nrc_paths<true>
        <<<(n + 127) / 128, 128, 0, s>>>(p, nullptr, 0, n, frame, depth, records);
  } else {
    dev::k_nrc_paths<false>
        <<<(n + 127) / 128, 128, 0, s>>>(p, nullptr, 0, n, frame, depth, records);
  }
  return cudaGetLastError();
}

cudaError_t launch_nrc_paths_batch(const RenderParams &p, const BatchScene *scenes,
                                   uint32_t n_scenes, uint32_t n, uint32_t frame,
                                   uint32_t depth, float *records, cudaStream_t s) {
  if (n == 0 || n_scenes == 0) {
    return cudaSuccess;
  }
  if (p.rng_uniform) {
    dev::k_nrc_paths<true>
        <<<(n + 127) / 128, 128, 0, s>>>(p, scenes, n_scenes, n, frame, depth, records);
  } else {
    dev::k_nrc_paths<false>
        <<<(n + 127) / 128, 128, 0, s>>>(p, scenes, n_scenes, n, frame, depth, records);
  }
  return cudaGetLastError();
}

cudaError_t launch_nrc_apply(float *sample_rgb, const float *beta, const float *pred, size_t n,
                             cudaStream_t s) {
  if (n == 0) {
    return cudaSuccess;
  }
  dev::k_nrc_apply<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(sample_rgb, beta, pred, n);
  return cudaGetLastError();
}

} // namespace pg

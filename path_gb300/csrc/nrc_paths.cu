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

template <bool kUniform>
__global__ void __launch_bounds__(128) k_nrc_paths(const RenderParams P, uint32_t n,
                                                   uint32_t frame, uint32_t depth,
                                                   float *records) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  const uint32_t h0 = mix32(i * 0x9e3779b9u ^ mix32(frame + 0x632be5abu));
  const uint32_t n_pix = P.x_dim * P.y_dim;
  const uint32_t pixel = h0 % n_pix;
  const uint32_t x = pixel % P.x_dim, y = pixel / P.x_dim;
  const uint32_t smp = mix32(h0) % P.spp;
  PathStateT<kUniform> s;
  uint32_t xw[kUniform ? kXorwowWords : 1];
  path_begin(P, smp, x, y, s, xw, 1);
  float q[kMaxRecordVertices][12];
  rgb gathered[kMaxRecordVertices], beta[kMaxRecordVertices];
  uint32_t nv = 0;
  Counts cnt = {0, 0, 0};
  const LightSet lights = lights_of(P);
  while (true) {
    Hit lh, nh;
    step_hits<kTravWide, false>(P, s, false, x, cnt, lh, nh);
    const rgb b = s.multiplier;
    StepTrace tr;
    const bool cont = path_continues(P, s, path_step(P, lights, s, lh, nh, &tr));
    if (tr.hit && nv < kMaxRecordVertices) {
      const f3 wo = -tr.in;
      const float v[12] = {tr.point.x, tr.point.y, tr.point.z, wo.x, wo.y, wo.z,
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
    const float v[16] = {s.o.x, s.o.y, s.o.z, 0.f, 0.f, 1.f, 0.f, 0.f, 1.f,
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
    dev::k_nrc_paths<true><<<(n + 127) / 128, 128, 0, s>>>(p, n, frame, depth, records);
  } else {
    dev::k_nrc_paths<false><<<(n + 127) / 128, 128, 0, s>>>(p, n, frame, depth, records);
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

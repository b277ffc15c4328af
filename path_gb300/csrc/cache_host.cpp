// Radiance cache on the host side: parameters, Adam state and the calls
// that train and query the network (kernels in cache.cu).
#include "cache_host.h"

#include <cmath>
#include <cstring>
#include <random>

namespace pg {

#define PG_TRY_CUDA(expr, what)                                                \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      return cuda_status(e_, what);                                            \
    }                                                                          \
  } while (0)

// grids: one training CTA per SM (each holds all 512 tensor-memory
// columns) and one inference CTA per SM (its four teams take 221 KB of
// shared memory)

Status RadianceCache::init(uint32_t seed, float lr) {
  if (ready_) {
    return Status::ok();
  }
  PG_TRY_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream");
  int dev = 0;
  PG_TRY_CUDA(cudaGetDevice(&dev), "device");
  PG_TRY_CUDA(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev), "sm count");
  lr_ = lr;
  const size_t nt = (size_t)kNrcLevels * kNrcTable * 2;
  // Xavier-uniform weights (rows 3.. of the output layer stay zero), small
  // uniform hash-table features
  std::mt19937 gen(seed);
  std::vector<float> w(kNrcWeights, 0.f), t(nt);
  for (uint32_t l = 0; l < kNrcLayers; ++l) {
    const uint32_t in_l = nrc_in_dim(l), out_l = nrc_out_dim(l);
    const uint32_t rows = l + 1 == kNrcLayers ? 3u : out_l;
    const uint32_t fan_in = l == 0 ? 41u : in_l;
    const float a = std::sqrt(6.f / (float)(fan_in + rows));
    std::uniform_real_distribution<float> u(-a, a);
    for (uint32_t o = 0; o < rows; ++o) {
      for (uint32_t i = 0; i < in_l; ++i) {
        w[nrc_weight_offset(l) + o * in_l + i] = (l == 0 && i >= 41) ? 0.f : u(gen);
      }
    }
  }
  std::uniform_real_distribution<float> ut(-1e-4f, 1e-4f);
  for (float &x : t) {
    x = ut(gen);
  }
  PG_TRY_CUDA(w_.upload(w.data(), w.size() * 4, stream_), "cache weights");
  PG_TRY_CUDA(table_.upload(t.data(), t.size() * 4, stream_), "cache table");
  for (DeviceBuffer *b : {&gw_, &mw_, &vw_}) {
    PG_TRY_CUDA(b->ensure(kNrcWeights * 4), "cache state");
    PG_TRY_CUDA(cudaMemsetAsync(b->get(), 0, kNrcWeights * 4, stream_), "cache state");
  }
  for (DeviceBuffer *b : {&gt_, &mt_, &vt_}) {
    PG_TRY_CUDA(b->ensure(nt * 4), "cache state");
    PG_TRY_CUDA(cudaMemsetAsync(b->get(), 0, nt * 4, stream_), "cache state");
  }
  PG_TRY_CUDA(wfwd_.ensure(kNrcWeightBytes), "cache images");
  PG_TRY_CUDA(wbwd_.ensure(kNrcWeightBytes), "cache images");
  PG_TRY_CUDA(scratch_.ensure(nrc_train_scratch_bytes(sms_)), "cache scratch");
  PG_TRY_CUDA(err_.ensure(4), "cache flags");
  PG_TRY_CUDA(loss_.ensure(4), "cache flags");
  PG_TRY_CUDA(launch_nrc_pack_weights(w_.as<float>(), wfwd_.as<unsigned char>(),
                                      wbwd_.as<unsigned char>(), stream_),
              "cache pack");
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "cache init");
  // level resolutions: geometric from 16 to 2048
  const float b = std::exp((std::log(2048.f) - std::log(16.f)) / (float)(kNrcLevels - 1));
  for (uint32_t l = 0; l < kNrcLevels; ++l) {
    level_res_[l] = std::floor(16.f * std::pow(b, (float)l));
  }
  for (int a = 0; a < 3; ++a) {
    lo_[a] = -1.f;
    inv_ext_[a] = 0.5f;
  }
  ready_ = true;
  return Status::ok();
}

RadianceCache::~RadianceCache() {
  if (stream_ != nullptr) {
    cudaStreamSynchronize(stream_);
    cudaStreamDestroy(stream_);
  }
}

void RadianceCache::set_bounds(const float *lo, const float *hi) {
  batch_ = false;
  for (int a = 0; a < 3; ++a) {
    const float ext = std::max(hi[a] - lo[a], 1e-6f);
    lo_[a] = lo[a];
    inv_ext_[a] = 1.f / ext;
  }
}

NrcParams RadianceCache::params() const {
  NrcParams c;
  std::memset(&c, 0, sizeof(c));
  c.table = table_.as<const float2>();
  for (int a = 0; a < 3; ++a) {
    c.lo[a] = lo_[a];
    c.inv_extent[a] = inv_ext_[a];
  }
  c.batch = batch_ ? 1u : 0u;
  std::memcpy(c.level_res, level_res_, sizeof(level_res_));
  c.w_fwd = wfwd_.as<const unsigned char>();
  c.w_bwd = wbwd_.as<const unsigned char>();
  return c;
}

Status RadianceCache::check_err(const char *what) {
  uint32_t err = 0;
  PG_TRY_CUDA(cudaMemcpyAsync(&err, err_.get(), 4, cudaMemcpyDeviceToHost, stream_), what);
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), what);
  if (err != 0) {
    return Status::err(PATH_ERR_DEVICE_TIMEOUT, std::string(what) +
                                                    ": tensor-core MMA did not complete");
  }
  return Status::ok();
}

Status RadianceCache::infer(const float *queries, uint32_t n, float *out, cudaStream_t s,
                            const float *live) {
  PG_TRY_CUDA(cudaMemsetAsync(err_.get(), 0, 4, s), "cache query");
  PG_TRY_CUDA(encoded_.ensure(std::max<size_t>(nrc_encoded_bytes(n), 16)), "cache query");
  PG_TRY_CUDA(launch_nrc_infer(infer_params(), queries, n, live, out, encoded_.as<unsigned char>(),
                               err_.as<uint32_t>(), sms_, s),
              "cache query");
  return Status::ok();
}

Status RadianceCache::gradients(const float *records, uint32_t n, float *loss) {
  PG_TRY_CUDA(dfeat_.ensure((size_t)std::max<uint32_t>(n, 1) * 32 * 4), "cache grads");
  PG_TRY_CUDA(cudaMemsetAsync(gw_.get(), 0, kNrcWeights * 4, stream_), "cache grads");
  PG_TRY_CUDA(cudaMemsetAsync(gt_.get(), 0, (size_t)kNrcLevels * kNrcTable * 8, stream_),
              "cache grads");
  PG_TRY_CUDA(cudaMemsetAsync(err_.get(), 0, 4, stream_), "cache train");
  PG_TRY_CUDA(cudaMemsetAsync(loss_.get(), 0, 4, stream_), "cache train");
  const NrcParams c = params();
  PG_TRY_CUDA(launch_nrc_train(c, records, n, 1.f / (float)std::max<uint32_t>(n, 1),
                               gw_.as<float>(), dfeat_.as<float>(),
                               scratch_.as<unsigned char>(), loss_.as<float>(),
                               err_.as<uint32_t>(), sms_, stream_),
              "cache train");
  PG_TRY_CUDA(launch_nrc_grid_backward(c, records, n, dfeat_.as<float>(), gt_.as<float2>(),
                                       stream_),
              "cache grid backward");
  if (loss != nullptr) {
    PG_TRY_CUDA(cudaMemcpyAsync(loss, loss_.get(), 4, cudaMemcpyDeviceToHost, stream_),
                "cache loss");
  }
  return check_err("cache train");
}

Status RadianceCache::train(const float *records, uint32_t n, float *loss) {
  Status sg = gradients(records, n, loss);
  if (!sg.good()) {
    return sg;
  }
  ++step_;
  const float st = (float)step_;
  PG_TRY_CUDA(launch_adam(w_.as<float>(), gw_.as<float>(), mw_.as<float>(), vw_.as<float>(),
                          kNrcWeights, lr_, 0.9f, 0.99f, 1e-15f, st, stream_),
              "cache adam");
  PG_TRY_CUDA(launch_adam(table_.as<float>(), gt_.as<float>(), mt_.as<float>(),
                          vt_.as<float>(), (size_t)kNrcLevels * kNrcTable * 2, lr_, 0.9f,
                          0.99f, 1e-15f, st, stream_),
              "cache adam");
  PG_TRY_CUDA(launch_nrc_pack_weights(w_.as<float>(), wfwd_.as<unsigned char>(),
                                      wbwd_.as<unsigned char>(), stream_),
              "cache pack");
  if (ema_decay_ > 0.f) {
    PG_TRY_CUDA(launch_ema(ema_w_.as<float>(), w_.as<float>(), kNrcWeights, ema_decay_, stream_),
                "cache average");
    PG_TRY_CUDA(launch_ema(ema_t_.as<float>(), table_.as<float>(),
                           (size_t)kNrcLevels * kNrcTable * 2, ema_decay_, stream_),
                "cache average");
    PG_TRY_CUDA(launch_nrc_pack_weights(ema_w_.as<float>(), ema_fwd_.as<unsigned char>(),
                                        ema_bwd_.as<unsigned char>(), stream_),
                "cache average");
  }
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "cache train");
  return Status::ok();
}

Status RadianceCache::reset_ema() {
  const size_t nt = (size_t)kNrcLevels * kNrcTable * 2 * 4;
  PG_TRY_CUDA(ema_w_.ensure(kNrcWeights * 4), "cache average");
  PG_TRY_CUDA(ema_t_.ensure(nt), "cache average");
  PG_TRY_CUDA(ema_fwd_.ensure(kNrcWeightBytes), "cache average");
  PG_TRY_CUDA(ema_bwd_.ensure(kNrcWeightBytes), "cache average");
  PG_TRY_CUDA(cudaMemcpyAsync(ema_w_.get(), w_.get(), kNrcWeights * 4, cudaMemcpyDeviceToDevice,
                              stream_),
              "cache average");
  PG_TRY_CUDA(cudaMemcpyAsync(ema_t_.get(), table_.get(), nt, cudaMemcpyDeviceToDevice, stream_),
              "cache average");
  PG_TRY_CUDA(launch_nrc_pack_weights(ema_w_.as<float>(), ema_fwd_.as<unsigned char>(),
                                      ema_bwd_.as<unsigned char>(), stream_),
              "cache average");
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "cache average");
  return Status::ok();
}

Status RadianceCache::set_ema(float decay) {
  if (!(decay >= 0.f && decay < 1.f)) {
    return Status::err(PATH_ERR_ARGUMENT, "the average's decay must be in [0, 1)");
  }
  ema_decay_ = decay;
  return decay > 0.f ? reset_ema() : Status::ok();
}

NrcParams RadianceCache::infer_params() const {
  NrcParams c = params();
  if (ema_decay_ > 0.f) {
    c.table = ema_t_.as<const float2>();
    c.w_fwd = ema_fwd_.as<const unsigned char>();
    c.w_bwd = ema_bwd_.as<const unsigned char>();
  }
  return c;
}

Status RadianceCache::access(float *weights, float *table, float *grad_w, float *grad_t,
                             bool set) {
  const size_t nt = (size_t)kNrcLevels * kNrcTable * 2 * 4;
  struct Item {
    float *host;
    DeviceBuffer *dev;
    size_t bytes;
  } items[] = {{weights, &w_, kNrcWeights * 4}, {table, &table_, nt},
               {grad_w, &gw_, kNrcWeights * 4}, {grad_t, &gt_, nt}};
  for (const Item &it : items) {
    if (it.host == nullptr) {
      continue;
    }
    PG_TRY_CUDA(cudaMemcpyAsync(set ? it.dev->get() : static_cast<void *>(it.host),
                                set ? static_cast<const void *>(it.host) : it.dev->get(),
                                it.bytes, set ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                                stream_),
                "cache parameters");
  }
  if (set) {
    PG_TRY_CUDA(launch_nrc_pack_weights(w_.as<float>(), wfwd_.as<unsigned char>(),
                                        wbwd_.as<unsigned char>(), stream_),
                "cache pack");
  }
  PG_TRY_CUDA(cudaStreamSynchronize(stream_), "cache parameters");
  if (set && ema_decay_ > 0.f) {
    // new parameters: the average starts again from them
    return reset_ema();
  }
  return Status::ok();
}

} // namespace pg

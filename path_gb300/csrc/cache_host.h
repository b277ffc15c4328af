// Host side of the neural radiance cache (see nrc.h for the network).
#pragma once

#include "nrc.h"
#include "renderer.h"

namespace pg {

class RadianceCache {
public:
  RadianceCache() = default;
  RadianceCache(const RadianceCache &) = delete;
  RadianceCache &operator=(const RadianceCache &) = delete;
  ~RadianceCache();

  Status init(uint32_t seed, float learning_rate);
  // scene box mapped to the unit cube of the hash grid
  void set_bounds(const float *lo, const float *hi);
  // inference on an exponential moving average of the parameters, updated
  // after every Adam step (decay in (0, 1); 0 turns it off and inference
  // uses the parameters themselves); the average starts from the current
  // parameters
  Status set_ema(float decay);
  // positions in batch-cell coordinates (a batch's cache, one cell per
  // scene: BatchScene::cache_cell); set_bounds returns to one scene box
  void set_batch_cells() { batch_ = true; }
  bool batch_cells() const { return batch_; }
  NrcParams params() const;
  // what inference reads: params(), or the moving average's table and
  // weight images
  NrcParams infer_params() const;
  // out [n][3] = network(queries [n][12]) on stream s (device pointers);
  // with live ([n][3]), queries whose three live values are zero are skipped
  Status infer(const float *queries, uint32_t n, float *out, cudaStream_t s,
               const float *live = nullptr);
  // gradients of the mean relative L2 loss over records [n][16] (query,
  // target rgb, pad) into the gradient buffers, without an update
  Status gradients(const float *records, uint32_t n, float *loss);
  // one Adam step on records (device pointer)
  Status train(const float *records, uint32_t n, float *loss);
  // host copies of (or into, with set) weights [kNrcWeights], table
  // [levels][entries][2], and the gradient buffers; NULL skips one
  Status access(float *weights, float *table, float *grad_w, float *grad_t, bool set);
  cudaStream_t stream() const { return stream_; }
  uint64_t steps() const { return step_; }

private:
  Status check_err(const char *what);
  bool ready_ = false;
  cudaStream_t stream_ = nullptr;
  float lr_ = 1e-2f;
  uint64_t step_ = 0;
  float level_res_[kNrcLevels] = {};
  float lo_[3] = {}, inv_ext_[3] = {};
  bool batch_ = false;
  int sms_ = 0;
  float ema_decay_ = 0.f;
  Status reset_ema();
  DeviceBuffer ema_w_, ema_t_, ema_fwd_, ema_bwd_;
  DeviceBuffer table_, w_, gw_, mw_, vw_, gt_, mt_, vt_, wfwd_, wbwd_, dfeat_, scratch_, err_,
      loss_, encoded_;
};

} // namespace pg

// kernel::WorkDivision restated for host and device
// (src/kernel/work_division.cpp:12-69, include/kernel/work_division_impl.h).
//
// A pixel's samples are split over n_threads_per_location threads (a power
// of two near spp / target samples per thread); sample_block_size of them
// sit in one CTA and are summed by a shuffle tree, the remaining
// num_sample_blocks factor is summed by a second reduction pass.
#pragma once

#include "pmath.h"
#include "path_gb300.h"

#include <stdint.h>

namespace pg {

struct WorkDiv {
  uint32_t block_size, base_samples_per_thread, n_threads_per_unit_extra,
      sample_block_size, x_block_size, y_block_size, num_sample_blocks,
      num_x_blocks, num_y_blocks, x_dim, y_dim;

  PM_HDM uint32_t total_blocks() const {
    return num_sample_blocks * num_x_blocks * num_y_blocks;
  }
};

struct ThreadWork {
  uint32_t start, end, x, y;
  bool exit;
};

// WorkDivision::get_thread_info (work_division_impl.h:10-55)
PM_HD ThreadWork thread_work(const WorkDiv &w, uint32_t block_idx,
                             uint32_t thread_idx) {
  uint32_t b_sample = block_idx % w.num_sample_blocks;
  uint32_t b_loc = block_idx / w.num_sample_blocks;
  uint32_t b_x = b_loc % w.num_x_blocks;
  uint32_t b_y = b_loc / w.num_x_blocks;
  uint32_t t_sample = thread_idx % w.sample_block_size;
  uint32_t t_loc = thread_idx / w.sample_block_size;
  uint32_t t_x = t_loc % w.x_block_size;
  uint32_t t_y = t_loc / w.x_block_size;
  uint32_t sample_idx = t_sample + b_sample * w.sample_block_size;
  ThreadWork o;
  o.x = t_x + b_x * w.x_block_size;
  o.y = t_y + b_y * w.y_block_size;
  uint32_t extra = sample_idx < w.n_threads_per_unit_extra ? sample_idx
                                                            : w.n_threads_per_unit_extra;
  o.start = sample_idx * w.base_samples_per_thread + extra;
  o.end = o.start + w.base_samples_per_thread +
          (sample_idx < w.n_threads_per_unit_extra ? 1u : 0u);
  o.exit = o.x >= w.x_dim || o.y >= w.y_dim;
  return o;
}

// constructor (host only; returns false on invalid settings)
bool make_workdiv(const path_work_division_settings &s, uint32_t samples_per,
                  uint32_t x_dim, uint32_t y_dim, WorkDiv &out);

} // namespace pg

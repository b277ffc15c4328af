// Radiance-cache network shapes and the parameters its kernels read.
//
// Input (48 BF16 per query): 16 hash-grid levels x 2 features of the
// position, then direction, normal and albedo (9 floats), then zeros.
// Six fully connected layers without biases: 48 -> 64, four 64 -> 64
// (ReLU after each of these five), 64 -> 16 of which the first 3 outputs
// are the RGB radiance.  Weights of layer l are [out_l][in_l].
#pragma once

#include <stdint.h>

#include <cuda_runtime.h>

namespace pg {

constexpr uint32_t kNrcLevels = 16;
constexpr uint32_t kNrcLog2Table = 19;
constexpr uint32_t kNrcTable = 1u << kNrcLog2Table; // entries per level
constexpr uint32_t kNrcIn = 48;
constexpr uint32_t kNrcHid = 64;
constexpr uint32_t kNrcOut = 16;
constexpr uint32_t kNrcLayers = 6;
constexpr uint32_t kNrcWeights = 64 * 48 + 4 * 64 * 64 + 16 * 64; // 20480
constexpr uint32_t kNrcWeightBytes = kNrcWeights * 2;             // one BF16 image
// tensor-memory columns: [0, 64) layer output / input gradient, then the
// weight-gradient accumulators of the six layers (in_l columns each)
constexpr uint32_t kNrcTmemDw = 64;

__host__ __device__ constexpr uint32_t nrc_in_dim(uint32_t l) { return l == 0 ? kNrcIn : kNrcHid; }
__host__ __device__ constexpr uint32_t nrc_out_dim(uint32_t l) {
  return l + 1 == kNrcLayers ? kNrcOut : kNrcHid;
}
// first element of layer l in the flat weight array (and byte offset / 2 in
// the BF16 images)
__host__ __device__ constexpr uint32_t nrc_weight_offset(uint32_t l) {
  return l == 0 ? 0u : 64u * 48u + (l - 1) * 64u * 64u;
}
// first tensor-memory column of layer l's weight gradient
__host__ __device__ constexpr uint32_t nrc_dw_column(uint32_t l) {
  return kNrcTmemDw + (l == 0 ? 0u : 48u + (l - 1) * 64u);
}

// Index of grid vertex (x, y, z) of a level with `side` vertices per axis:
// dense when the level fits the table, else the spatial hash of Teschner et
// al. (2003) as used by Mueller et al. (2022), modulo the table size.
__host__ __device__ inline uint32_t nrc_grid_index(uint32_t x, uint32_t y, uint32_t z,
                                                   uint32_t side) {
  if ((uint64_t)side * side * side <= kNrcTable) {
    return x + side * (y + side * z);
  }
  return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & (kNrcTable - 1);
}

// A batch's cache: positions arrive as x in [0, 1]^3 plus twice an integer
// cell (one cell per scene of the batch); the cell offsets the grid vertex
// coordinates so that every scene has vertices of its own, all hashed.
__host__ __device__ inline uint32_t nrc_batch_grid_index(uint32_t x, uint32_t y, uint32_t z,
                                                         uint32_t side, const uint32_t *cell) {
  return ((x + side * cell[0]) ^ ((y + side * cell[1]) * 2654435761u) ^
          ((z + side * cell[2]) * 805459861u)) &
         (kNrcTable - 1);
}

struct NrcParams {
  const float2 *table;        // [levels][kNrcTable] feature pairs
  float lo[3], inv_extent[3]; // scene box: position -> [0, 1]^3
  uint32_t batch;             // positions in batch-cell coordinates (lo, inv_extent unused)
  float level_res[kNrcLevels];
  const unsigned char *w_fwd; // BF16 [out][in] K-major tiles (tc.cuh layout)
  const unsigned char *w_bwd; // BF16 [in][out] K-major tiles
};

// live: optional [n][3], a query whose three values are zero is skipped;
// encoded: nrc_encoded_bytes(n) of scratch for the encoded input tiles
cudaError_t launch_nrc_infer(const NrcParams &c, const float *queries, uint32_t n,
                             const float *live, float *out, unsigned char *encoded,
                             uint32_t *err, int grid, cudaStream_t s);
size_t nrc_encoded_bytes(uint32_t n);
cudaError_t launch_nrc_train(const NrcParams &c, const float *records, uint32_t n,
                             float inv_batch, float *grad_w, float *d_feat,
                             unsigned char *scratch, float *loss, uint32_t *err, int grid,
                             cudaStream_t s);
cudaError_t launch_nrc_grid_backward(const NrcParams &c, const float *records, uint32_t n,
                                     const float *d_feat, float2 *grad_table, cudaStream_t s);
cudaError_t launch_nrc_pack_weights(const float *w, unsigned char *w_fwd, unsigned char *w_bwd,
                                    cudaStream_t s);
// avg = decay avg + (1 - decay) param over n floats
cudaError_t launch_ema(float *avg, const float *param, size_t n, float decay, cudaStream_t s);
cudaError_t launch_adam(float *param, float *grad, float *m, float *v, size_t n, float lr,
                        float beta1, float beta2, float eps, float step, cudaStream_t s);
size_t nrc_train_scratch_bytes(int grid);
size_t nrc_infer_smem_bytes();
size_t nrc_train_smem_bytes();

} // namespace pg

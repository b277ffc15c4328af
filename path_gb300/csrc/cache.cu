// Neural radiance cache: hash-grid encoding and a BF16 MLP on the fifth-
// generation tensor cores (tcgen05, accumulators in tensor memory).
//
// This file holds the tensor-core building block (one 128-row tile of
// D = A . B^T, the operands staged in shared memory in the canonical
// K-major layout of tc.cuh) and its self-test entry point.
#include "kernels.h"
#include "nrc.h"
#include "tc.cuh"

#include <cuda_bf16.h>

namespace pg {
namespace dev {

constexpr uint32_t kTcWaitLimit = 1u << 24; // polls before a wait gives up

// D [128][n] = A [128][k] . B [n][k]^T, BF16 in, FP32 out, one CTA of 128
// threads.  err: set to 1 when the tensor core did not signal completion
// within wait_limit polls of the mbarrier.  With issue 0 no MMA is issued
// and nothing arrives on the mbarrier: the wait runs out, which is how the
// tests exercise the bounded waits without faulting anything.
__global__ void __launch_bounds__(128) k_tc_gemm(const __nv_bfloat16 *a,
                                                 const __nv_bfloat16 *b, float *d,
                                                 uint32_t k_dim, uint32_t n_dim,
                                                 uint32_t *err, uint32_t wait_limit,
                                                 uint32_t issue) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const uint32_t tid = threadIdx.x;
  unsigned char *sa = smem;
  unsigned char *sb = smem + 128 * k_dim * 2;
  // stage A and B in the canonical layout
  for (uint32_t i = tid; i < 128 * k_dim; i += 128) {
    const uint32_t r = i / k_dim, c = i % k_dim;
    *reinterpret_cast<__nv_bfloat16 *>(sa + tc::smem_offset(r, c, k_dim)) = a[i];
  }
  for (uint32_t i = tid; i < n_dim * k_dim; i += 128) {
    const uint32_t r = i / k_dim, c = i % k_dim;
    *reinterpret_cast<__nv_bfloat16 *>(sb + tc::smem_offset(r, c, k_dim)) = b[i];
  }
  uint32_t ncols = 32;
  while (ncols < n_dim) {
    ncols <<= 1;
  }
  if (tid < 32) {
    tc::tmem_alloc(tc::smem_addr(&tmem_base), ncols);
  }
  if (tid == 0) {
    tc::mbar_init(tc::smem_addr(&mbar), 1);
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  if (tid == 0 && issue != 0) {
    const uint32_t idesc = tc::idesc_bf16(128, n_dim);
    for (uint32_t k0 = 0; k0 < k_dim; k0 += 16) {
      const uint64_t ad = tc::smem_desc(tc::smem_addr(sa) + k0 * 16, k_dim);
      const uint64_t bd = tc::smem_desc(tc::smem_addr(sb) + k0 * 16, k_dim);
      tc::mma_bf16(tmem, ad, bd, idesc, k0 > 0 ? 1u : 0u);
    }
    tc::commit(tc::smem_addr(&mbar));
  }
  const bool ok = __syncthreads_and(tc::mbar_wait(tc::smem_addr(&mbar), 0, wait_limit)) != 0;
  tc::fence_after_sync();
  if (!ok) {
    if (tid == 0) {
      atomicExch(err, 1u);
    }
  } else {
    const uint32_t warp = tid / 32;
    const uint32_t row = tid;
    for (uint32_t c0 = 0; c0 < n_dim; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((warp * 32) << 16) + c0, v);
      for (int j = 0; j < 16; ++j) {
        d[(size_t)row * n_dim + c0 + j] = v[j];
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) {
    tc::tmem_dealloc(tmem, ncols);
  }
}

} // namespace dev

cudaError_t launch_tc_gemm(const void *a, const void *b, float *d, uint32_t k_dim,
                           uint32_t n_dim, uint32_t *err, cudaStream_t s, uint32_t wait_limit,
                           bool issue) {
  const size_t smem = (size_t)(128 + n_dim) * k_dim * 2;
  cudaError_t e = cudaFuncSetAttribute(dev::k_tc_gemm,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    return e;
  }
  dev::k_tc_gemm<<<1, 128, smem, s>>>(static_cast<const __nv_bfloat16 *>(a),
                                      static_cast<const __nv_bfloat16 *>(b), d, k_dim, n_dim,
                                      err, wait_limit == 0 ? dev::kTcWaitLimit : wait_limit,
                                      issue ? 1u : 0u);
  return cudaGetLastError();
}

} // namespace pg

// ---------------------------------------------------------------------------
// Radiance cache MLP and hash-grid encoding

namespace pg {
namespace dev {

using tc::smem_offset;

// a query position in [0, 1]^3 of the hash grid and, for a batch's cache,
// its cell (zero otherwise)
__device__ __forceinline__ void nrc_position(const NrcParams &C, const float *q, float *p,
                                             uint32_t *cell) {
  for (int a = 0; a < 3; ++a) {
    if (C.batch) {
      const float c = fminf(fmaxf(floorf(q[a] * 0.5f), 0.f), (float)(kCacheCellsPerAxis - 1));
      cell[a] = (uint32_t)c;
      p[a] = q[a] - 2.f * c;
    } else {
      cell[a] = 0;
      p[a] = (q[a] - C.lo[a]) * C.inv_extent[a];
    }
    p[a] = fminf(fmaxf(p[a], 0.f), 1.f);
  }
}

// hash features of levels [l0, l1) of a query's position (trilinear
// interpolation of the 8 grid vertices per level) into in[2 (l - l0)] and
// in[2 (l - l0) + 1]
// levels [l0, l0 + kN), unrolled so that all 8 kN corner loads can be in
// flight together (the encoding waits on these table reads)
template <uint32_t kN>
__device__ __forceinline__ void nrc_encode_levels(const NrcParams &C, const float *q, uint32_t l0,
                                                  float *in) {
  float p[3];
  uint32_t cell[3];
  nrc_position(C, q, p, cell);
#pragma unroll
  for (uint32_t j = 0; j < kN; ++j) {
    const uint32_t l = l0 + j;
    const float res = C.level_res[l];
    const uint32_t side = (uint32_t)res + 1;
    float x[3], fr[3];
    uint32_t c0[3];
    for (int a = 0; a < 3; ++a) {
      x[a] = p[a] * res;
      const float fl = fminf(floorf(x[a]), res - 1.f); // cell in [0, res - 1]
      c0[a] = (uint32_t)fl;
      fr[a] = x[a] - fl;
    }
    float f0 = 0.f, f1 = 0.f;
#pragma unroll
    for (uint32_t c = 0; c < 8; ++c) {
      const uint32_t gx = c0[0] + (c & 1u), gy = c0[1] + ((c >> 1) & 1u),
                     gz = c0[2] + ((c >> 2) & 1u);
      const float w = ((c & 1u) ? fr[0] : 1.f - fr[0]) * (((c >> 1) & 1u) ? fr[1] : 1.f - fr[1]) *
                      (((c >> 2) & 1u) ? fr[2] : 1.f - fr[2]);
      const uint32_t idx =
          C.batch ? nrc_batch_grid_index(gx, gy, gz, side, cell) : nrc_grid_index(gx, gy, gz, side);
      const float2 e = __ldg(C.table + (size_t)l * kNrcTable + idx);
      f0 += w * e.x;
      f1 += w * e.y;
    }
    in[2 * j] = f0;
    in[2 * j + 1] = f1;
  }
}

// one query row of the MLP (q: position, direction, normal, albedo): hash
// features of the position, then direction, normal, albedo (9 floats), zero
// padding to kNrcIn
__device__ void nrc_encode(const NrcParams &C, const float *q, float *in) {
#pragma unroll
  for (uint32_t g = 0; g < kNrcLevels; g += 4) {
    nrc_encode_levels<4>(C, q, g, in + 2 * g);
  }
  for (int k = 0; k < 9; ++k) {
    in[32 + k] = q[3 + k];
  }
  for (uint32_t k = 41; k < kNrcIn; ++k) {
    in[k] = 0.f;
  }
}

__device__ __forceinline__ void store_bf16(unsigned char *tile, uint32_t row, uint32_t k,
                                           uint32_t k_dim, float v) {
  *reinterpret_cast<__nv_bfloat16 *>(tile + smem_offset(row, k, k_dim)) = __float2bfloat16(v);
}

__device__ __forceinline__ float load_bf16(const unsigned char *tile, uint32_t row, uint32_t k,
                                           uint32_t k_dim) {
  return __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(tile + smem_offset(row, k, k_dim)));
}

// copy n bytes global -> shared with 16-byte loads (n a multiple of 16)
__device__ __forceinline__ void copy16(unsigned char *dst, const unsigned char *src, uint32_t n,
                                       uint32_t tid, uint32_t nthreads) {
  for (uint32_t i = tid * 16; i < n; i += nthreads * 16) {
    *reinterpret_cast<uint4 *>(dst + i) = __ldg(reinterpret_cast<const uint4 *>(src + i));
  }
}

struct TcSync {
  uint32_t mbar;
  uint32_t phase;
  bool ok;
};

// all threads: make shared-memory writes visible to the tensor core and
// order earlier tensor-memory reads before the next MMA
__device__ __forceinline__ void tc_barrier() {
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
}

// thread 0 issues D (+)= A . B^T over k_dim, then everyone waits for it
__device__ __forceinline__ void tc_layer(TcSync &s, uint32_t tid, uint32_t tmem_d,
                                         const unsigned char *a, const unsigned char *b,
                                         uint32_t k_dim, uint32_t n_dim, uint32_t accumulate) {
  if (tid == 0 && s.ok) {
    const uint32_t idesc = tc::idesc_bf16(128, n_dim);
    for (uint32_t k0 = 0; k0 < k_dim; k0 += 16) {
      tc::mma_bf16(tmem_d, tc::smem_desc(tc::smem_addr(a) + k0 * 16, k_dim),
                   tc::smem_desc(tc::smem_addr(b) + k0 * 16, k_dim), idesc,
                   (k0 > 0 || accumulate) ? 1u : 0u);
    }
  }
}

// thread 0 commits the issued MMAs; every thread waits (bounded) and the
// CTA agrees on the outcome, so a wait that gave up stops all threads alike
__device__ __forceinline__ void tc_wait(TcSync &s, uint32_t tid, uint32_t *err) {
  if (tid == 0 && s.ok) {
    tc::commit(s.mbar);
  }
  bool ok = s.ok;
  if (ok) {
    ok = tc::mbar_wait(s.mbar, s.phase, kTcWaitLimit);
  }
  s.phase ^= 1u;
  s.ok = __syncthreads_and(ok ? 1 : 0) != 0;
  if (!s.ok && tid == 0 && err != nullptr) {
    atomicExch(err, 1u);
  }
  tc::fence_after_sync();
}

// The network's first-layer input of every query as BF16 tiles of 128 rows
// in the tensor core's K-major layout (kNrcTileBytes per tile, rows past n
// zero), written by k_nrc_encode and copied whole into shared memory by
// k_nrc_infer.  Four threads per row: thread g encodes hash levels 4 g ...
// 4 g + 3 (one 16-byte core-matrix row of eight features); threads 0 and 1
// also write the direction, normal and albedo columns and the zero padding.
constexpr uint32_t kNrcTileBytes = 128 * kNrcIn * 2;

__device__ __forceinline__ uint4 pack_bf16x8(const float (&v)[8]) {
  uint4 r;
  uint32_t *w = &r.x;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
    w[k] = *reinterpret_cast<const uint32_t *>(&h);
  }
  return r;
}

// live (optional): per query 3 floats, all zero for a query no path uses
// (its encoding is skipped: zeros)
__global__ void __launch_bounds__(256) k_nrc_encode(const __grid_constant__ NrcParams C,
                                                    const float *queries, uint32_t n,
                                                    uint32_t n_rows, const float *live,
                                                    unsigned char *x0) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t qi = t >> 2, g = t & 3u;
  if (qi >= n_rows) {
    return;
  }
  const float *q = queries + (size_t)qi * 12;
  const bool used = qi < n && (live == nullptr || live[3 * (size_t)qi] != 0.f ||
                               live[3 * (size_t)qi + 1] != 0.f ||
                               live[3 * (size_t)qi + 2] != 0.f);
  float in[8];
  if (used) {
    nrc_encode_levels<4>(C, q, 4 * g, in);
  } else {
    for (int k = 0; k < 8; ++k) {
      in[k] = 0.f;
    }
  }
  unsigned char *tile = x0 + (size_t)(qi >> 7) * kNrcTileBytes;
  const uint32_t row = qi & 127u;
  *reinterpret_cast<uint4 *>(tile + smem_offset(row, 8 * g, kNrcIn)) = pack_bf16x8(in);
  if (g < 2) {
    // columns 32 ... 39: direction, normal, albedo r g; 40 ... 47: albedo b, zeros
    float e[8];
    for (int k = 0; k < 8; ++k) {
      const uint32_t c = 8 * g + (uint32_t)k; // 0 ... 15 past the hash features
      e[k] = used && c < 9 ? q[3 + c] : 0.f;
    }
    *reinterpret_cast<uint4 *>(tile + smem_offset(row, 32 + 8 * g, kNrcIn)) = pack_bf16x8(e);
  }
}

// Inference: out[i] = MLP(x0 row i) for i < n.  One CTA per SM of four
// independent teams (warpgroups) that share the weights in shared memory;
// each team takes every fourth tile of the CTA's share, with its own 64
// tensor-memory columns, mbarriers and 44 KB of tile buffers: its tile's
// input is copied in by one bulk copy (the next tile's copy starts as soon
// as the first layer has consumed the buffer), its leader issues the six
// layers' MMAs, and its four warps read the accumulator lanes of their
// rows (warp q of the team: lanes 32 q ... 32 q + 31) for the ReLU / BF16
// epilogue.  The four teams' MMAs, epilogues and copies overlap.
constexpr uint32_t kInferTeams = 4;
constexpr uint32_t kInferThreads = 128 * kInferTeams;
constexpr uint32_t kInferTeamBytes = kNrcTileBytes + 2 * 128 * kNrcHid * 2;

__global__ void __launch_bounds__(kInferThreads, 1) k_nrc_infer(const __grid_constant__ NrcParams C,
                                                                const unsigned char *x0g,
                                                                uint32_t n, float *out,
                                                                uint32_t *err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar_mma[kInferTeams];
  __shared__ __align__(8) uint64_t mbar_x[kInferTeams];
  __shared__ uint32_t tmem_base;
  const uint32_t tid = threadIdx.x;
  const uint32_t team = tid / 128, ttid = tid % 128;
  const uint32_t bar_id = 1 + team; // named barrier of the team (0 is __syncthreads)
  unsigned char *w = smem;          // forward weights, kNrcWeightBytes
  unsigned char *x0 = smem + kNrcWeightBytes + team * kInferTeamBytes; // [128][kNrcIn]
  unsigned char *ha = x0 + kNrcTileBytes;                               // [128][64]
  unsigned char *hb = ha + 128 * kNrcHid * 2;                           // [128][64]
  copy16(w, C.w_fwd, kNrcWeightBytes, tid, kInferThreads);
  if (tid < 32) {
    tc::tmem_alloc(tc::smem_addr(&tmem_base), 64 * kInferTeams);
  }
  if (tid < kInferTeams) {
    tc::mbar_init(tc::smem_addr(&mbar_mma[tid]), 1);
    tc::mbar_init(tc::smem_addr(&mbar_x[tid]), 1);
  }
  tc_barrier();
  const uint32_t tmem = tmem_base + 64 * team;
  const uint32_t mm = tc::smem_addr(&mbar_mma[team]), mx = tc::smem_addr(&mbar_x[team]);
  const uint32_t quarter = ttid / 32;
  const uint32_t erow = ttid; // epilogue row: warp quarter's lanes
  const uint32_t n_tiles = (n + 127) / 128;
  const uint32_t stride = gridDim.x * kInferTeams;
  uint32_t tile = blockIdx.x * kInferTeams + team;
  uint32_t phase_m = 0, phase_x = 0;
  bool copying = false; // the leader's bulk copy into x0 not yet waited for
  bool ok = true;
  if (ttid == 0 && tile < n_tiles) {
    tc::mbar_arrive_expect_tx(mx, kNrcTileBytes);
    tc::bulk_g2s(tc::smem_addr(x0), x0g + (size_t)tile * kNrcTileBytes, kNrcTileBytes, mx);
    copying = true;
  }
  for (; tile < n_tiles && ok; tile += stride) {
    ok = tc::bar_and(bar_id, 128, tc::mbar_wait(mx, phase_x, kTcWaitLimit));
    phase_x ^= 1u;
    copying = false;
    if (!ok) {
      break;
    }
    tc::fence_after_sync();
    const unsigned char *a = x0;
    for (uint32_t l = 0; l < kNrcLayers; ++l) {
      const uint32_t k_dim = nrc_in_dim(l), n_dim = nrc_out_dim(l);
      if (ttid == 0) {
        const uint32_t idesc = tc::idesc_bf16(128, n_dim);
        const unsigned char *b = w + nrc_weight_offset(l) * 2;
        for (uint32_t k0 = 0; k0 < k_dim; k0 += 16) {
          tc::mma_bf16(tmem, tc::smem_desc(tc::smem_addr(a) + k0 * 16, k_dim),
                       tc::smem_desc(tc::smem_addr(b) + k0 * 16, k_dim), idesc,
                       k0 > 0 ? 1u : 0u);
        }
        tc::commit(mm);
      }
      ok = tc::bar_and(bar_id, 128, tc::mbar_wait(mm, phase_m, kTcWaitLimit));
      phase_m ^= 1u;
      if (!ok) {
        break;
      }
      tc::fence_after_sync();
      if (l == 0 && ttid == 0 && tile + stride < n_tiles) {
        // the first layer has read x0: copy the team's next tile in
        tc::mbar_arrive_expect_tx(mx, kNrcTileBytes);
        tc::bulk_g2s(tc::smem_addr(x0), x0g + (size_t)(tile + stride) * kNrcTileBytes,
                     kNrcTileBytes, mx);
        copying = true;
      }
      unsigned char *dst = (l & 1) ? hb : ha;
      const uint32_t lane_base = (quarter * 32) << 16;
      if (l + 1 < kNrcLayers) {
#pragma unroll
        for (uint32_t c0 = 0; c0 < kNrcHid; c0 += 16) {
          float v[16];
          tc::tmem_ld16(tmem + lane_base + c0, v);
          float lo[8], hi[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            lo[j] = fmaxf(v[j], 0.f);
            hi[j] = fmaxf(v[8 + j], 0.f);
          }
          *reinterpret_cast<uint4 *>(dst + smem_offset(erow, c0, kNrcHid)) = pack_bf16x8(lo);
          *reinterpret_cast<uint4 *>(dst + smem_offset(erow, c0 + 8, kNrcHid)) =
              pack_bf16x8(hi);
        }
      } else {
        float v[16];
        tc::tmem_ld16(tmem + lane_base, v);
        const uint32_t oi = tile * 128 + erow;
        if (oi < n) {
          out[(size_t)oi * 3 + 0] = v[0];
          out[(size_t)oi * 3 + 1] = v[1];
          out[(size_t)oi * 3 + 2] = v[2];
        }
      }
      // epilogue writes visible to the tensor core, tensor-memory reads
      // ordered before the next MMA
      tc::fence_async_smem();
      tc::fence_before_sync();
      tc::bar_sync(bar_id, 128);
      tc::fence_after_sync();
      a = dst;
    }
  }
  if (!ok) {
    if (ttid == 0) {
      atomicExch(err, 1u);
    }
    if (copying) {
      // a bulk copy still in flight lands before the CTA may exit
      tc::mbar_wait(mx, phase_x, kTcWaitLimit);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) {
    tc::tmem_dealloc(tmem_base, 64 * kInferTeams);
  }
}

// Training on tiles of 128 records (query: 12 floats, target: 3 floats,
// padding: 1).  Forward as in inference, keeping each layer's input
// transposed ([in][128], K-major) in this CTA's global scratch; relative L2
// loss (pred - target)^2 / (pred^2 + 0.01) with the denominator held
// constant; backward per layer: dW_l += dY_l^T . X_l (tensor memory,
// accumulated over the CTA's tiles, dY^T padded to 128 rows with zeros) and
// dX_l = dY_l . W_l, ReLU-masked into dY_{l-1}.  dLoss/d(hash features) of
// every record goes to d_feat [n][32]; the CTA's dW is added to grad_w at
// the end.  inv_batch scales the loss (1 / records of the step).
__global__ void __launch_bounds__(128) k_nrc_train(const __grid_constant__ NrcParams C, const float *records,
                                                   uint32_t n, float inv_batch, float *grad_w,
                                                   float *d_feat, unsigned char *scratch,
                                                   float *loss_out, uint32_t *err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const uint32_t tid = threadIdx.x;
  unsigned char *wf = smem;                           // [out][in] tiles
  unsigned char *wb = wf + kNrcWeightBytes;           // [in][out] tiles
  unsigned char *x0 = wb + kNrcWeightBytes;           // [128][48]
  unsigned char *pa = x0 + 128 * kNrcIn * 2;          // [128][64]
  unsigned char *pb = pa + 128 * kNrcHid * 2;         // [128][64]
  unsigned char *st = pb + 128 * kNrcHid * 2;         // X_l^T staging [64][128]
  unsigned char *tt = st + kNrcHid * 128 * 2;         // dY^T [128][128], rows >= 64 zero
  // this CTA's scratch: X_l^T of the six layers
  unsigned char *scr = scratch + (size_t)blockIdx.x * (kNrcIn + 5 * kNrcHid) * 128 * 2;
  auto scr_off = [](uint32_t l) -> uint32_t {
    return l == 0 ? 0u : (kNrcIn + (l - 1) * kNrcHid) * 128 * 2;
  };
  copy16(wf, C.w_fwd, kNrcWeightBytes, tid, 128);
  copy16(wb, C.w_bwd, kNrcWeightBytes, tid, 128);
  for (uint32_t i = tid; i < 128 * 128 * 2 / 16; i += 128) {
    reinterpret_cast<uint4 *>(tt)[i] = make_uint4(0, 0, 0, 0);
  }
  if (tid < 32) {
    tc::tmem_alloc(tc::smem_addr(&tmem_base), 512);
  }
  if (tid == 0) {
    tc::mbar_init(tc::smem_addr(&mbar), 1);
  }
  tc_barrier();
  TcSync sync{tc::smem_addr(&mbar), 0, true};
  const uint32_t tmem = tmem_base;
  const uint32_t lane_base = (tid / 32) * 32;
  const uint32_t row = tid;
  uint32_t tiles_done = 0;
  float loss_sum = 0.f;
  for (uint32_t tile = blockIdx.x; tile * 128 < n && sync.ok; tile += gridDim.x) {
    const uint32_t ri = tile * 128 + row;
    const bool valid = ri < n;
    float in[kNrcIn];
    float target[3] = {0.f, 0.f, 0.f};
    if (valid) {
      const float *rec = records + (size_t)ri * 16;
      nrc_encode(C, rec, in);
      target[0] = rec[12];
      target[1] = rec[13];
      target[2] = rec[14];
    } else {
      for (uint32_t k = 0; k < kNrcIn; ++k) {
        in[k] = 0.f;
      }
    }
    for (uint32_t k = 0; k < kNrcIn; ++k) {
      store_bf16(x0, row, k, kNrcIn, in[k]);
      store_bf16(scr + scr_off(0), k, row, 128, in[k]);
    }
    tc_barrier();
    // forward
    const unsigned char *a = x0;
    for (uint32_t l = 0; l < kNrcLayers && sync.ok; ++l) {
      const uint32_t k_dim = nrc_in_dim(l), n_dim = nrc_out_dim(l);
      tc_layer(sync, tid, tmem, a, wf + nrc_weight_offset(l) * 2, k_dim, n_dim, 0);
      tc_wait(sync, tid, err);
      if (!sync.ok) {
        break;
      }
      unsigned char *dst = (l & 1) ? pb : pa;
      for (uint32_t c0 = 0; c0 < n_dim; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tmem + (lane_base << 16) + c0, v);
        if (l + 1 < kNrcLayers) {
          for (int j = 0; j < 16; ++j) {
            const float h = fmaxf(v[j], 0.f);
            store_bf16(dst, row, c0 + j, kNrcHid, h);
            store_bf16(scr + scr_off(l + 1), c0 + j, row, 128, h);
          }
        } else {
          // output layer: dLoss/dpred into dY5 ([128][16]) and dY5^T
          for (int j = 0; j < 16; ++j) {
            float g = 0.f;
            if (j < 3 && valid) {
              const float pr = v[j];
              const float den = pr * pr + 0.01f;
              const float diff = pr - target[j];
              g = 2.f * diff / den * inv_batch;
              loss_sum += diff * diff / den * inv_batch;
            }
            store_bf16(dst, row, j, kNrcOut, g);
            store_bf16(tt, j, row, 128, g);
          }
          for (uint32_t j = kNrcOut; j < kNrcHid; ++j) {
            store_bf16(tt, j, row, 128, 0.f);
          }
        }
      }
      tc_barrier();
      a = dst;
    }
    // backward; `a` holds dY5 in the A layout (K = 16)
    unsigned char *dy = const_cast<unsigned char *>(a);
    for (int l = (int)kNrcLayers - 1; l >= 0 && sync.ok; --l) {
      const uint32_t in_l = nrc_in_dim((uint32_t)l), out_l = nrc_out_dim((uint32_t)l);
      for (uint32_t i = tid * 16; i < in_l * 128 * 2; i += 128 * 16) {
        *reinterpret_cast<uint4 *>(st + i) =
            *reinterpret_cast<const uint4 *>(scr + scr_off((uint32_t)l) + i);
      }
      tc_barrier();
      // dW_l (+)= dY_l^T . X_l ; dX_l = dY_l . W_l
      tc_layer(sync, tid, tmem + nrc_dw_column((uint32_t)l), tt, st, 128, in_l,
               tiles_done > 0 ? 1u : 0u);
      tc_layer(sync, tid, tmem, dy, wb + nrc_weight_offset((uint32_t)l) * 2, out_l, in_l, 0);
      tc_wait(sync, tid, err);
      if (!sync.ok) {
        break;
      }
      unsigned char *next = (dy == pa) ? pb : pa;
      for (uint32_t c0 = 0; c0 < in_l; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tmem + (lane_base << 16) + c0, v);
        for (int j = 0; j < 16; ++j) {
          const uint32_t i = c0 + j;
          if (l > 0) {
            const float x = load_bf16(st, i, row, 128); // X_l = H_l, ReLU output
            const float g = x > 0.f ? v[j] : 0.f;
            store_bf16(next, row, i, kNrcHid, g);
            store_bf16(tt, i, row, 128, g);
          } else if (valid && i < 2 * kNrcLevels) {
            d_feat[(size_t)ri * 32 + i] = v[j];
          }
        }
      }
      tc_barrier();
      dy = next;
    }
    ++tiles_done;
  }
  if (tiles_done > 0 && sync.ok) {
    // this CTA's weight gradients, lane = output row
    for (uint32_t l = 0; l < kNrcLayers; ++l) {
      const uint32_t in_l = nrc_in_dim(l), out_l = nrc_out_dim(l);
      const uint32_t rows = l + 1 == kNrcLayers ? 3u : out_l;
      for (uint32_t c0 = 0; c0 < in_l; c0 += 16) {
        float v[16];
        tc::tmem_ld16(tmem + (lane_base << 16) + nrc_dw_column(l) + c0, v);
        if (row < rows) {
          for (int j = 0; j < 16; ++j) {
            atomicAdd(grad_w + nrc_weight_offset(l) + row * in_l + c0 + j, v[j]);
          }
        }
      }
    }
  }
  if (loss_out != nullptr) {
    atomicAdd(loss_out, loss_sum);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid < 32) {
    tc::tmem_dealloc(tmem, 512);
  }
}

// dLoss/d(hash table): each record's feature gradient spread over the
// eight grid vertices of every level with the trilinear weights
__global__ void k_nrc_grid_backward(const __grid_constant__ NrcParams C, const float *records, uint32_t n,
                                    const float *d_feat, float2 *grad_table) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  const float *q = records + (size_t)i * 16;
  const float *g = d_feat + (size_t)i * 32;
  float p[3];
  uint32_t cell[3];
  nrc_position(C, q, p, cell);
  for (uint32_t l = 0; l < kNrcLevels; ++l) {
    const float res = C.level_res[l];
    const uint32_t side = (uint32_t)res + 1;
    float fr[3];
    uint32_t c0[3];
    for (int a = 0; a < 3; ++a) {
      const float x = p[a] * res;
      const float fl = fminf(floorf(x), res - 1.f);
      c0[a] = (uint32_t)fl;
      fr[a] = x - fl;
    }
    for (uint32_t c = 0; c < 8; ++c) {
      const uint32_t gx = c0[0] + (c & 1u), gy = c0[1] + ((c >> 1) & 1u),
                     gz = c0[2] + ((c >> 2) & 1u);
      const float w = ((c & 1u) ? fr[0] : 1.f - fr[0]) * (((c >> 1) & 1u) ? fr[1] : 1.f - fr[1]) *
                      (((c >> 2) & 1u) ? fr[2] : 1.f - fr[2]);
      float2 *e = grad_table + (size_t)l * kNrcTable +
                  (C.batch ? nrc_batch_grid_index(gx, gy, gz, side, cell)
                           : nrc_grid_index(gx, gy, gz, side));
      atomicAdd(&e->x, w * g[2 * l]);
      atomicAdd(&e->y, w * g[2 * l + 1]);
    }
  }
}

// FP32 master weights -> the two BF16 tile images (forward [out][in],
// backward [in][out]); one thread per weight
__global__ void k_nrc_pack(const float *w, unsigned char *w_fwd, unsigned char *w_bwd) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kNrcWeights) {
    return;
  }
  uint32_t l = 0;
  while (l + 1 < kNrcLayers && e >= nrc_weight_offset(l + 1)) {
    ++l;
  }
  const uint32_t in_l = nrc_in_dim(l), out_l = nrc_out_dim(l);
  const uint32_t local = e - nrc_weight_offset(l);
  const uint32_t o = local / in_l, i = local % in_l;
  const __nv_bfloat16 v = __float2bfloat16(w[e]);
  unsigned char *f = w_fwd + nrc_weight_offset(l) * 2;
  unsigned char *b = w_bwd + nrc_weight_offset(l) * 2;
  *reinterpret_cast<__nv_bfloat16 *>(f + smem_offset(o, i, in_l)) = v;
  *reinterpret_cast<__nv_bfloat16 *>(b + smem_offset(i, o, out_l)) = v;
}

// avg = decay avg + (1 - decay) param: the exponential moving average of the
// parameters that inference may use instead of the parameters themselves
__global__ void k_ema(float *avg, const float *param, size_t n, float decay) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    avg[i] = decay * avg[i] + (1.f - decay) * param[i];
  }
}

// Adam (Kingma and Ba 2015) with bias correction; clears the gradient
__global__ void k_adam(float *param, float *grad, float *m, float *v, size_t n, float lr,
                       float beta1, float beta2, float eps, float step) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) {
    return;
  }
  const float g = grad[i];
  const float mi = beta1 * m[i] + (1.f - beta1) * g;
  const float vi = beta2 * v[i] + (1.f - beta2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(beta1, step));
  const float vh = vi / (1.f - powf(beta2, step));
  param[i] -= lr * mh / (sqrtf(vh) + eps);
  grad[i] = 0.f;
}

} // namespace dev

size_t nrc_infer_smem_bytes() {
  return kNrcWeightBytes + dev::kInferTeams * dev::kInferTeamBytes;
}

size_t nrc_encoded_bytes(uint32_t n) {
  return (size_t)((n + 127) / 128) * dev::kNrcTileBytes;
}

size_t nrc_train_smem_bytes() {
  return 2 * kNrcWeightBytes + 128 * kNrcIn * 2 + 2 * 128 * kNrcHid * 2 + kNrcHid * 128 * 2 +
         128 * 128 * 2;
}

size_t nrc_train_scratch_bytes(int grid) {
  return (size_t)grid * (kNrcIn + 5 * kNrcHid) * 128 * 2;
}

cudaError_t launch_nrc_infer(const NrcParams &c, const float *queries, uint32_t n,
                             const float *live, float *out, unsigned char *encoded,
                             uint32_t *err, int grid, cudaStream_t s) {
  const size_t smem = nrc_infer_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(dev::k_nrc_infer,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess || n == 0) {
    return e;
  }
  const uint32_t n_rows = (n + 127) / 128 * 128;
  dev::k_nrc_encode<<<(n_rows * 4 + 255) / 256, 256, 0, s>>>(c, queries, n, n_rows, live,
                                                             encoded);
  if ((e = cudaGetLastError()) != cudaSuccess) {
    return e;
  }
  dev::k_nrc_infer<<<grid, dev::kInferThreads, smem, s>>>(c, encoded, n, out, err);
  return cudaGetLastError();
}

cudaError_t launch_nrc_train(const NrcParams &c, const float *records, uint32_t n,
                             float inv_batch, float *grad_w, float *d_feat,
                             unsigned char *scratch, float *loss, uint32_t *err, int grid,
                             cudaStream_t s) {
  const size_t smem = nrc_train_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(dev::k_nrc_train,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess || n == 0) {
    return e;
  }
  dev::k_nrc_train<<<grid, 128, smem, s>>>(c, records, n, inv_batch, grad_w, d_feat, scratch,
                                           loss, err);
  return cudaGetLastError();
}

cudaError_t launch_nrc_grid_backward(const NrcParams &c, const float *records, uint32_t n,
                                     const float *d_feat, float2 *grad_table, cudaStream_t s) {
  if (n == 0) {
    return cudaSuccess;
  }
  dev::k_nrc_grid_backward<<<(n + 255) / 256, 256, 0, s>>>(c, records, n, d_feat, grad_table);
  return cudaGetLastError();
}

cudaError_t launch_nrc_pack_weights(const float *w, unsigned char *w_fwd, unsigned char *w_bwd,
                                    cudaStream_t s) {
  dev::k_nrc_pack<<<(kNrcWeights + 255) / 256, 256, 0, s>>>(w, w_fwd, w_bwd);
  return cudaGetLastError();
}

cudaError_t launch_ema(float *avg, const float *param, size_t n, float decay, cudaStream_t s) {
  if (n == 0) {
    return cudaSuccess;
  }
  dev::k_ema<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(avg, param, n, decay);
  return cudaGetLastError();
}

cudaError_t launch_adam(float *param, float *grad, float *m, float *v, size_t n, float lr,
                        float beta1, float beta2, float eps, float step, cudaStream_t s) {
  if (n == 0) {
    return cudaSuccess;
  }
  dev::k_adam<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(param, grad, m, v, n, lr, beta1,
                                                           beta2, eps, step);
  return cudaGetLastError();
}

} // namespace pg

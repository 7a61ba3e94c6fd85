// MLP path guide: fused tcgen05 kernels for inference, training (forward,
// loss gradient, backward) and Adam.  The renderer trains with
// k_guide_train_rounds (every Adam round of a wave in one cooperative
// launch); k_guide_train + k_guide_adam are the same steps as separate
// launches, for the guide's own C ABI.
//
// Network: 64 encoded inputs -> 4 x (64, ReLU) -> 40 outputs = 8 vMF lobes
// (guide_mix.cuh).  FP32 master weights; BF16 copies, pre-swizzled into the
// K-major 128-byte-swizzle layout the UMMA descriptors expect, are copied
// into each CTA's shared memory.  A training CTA of 128 threads processes
// tiles of 128 samples: thread t owns row t of every activation tile, and
// TMEM lane t of every accumulator.  One elected thread issues tcgen05.mma (M = 128,
// K = 16 per instruction) and commits to an mbarrier; waits are bounded and
// a time-out sets a status bit instead of hanging.
//
// Backward of layer l (weights W_l: out x in; its input H_{l-1} is
// activation tile l, rows = samples):
//   dH_{l-1} = dZ_l W_l          A = dZ_l tile [b][o] (K-major, K = o),
//                                B = W_l^T rows
//   dW_l    += dZ_l^T H_{l-1}    A = [H_{l-1}^T ; dZ_l^T] (M = 128, K = batch),
//                                B = H_{l-1}^T; rows 64..127 of D are dW_l
// dW reads the row-per-sample tiles as MN-major operands, so nothing is
// transposed: dZ_l is written to tile l + 1 (dead by then: its last reader
// was the ReLU mask of layer l + 1), one 16 KB tile after H_{l-1}, which is
// the stride between A's two 64-row blocks.  dW accumulates in TMEM across
// all tiles of the CTA and is added to the global FP32 gradient once at the
// end.
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "guide.cuh"
#include "guide_infer.cuh"
#include "guide_mix.cuh"
#include "lisa_device.cuh"
#include "tcgen05.cuh"

namespace lisa {

// master -> packed BF16 (forward and transposed copies)
__global__ void k_guide_pack(const float* __restrict__ master, uint16_t* __restrict__ pack) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;  // one element of the 560 x 64 image
  if (e >= R_TOTAL * 64) return;
  const int row = e >> 6, k = e & 63;
  float v = 0.0f;
  if (row < R_W5) {
    const int l = row >> 6, o = row & 63;
    v = master[P_W + l * 4096 + o * 64 + k];
  } else if (row < R_T) {
    const int o = row - R_W5;
    v = o < 40 ? master[P_W5 + o * 64 + k] : 0.0f;
  } else {
    const int l = 1 + ((row - R_T) >> 6);  // W2..W5 (0-based layer 1..4)
    const int i = (row - R_T) & 63, o = k;
    if (l < 4) v = master[P_W + l * 4096 + o * 64 + i];
    else v = o < 40 ? master[P_W5 + o * 64 + i] : 0.0f;
  }
  uint8_t* base = (uint8_t*)pack + (size_t)(row & ~7) * 128;
  *(uint16_t*)(base + tc::sw128_offset(row & 7, k)) = f2bf(v);
}


// One Adam update (Kingma & Ba 2015; beta1 0.9, beta2 0.999, eps 1e-8) of
// weight w with gradient g; m, v in/out.  Written with explicitly rounded
// operations (no contraction), so the separate Adam kernel and the training
// rounds give the same bits.
__device__ __forceinline__ float adam_update(float w, float g, float& m, float& v, float lr, float b1c, float b2c) {
  m = __fadd_rn(__fmul_rn(0.9f, m), __fmul_rn(0.1f, g));
  v = __fadd_rn(__fmul_rn(0.999f, v), __fmul_rn(__fmul_rn(0.001f, g), g));
  const float step = __fdiv_rn(__fmul_rn(lr, __fdiv_rn(m, b1c)), __fadd_rn(__fsqrt_rn(__fdiv_rn(v, b2c)), 1e-8f));
  return __fsub_rn(w, step);
}

__device__ __forceinline__ void pack_store(uint16_t* pack, int row, int col, float v) {
  uint8_t* base = (uint8_t*)pack + (size_t)(row & ~7) * 128;
  *(uint16_t*)(base + tc::sw128_offset(row & 7, col)) = f2bf(v);
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters, fused with what
// surrounds a step: the gradient is the sum of the training CTAs' partial
// gradients, the BF16 forward and transposed copies of each updated weight
// are written in place (the zero padding rows never change), and the summed
// loss goes to loss_last.  The step count lives on the device (the training
// kernel increments it).
__global__ void k_guide_adam(float* __restrict__ master, float* __restrict__ m, float* __restrict__ v,
                             const float* __restrict__ part, const float* __restrict__ loss_part, uint32_t nparts,
                             float* __restrict__ loss_last, float lr, const uint32_t* __restrict__ step,
                             uint32_t* status, uint16_t* __restrict__ pack) {
  // four threads per parameter (neighbouring lanes) each sum every fourth
  // partial slot; the sums meet by shuffles
  const int t4 = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t4 >> 2, q = t4 & 3;
  if (t4 == 0) {
    float l = 0.0f;
    for (uint32_t c = 0; c < nparts; ++c) l += loss_part[c];
    *loss_last = l;
  }
  float gi = 0.0f;
  if (i < NPARAM) {
#pragma unroll 8
    for (uint32_t c = q; c < nparts; c += 4) gi += part[(size_t)c * NPARAM + i];
  }
  gi += __shfl_xor_sync(0xffffffffu, gi, 1);
  gi += __shfl_xor_sync(0xffffffffu, gi, 2);
  if (i >= NPARAM || q != 0) return;
  const float t = (float)max(*step, 1u);
  const float b1c = 1.0f - powf(0.9f, t), b2c = 1.0f - powf(0.999f, t);
  if (!isfinite(gi)) {
    atomicOr(status, ST_GUIDE_NONFINITE);
    return;
  }
  float mi = m[i], vi = v[i];
  const float w = adam_update(master[i], gi, mi, vi, lr, b1c, b2c);
  m[i] = mi;
  v[i] = vi;
  master[i] = w;
  if (i < P_W5) {  // W1..W4 (output o, input k): forward row l*64+o; transposed for l >= 1
    const int l = i >> 12, o = (i >> 6) & 63, k = i & 63;
    pack_store(pack, R_FWD + l * 64 + o, k, w);
    if (l >= 1) pack_store(pack, R_T + (l - 1) * 64 + k, o, w);
  } else if (i < P_B) {  // W5: forward row R_W5+o, transposed block 3
    const int o = (i - P_W5) >> 6, k = (i - P_W5) & 63;
    pack_store(pack, R_W5 + o, k, w);
    pack_store(pack, R_T + 3 * 64 + k, o, w);
  }
}

// ---------------------------------------------------------------------------------
// inference: out[i][0..39] = network(features_i)

// Sum of the partial gradients and losses (for callers that read them).
__global__ void k_guide_reduce(const float* __restrict__ part, const float* __restrict__ loss_part, uint32_t nparts,
                               float* __restrict__ grads, float* __restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    float l = 0.0f;
    for (uint32_t c = 0; c < nparts; ++c) l += loss_part[c];
    *loss = l;
  }
  if (i >= NPARAM) return;
  float gi = 0.0f;
  for (uint32_t c = 0; c < nparts; ++c) gi += part[(size_t)c * NPARAM + i];
  grads[i] = gi;
}

template <int SRC>
__global__ void __launch_bounds__(INFER_THREADS, INFER_BLOCKS_PER_SM) k_guide_infer(const uint16_t* __restrict__ pack,
                                                                          const float* __restrict__ master,
                                                                          GuideSrc src, float* __restrict__ out,
                                                                          uint32_t* status) {
  infer_tiles<SRC>(pack, master, src, status, [](uint32_t) {}, [&](uint32_t i, bool valid, const float* o) {
    if (!valid) return;
    float4* d = reinterpret_cast<float4*>(out + 40ull * i);
#pragma unroll
    for (int k = 0; k < 10; ++k) d[k] = make_float4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
  });
}

// ---------------------------------------------------------------------------------
// training: grads += d loss / d params, loss += sum of the per-sample losses

constexpr int TILE = 16384;
// tiles X, H1..H4 (tile l = the input of layer l), a sixth tile for dZ of
// the output layer, and a seventh that no step writes: the dW steps of the
// output layer read at most 32 KB past the start of tile 4 (two 1024-byte
// K atoms and two 64-row blocks, whichever of the descriptor's two strides
// the hardware takes for which), so every operand read stays inside the
// allocation
constexpr int TRAIN_OFF_ACT = PACK_BYTES;
constexpr int TRAIN_SMEM_USED = TRAIN_OFF_ACT + 7 * TILE;
constexpr int TRAIN_SMEM = TRAIN_SMEM_USED + 1024 + 2048;  // manual 1024-B alignment, slack
static_assert(TRAIN_SMEM <= 227 * 1024, "training kernel shared memory");
constexpr uint32_t TM_FWD = 0, TM_DH = 64, TM_DW = 128;  // TMEM columns; dW_l at 128 + 64 l

// One halving round of a warp reduce-scatter: the lane keeps the upper or
// lower half of its n values (by lane bit m) plus the partner's same half.
template <int N>
__device__ __forceinline__ void reduce_scatter_round(const float* in, float* out, int m) {
  const bool up = (threadIdx.x & m) != 0;
#pragma unroll
  for (int k = 0; k < N / 2; ++k) {
    const float send = up ? in[k] : in[k + N / 2];
    const float keep = up ? in[k + N / 2] : in[k];
    out[k] = keep + __shfl_xor_sync(0xffffffffu, send, m);
  }
}

// Column sums of the warp's 32 rows of v[64] added to the warp's own
// s_db[0 .. count): a reduce-scatter by recursive halving leaves each lane
// two of the 64 column sums (different columns in different lanes), which
// it adds with plain stores -- no atomics, so the sums are the same in
// every run.
__device__ __forceinline__ void add_bias_grad(float* s_db, const float* v, int count) {
  float a[32], b[16], c[8], d[4], e[2];
  reduce_scatter_round<64>(v, a, 16);
  reduce_scatter_round<32>(a, b, 8);
  reduce_scatter_round<16>(b, c, 4);
  reduce_scatter_round<8>(c, d, 2);
  reduce_scatter_round<4>(d, e, 1);
  const int lane = threadIdx.x & 31;
  const int col = ((lane & 16) ? 32 : 0) + ((lane & 8) ? 16 : 0) + ((lane & 4) ? 8 : 0) + ((lane & 2) ? 4 : 0) +
                  ((lane & 1) ? 2 : 0);
  if (col < count) s_db[col] += e[0];
  if (col + 1 < count) s_db[col + 1] += e[1];
}

constexpr int DB_WORDS = 4 * 64 + 40;  // bias gradients of the five layers

// Bias gradient k (or, for k == DB_WORDS, the loss) of the CTA: the four
// warps' sums in warp order.
__device__ __forceinline__ float bias_grad_total(const float* s_db, const float* s_loss, int k) {
  if (k == DB_WORDS) return ((s_loss[0] + s_loss[1]) + s_loss[2]) + s_loss[3];
  return ((s_db[k] + s_db[DB_WORDS + k]) + s_db[2 * DB_WORDS + k]) + s_db[3 * DB_WORDS + k];
}

// Forward, loss gradient and backward of one 128-sample tile (thread t owns
// sample i = row t): dW accumulates in TMEM (initialised by the first tile
// of a batch), db and the loss in per-warp shared-memory sums (s_db: 4 x
// DB_WORDS, s_loss: 4), added up in warp order by bias_grad_total.  The caller has the weights
// (w) and biases (s_b) in shared memory and has met at a barrier since.
template <int SRC>
__device__ __forceinline__ void train_tile(const GuideSrc& src, uint32_t i, uint32_t n, float inv_n, uint8_t* w,
                                           uint8_t* act, uint32_t tmem, uint32_t lane_off, uint64_t* mbar,
                                           uint32_t& phase, bool first, volatile int* failed, uint32_t* status,
                                           const float* s_b, float* s_db, float* s_loss) {
  const int tid = threadIdx.x;
  auto wait_mma = [&]() {
    if (tid == 0 && !tc::mbar_wait(mbar, phase)) {
      atomicOr(status, ST_GUIDE_NONFINITE << 1);
      *failed = 1;
    }
    phase ^= 1;
    __syncthreads();
    tc::fence_after_sync();
  };
  auto sync_for_mma = [&]() {
    tc::fence_smem_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  };
  const bool valid = i < n;
  float v[64];
  float wx = 0.0f, wy = 0.0f, wz = 1.0f, wt = 0.0f;
  if (valid) {
    load_features<SRC>(src, i, v);
    if (SRC == SRC_RAW) {
      wx = __ldg(src.dirs + 3ull * i);
      wy = __ldg(src.dirs + 3ull * i + 1);
      wz = __ldg(src.dirs + 3ull * i + 2);
      wt = __ldg(src.weights + i);
    } else {
      const float4 c = src.geom[4ull * i + 2], d = src.geom[4ull * i + 3];
      wx = c.y;
      wy = c.z;
      wz = c.w;
      wt = d.x;
    }
  } else {
#pragma unroll
    for (int k = 0; k < 64; ++k) v[k] = 0.0f;
  }
  store_row_bf16(act, tid, v);
  // forward
  for (int l = 0; l < 5; ++l) {
    sync_for_mma();
    const uint32_t N = l < 4 ? 64u : 48u;
    if (tid == 0) issue_layer(tmem + TM_FWD, act + l * TILE, w + (l < 4 ? (R_FWD + 64 * l) : R_W5) * 128, N, mbar);
    wait_mma();
    if (*failed) return;
    if (l < 4) {
      tc::tmem_ld16x<4>(tmem + TM_FWD + lane_off, v);
      store_row_bias_relu(act + (l + 1) * TILE, tid, v, s_b + 64 * l);
    } else {
      tc::tmem_ld16x<3>(tmem + TM_FWD + lane_off, v);
    }
    tc::fence_before_sync();
  }
  // loss gradient at the output (40 values, padded with zeros to 64)
  float g[64];
  {
    float o[40];
#pragma unroll
    for (int k = 0; k < 40; ++k) o[k] = v[k] + s_b[4 * 64 + k];
    float lsum = 0.0f;
    if (valid && wt != 0.0f) {
      const float il = rsqrtf(fmaxf(wx * wx + wy * wy + wz * wz, 1e-30f));
      lsum = guide::loss_grad(o, wx * il, wy * il, wz * il, wt * inv_n, g);
    } else {
#pragma unroll
      for (int k = 0; k < 40; ++k) g[k] = 0.0f;
    }
#pragma unroll
    for (int k = 40; k < 64; ++k) g[k] = 0.0f;
#pragma unroll
    for (int o2 = 16; o2 > 0; o2 >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o2);
    if ((tid & 31) == 0) s_loss[tid >> 5] += lsum;
  }
  float* const s_dbw = s_db + (tid >> 5) * DB_WORDS;  // this warp's sums
  add_bias_grad(s_dbw + 4 * 64, g, 40);
  // backward, layer 5 (index 4) down to layer 1 (index 0)
  for (int l = 4; l >= 0; --l) {
    // dZ_l (registers g) -> tile l + 1: A of dH (K-major) and the upper
    // 64-row block of A of dW (MN-major)
    uint8_t* tl = act + l * TILE;
    store_row_bf16(tl + TILE, tid, g);
    sync_for_mma();
    if (tid == 0) {
      // dW_l += [H^T ; dZ^T] x (H^T)^T over the 128 samples (K = 128):
      // both operands MN-major, 16 samples (two 8-row atoms) per step
      const uint32_t idesc_mn = tc::idesc_bf16_f32_mn(128, 64);
      const uint32_t sh = tc::smem_u32(tl);
#pragma unroll
      for (uint32_t ks = 0; ks < 8; ++ks) {
        const uint32_t base = sh + ks * 2048;
        tc::mma_bf16(tmem + TM_DW + 64 * l, tc::sw128_mn_desc(base, TILE), tc::sw128_mn_desc(base, TILE), idesc_mn,
                     (first && ks == 0) ? 0u : 1u);
      }
      if (l > 0) {
        // dH_{l-1} = dZ_l W_l  (B = W_l^T rows)
        const uint32_t idesc = tc::idesc_bf16_f32(128, 64);
        const uint32_t sdz = sh + TILE, swt = tc::smem_u32(w + (R_T + 64 * (l - 1)) * 128);
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k)
          tc::mma_bf16(tmem + TM_DH, tc::sw128_desc(sdz + 32 * k), tc::sw128_desc(swt + 32 * k), idesc, k);
      }
      tc::mma_commit(mbar);
    }
    wait_mma();
    if (*failed) return;
    if (l > 0) {
      // dZ_{l-1} = dH_{l-1} where H_{l-1} > 0: the BF16 bits of this
      // sample's row of tile l, +-0 masked out
      tc::tmem_ld16x<4>(tmem + TM_DH + lane_off, g);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const uint4 q = *(const uint4*)(tl + tid * 128 + ((c ^ (tid & 7)) << 4));
        const uint32_t hw[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if ((hw[j] & 0x7fffu) == 0u) g[8 * c + 2 * j] = 0.0f;
          if ((hw[j] & 0x7fff0000u) == 0u) g[8 * c + 2 * j + 1] = 0.0f;
        }
      }
      add_bias_grad(s_dbw + 64 * (l - 1), g, 64);
    }
    tc::fence_before_sync();
  }
}

// Reads this thread's row o (< 64) of dW_l, l = 0..4 (rows 64..127 of the
// accumulators: the TMEM lanes of warps 2 and 3), and hands each layer's
// row to put(l, o, d) when the layer has that row (W5 has 40).
template <class Put>
__device__ __forceinline__ void flush_dw(uint32_t tmem, uint32_t lane_off, bool ok, Put&& put) {
  const int warp = threadIdx.x >> 5;
  if (warp < 2) return;
  const int o = (warp - 2) * 32 + (threadIdx.x & 31);
  for (int l = 0; l < 5; ++l) {
    const int rows = l < 4 ? 64 : 40;
    float d[64];
    if (ok) {
#pragma unroll
      for (int c = 0; c < 4; ++c) tc::tmem_ld16(tmem + TM_DW + 64 * l + lane_off + c * 16, d + c * 16);
    } else {
#pragma unroll
      for (int c = 0; c < 64; ++c) d[c] = 0.0f;
    }
    if (o < rows) put(l, o, d);
  }
}

template <int SRC>
__global__ void __launch_bounds__(128, 1) k_guide_train(const uint16_t* __restrict__ pack, const float* __restrict__ master,
                                                        GuideSrc src, float inv_n, float* __restrict__ part,
                                                        float* __restrict__ loss_part, uint32_t* status,
                                                        uint32_t* __restrict__ step_bump) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* w = smem;
  uint8_t* act = smem + TRAIN_OFF_ACT;  // tile l = the input of layer l (tile 0 = X)
  __shared__ uint64_t mbar;
  __shared__ uint64_t mbar_w;  // the packed weights' bulk copy
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  __shared__ float s_db[4 * DB_WORDS];  // per warp
  __shared__ __align__(16) float s_b[4 * 64 + 48];  // biases
  __shared__ float s_loss[4];
  const int tid = threadIdx.x, warp = tid >> 5;
  // samples [src.first, n)
  const uint32_t n = max(src.count ? min(*(volatile const uint32_t*)src.count, src.n) : src.n, src.first);
  const uint32_t ntiles = (n - src.first + 127) / 128;
  // the Adam step that follows (none for an empty slice)
  if (step_bump && n > src.first && blockIdx.x == 0 && threadIdx.x == 0) *step_bump += 1;
  float* slot = part + (size_t)blockIdx.x * NPARAM;  // this CTA's partial gradient
  if (blockIdx.x >= ntiles) {
    for (int k = threadIdx.x; k < NPARAM; k += blockDim.x) slot[k] = 0.0f;
    if (threadIdx.x == 0) loss_part[blockIdx.x] = 0.0f;
    return;
  }
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    tc::mbar_init(&mbar_w, 1);
    tc::fence_mbar_init();
    tc::bulk_load(w, pack, PACK_BYTES, &mbar_w);  // weights by TMA while the rest is set up
    failed = 0;
  }
  if (tid < 4) s_loss[tid] = 0.0f;
  for (int k = tid; k < 4 * DB_WORDS; k += 128) s_db[k] = 0.0f;
  if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
  for (int k = tid; k < 4 * 64 + 48; k += 128) s_b[k] = k < 4 * 64 + 40 ? __ldg(master + P_B + k) : 0.0f;
  if (tid == 0 && !tc::mbar_wait(&mbar_w, 0)) {
    atomicOr(status, ST_GUIDE_NONFINITE << 1);
    failed = 1;
  }
  tc::fence_smem_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
  uint32_t phase = 0;
  bool first = true;
  for (uint32_t t = blockIdx.x; t < ntiles && !failed; t += gridDim.x) {
    train_tile<SRC>(src, src.first + t * 128 + tid, n, inv_n, w, act, tmem, lane_off, &mbar, phase, first, &failed,
                    status, s_b, s_db, s_loss);
    first = false;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const bool ok = !failed && !first;
  flush_dw(tmem, lane_off, ok, [&](int l, int o, const float* d) {
    float4* gw = reinterpret_cast<float4*>(slot + (l < 4 ? P_W + l * 4096 : P_W5) + o * 64);
#pragma unroll
    for (int k = 0; k < 16; ++k) gw[k] = make_float4(d[4 * k], d[4 * k + 1], d[4 * k + 2], d[4 * k + 3]);
  });
  __syncthreads();
  for (int k = tid; k < DB_WORDS; k += 128) slot[P_B + k] = ok ? bias_grad_total(s_db, s_loss, k) : 0.0f;
  if (tid == 0) loss_part[blockIdx.x] = ok ? bias_grad_total(s_db, s_loss, DB_WORDS) : 0.0f;
  if (tid == 0 && failed) {
    tc::mbar_wait(&mbar_w, 0, 1u << 20);       // a late weight copy: bounded second chance
    tc::mbar_wait(&mbar, phase ^ 1u, 1u << 20);  // and an MMA still in flight
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// All CTAs of a cooperative grid meet here: the k-th barrier of a launch
// completes when the arrival counter (zeroed before the launch) reaches
// (k + 1) x gridDim.x.  Memory written before the barrier (with a device
// fence) is visible after it to loads that bypass L1.  The wait has an
// iteration limit; false (the same in every thread of the CTA) when it
// ran out, with the status bit set.
__device__ __forceinline__ bool grid_barrier(uint32_t* counter, uint32_t k, uint32_t* status, volatile int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(counter, 1u);
    const uint32_t target = (k + 1) * gridDim.x;
    bool ok = false;
    for (uint32_t it = 0; it < (1u << 22); ++it) {
      uint32_t v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(counter) : "memory");
      if (v >= target) {
        ok = true;
        break;
      }
      __nanosleep(64);
    }
    if (!ok) atomicOr(status, ST_GUIDE_NONFINITE << 1);
    *s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  return *s_ok != 0;
}

// One wave's training rounds in one cooperative launch (one CTA per SM, all
// resident): for each slice of `chunk` samples [s * chunk, (s + 1) * chunk)
// of the batch (while the batch has samples), every CTA
//   1. reads the current weights (a bulk copy behind a proxy fence) and
//      biases (loads that bypass L1): other CTAs wrote them last round,
//   2. runs its tiles of the slice (forward, loss gradient, backward),
//   3. writes its dW, db and loss to its own slot of part / loss_part,
// the grid meets, CTA c sums the slots over its share of 128 parameters
// (the same order as k_guide_adam: deterministic) and applies Adam to
// them, refreshing their FP32 master and BF16 forward / transposed copies,
// and the grid meets again.  The same steps as a training launch followed
// by an Adam launch per slice, without their launches and per-launch
// set-up.  grid_bar: the grid barrier's arrival counter, zero at launch.
constexpr uint32_t ADAM_SHARE = 128;  // parameters per CTA in the Adam phase (a multiple of 4)

template <int SRC>
__global__ void __launch_bounds__(128, 1) k_guide_train_rounds(uint16_t* __restrict__ pack, float* __restrict__ master,
                                                               float* __restrict__ adam_m, float* __restrict__ adam_v,
                                                               GuideSrc src, uint32_t chunk, uint32_t rounds,
                                                               float lr, float* __restrict__ part,
                                                               float* __restrict__ loss_part, uint32_t* grid_bar,
                                                               float* __restrict__ loss_last, uint32_t* step_count,
                                                               uint32_t* status,
                                                               unsigned long long* __restrict__ sample_count) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* w = smem;
  uint8_t* act = smem + TRAIN_OFF_ACT;
  __shared__ uint64_t mbar;
  __shared__ uint64_t mbar_w;  // the weights' bulk copy, once per round
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  __shared__ int bar_ok;
  __shared__ float s_db[4 * DB_WORDS];  // per warp
  __shared__ __align__(16) float s_b[4 * 64 + 48];
  __shared__ float s_loss[4];
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t n = src.count ? min(*(volatile const uint32_t*)src.count, src.n) : src.n;
  const uint32_t t0 = *(volatile const uint32_t*)step_count;  // Adam steps before this launch
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    tc::mbar_init(&mbar_w, 1);
    tc::fence_mbar_init();
    failed = 0;
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
  const float inv_n = 1.0f / (float)chunk;
  // the Adam phase: for each share of 128 parameters p0.. of this CTA,
  // thread (g, q) = (tid / 4, tid % 4) sums the slots j = q (mod 4) of
  // parameters p0 + 4 g .. + 3 (one float4 a slot); the quad's sums meet by
  // shuffles and thread (g, q) updates parameter p0 + 4 g + q
  const uint32_t qq = tid & 3;
  float* slot = part + (size_t)blockIdx.x * NPARAM;
  uint32_t phase = 0, wphase = 0, bars = 0, done = 0;
  bool w_busy = false;  // thread 0: a weight copy not waited for
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t first = r * chunk;
    if (first >= n) break;  // the same in every CTA
    const uint32_t last = min(first + chunk, n);
    // 1. weights (bulk copy; the other CTAs' generic-proxy writes of the
    // last round are ordered before it by the grid barrier and the proxy
    // fence) and biases (loads that bypass L1)
    if (tid == 0) {
      asm volatile("fence.proxy.async.global;" ::: "memory");
      tc::bulk_load(w, pack, PACK_BYTES, &mbar_w);
      w_busy = true;
    }
    for (int k = tid; k < 4 * 64 + 48; k += 128) s_b[k] = k < 4 * 64 + 40 ? __ldcg(master + P_B + k) : 0.0f;
    for (int k = tid; k < 4 * DB_WORDS; k += 128) s_db[k] = 0.0f;
    if (tid < 4) s_loss[tid] = 0.0f;
    if (tid == 0) {
      if (tc::mbar_wait(&mbar_w, wphase)) {
        w_busy = false;
      } else {
        atomicOr(status, ST_GUIDE_NONFINITE << 1);
        failed = 1;
      }
      wphase ^= 1u;
    }
    tc::fence_smem_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // 2. this CTA's tiles of the slice
    const uint32_t ntiles = (last - first + 127) / 128;
    bool any = false;
    for (uint32_t t = blockIdx.x; t < ntiles && !failed; t += gridDim.x) {
      train_tile<SRC>(src, first + t * 128 + tid, last, inv_n, w, act, tmem, lane_off, &mbar, phase, !any, &failed,
                      status, s_b, s_db, s_loss);
      any = true;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // 3. this CTA's slot (zeros when it had no tile this round)
    const bool ok = any && !failed;
    flush_dw(tmem, lane_off, ok, [&](int l, int o, const float* d) {
      float4* gw = reinterpret_cast<float4*>(slot + (l < 4 ? P_W + l * 4096 : P_W5) + o * 64);
#pragma unroll
      for (int k = 0; k < 16; ++k) gw[k] = make_float4(d[4 * k], d[4 * k + 1], d[4 * k + 2], d[4 * k + 3]);
    });
    for (int k = tid; k < DB_WORDS; k += 128) slot[P_B + k] = ok ? bias_grad_total(s_db, s_loss, k) : 0.0f;
    if (tid == 0) loss_part[blockIdx.x] = ok ? bias_grad_total(s_db, s_loss, DB_WORDS) : 0.0f;
    if (!grid_barrier(grid_bar, bars++, status, &bar_ok) || failed) break;
    // Adam on this CTA's share (the step of k_guide_adam)
    const float t = (float)(t0 + done + 1);
    const float b1c = 1.0f - powf(0.9f, t), b2c = 1.0f - powf(0.999f, t);
    if (blockIdx.x == 0 && warp == 0) {
      float l = 0.0f;
      for (uint32_t j = tid; j < gridDim.x; j += 32) l += __ldcg(loss_part + j);
#pragma unroll
      for (int m = 16; m > 0; m >>= 1) l += __shfl_xor_sync(0xffffffffu, l, m);
      if (tid == 0) *loss_last = l;
    }
    for (uint32_t p0 = blockIdx.x * ADAM_SHARE; p0 < (uint32_t)NPARAM; p0 += gridDim.x * ADAM_SHARE) {
      const uint32_t pq = p0 + 4u * (tid >> 2);
      float4 g4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (pq < (uint32_t)NPARAM) {
        // (sixteen slots in flight per thread: the sum is latency-bound)
#pragma unroll 16
        for (uint32_t j = qq; j < gridDim.x; j += 4) {
          const float4 x = __ldcg(reinterpret_cast<const float4*>(part + (size_t)j * NPARAM + pq));
          g4.x += x.x;
          g4.y += x.y;
          g4.z += x.z;
          g4.w += x.w;
        }
      }
#pragma unroll
      for (int m = 1; m <= 2; m <<= 1) {
        g4.x += __shfl_xor_sync(0xffffffffu, g4.x, m);
        g4.y += __shfl_xor_sync(0xffffffffu, g4.y, m);
        g4.z += __shfl_xor_sync(0xffffffffu, g4.z, m);
        g4.w += __shfl_xor_sync(0xffffffffu, g4.w, m);
      }
      const uint32_t i = pq + qq;
      const float gi = qq == 0 ? g4.x : qq == 1 ? g4.y : qq == 2 ? g4.z : g4.w;
      if (i < (uint32_t)NPARAM) {
        if (!isfinite(gi)) atomicOr(status, ST_GUIDE_NONFINITE);
        else {
          float mi = __ldcg(adam_m + i), vi = __ldcg(adam_v + i);
          const float wv = adam_update(__ldcg(master + i), gi, mi, vi, lr, b1c, b2c);
          adam_m[i] = mi;
          adam_v[i] = vi;
          master[i] = wv;
          if (i < P_W5) {
            const int l = i >> 12, o = (i >> 6) & 63, k = i & 63;
            pack_store(pack, R_FWD + l * 64 + o, k, wv);
            if (l >= 1) pack_store(pack, R_T + (l - 1) * 64 + k, o, wv);
          } else if (i < P_B) {
            const int o = (i - P_W5) >> 6, k = (i - P_W5) & 63;
            pack_store(pack, R_W5 + o, k, wv);
            pack_store(pack, R_T + 3 * 64 + k, o, wv);
          }
        }
      }
    }
    asm volatile("fence.proxy.async.global;" ::: "memory");  // the pack, read next round by bulk copies
    ++done;
    if (!grid_barrier(grid_bar, bars++, status, &bar_ok)) break;
  }
  if (blockIdx.x == 0 && tid == 0) {
    *step_count = t0 + done;
    if (sample_count) *sample_count += min(n, done * chunk);
  }
  // after a time-out, an MMA may still be in flight (its completion has the
  // parity before the last toggle): a bounded chance to finish before its
  // TMEM is freed
  if (tid == 0 && failed) tc::mbar_wait(&mbar, phase ^ 1u, 1u << 20);
  if (tid == 0 && w_busy) tc::mbar_wait(&mbar_w, wphase ^ 1u, 1u << 20);  // a late weight copy
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------------
// host

GuideNet::~GuideNet() {
  if (master) cudaFree(master);
  if (adam_m) cudaFree(adam_m);
  if (adam_v) cudaFree(adam_v);
  if (grads) cudaFree(grads);
  if (w_bf16) cudaFree(w_bf16);
  if (loss) cudaFree(loss);
  if (loss_last) cudaFree(loss_last);
  if (status) cudaFree(status);
  if (d_step) cudaFree(d_step);
  if (owns_part) {
    if (grad_part) cudaFree(grad_part);
    if (loss_part) cudaFree(loss_part);
  }
}

namespace {

Status guide_alloc(GuideNet& g) {
  LISA_CUDA(cudaMalloc(&g.master, sizeof(float) * NPARAM));
  LISA_CUDA(cudaMalloc(&g.adam_m, sizeof(float) * NPARAM));
  LISA_CUDA(cudaMalloc(&g.adam_v, sizeof(float) * NPARAM));
  LISA_CUDA(cudaMalloc(&g.grads, sizeof(float) * NPARAM));
  LISA_CUDA(cudaMalloc(&g.w_bf16, PACK_BYTES));
  LISA_CUDA(cudaMalloc(&g.loss, sizeof(float)));
  LISA_CUDA(cudaMalloc(&g.loss_last, sizeof(float)));
  LISA_CUDA(cudaMalloc(&g.status, sizeof(uint32_t)));
  LISA_CUDA(cudaMalloc(&g.d_step, sizeof(uint32_t)));
  LISA_CUDA(cudaMemset(g.d_step, 0, sizeof(uint32_t)));
  LISA_CUDA(cudaMemset(g.adam_m, 0, sizeof(float) * NPARAM));
  LISA_CUDA(cudaMemset(g.adam_v, 0, sizeof(float) * NPARAM));
  LISA_CUDA(cudaMemset(g.grads, 0, sizeof(float) * NPARAM));
  LISA_CUDA(cudaMemset(g.loss, 0, sizeof(float)));
  LISA_CUDA(cudaMemset(g.loss_last, 0, sizeof(float)));
  LISA_CUDA(cudaMemset(g.status, 0, sizeof(uint32_t)));
  return Status();
}

// He-uniform weights (ReLU layers), small output layer, zero biases; the
// kappa logits start at log(2).
std::vector<float> guide_init(uint32_t seed) {
  std::vector<float> p(NPARAM, 0.0f);
  std::mt19937 gen(seed * 2654435761u + 12345u);
  const float a = std::sqrt(6.0f / 64.0f);
  std::uniform_real_distribution<float> U(-a, a), U5(-0.1f, 0.1f);
  for (int i = 0; i < 4 * 4096; ++i) p[P_W + i] = U(gen);
  for (int i = 0; i < 40 * 64; ++i) p[P_W5 + i] = U5(gen);
  for (int k = 0; k < 8; ++k) p[P_B5 + 5 * k + 3] = std::log(2.0f);
  return p;
}

}  // namespace

static int sm_count_current() {
  int dev = 0, sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
  return sm > 0 ? sm : 1;
}

// Partial-gradient slots for `slots` training CTAs.
Status guide_alloc_partials(float** grad_part, float** loss_part, uint32_t slots) {
  LISA_CUDA(cudaMalloc(grad_part, sizeof(float) * (size_t)NPARAM * slots));
  LISA_CUDA(cudaMalloc(loss_part, sizeof(float) * slots));
  return Status();
}

Status guide_pack(GuideNet& g, cudaStream_t s) {
  k_guide_pack<<<(R_TOTAL * 64 + 255) / 256, 256, 0, s>>>(g.master, g.w_bf16);
  LISA_CUDA(cudaGetLastError());
  return Status();
}

Status guide_create(uint32_t seed, std::unique_ptr<GuideNet>& out, cudaStream_t s, bool own_partials) {
  std::unique_ptr<GuideNet> g(new GuideNet());
  LISA_TRY(guide_alloc(*g));
  if (own_partials) {
    g->owns_part = true;
    LISA_TRY(guide_alloc_partials(&g->grad_part, &g->loss_part, (uint32_t)sm_count_current()));
  }
  std::vector<float> p = guide_init(seed);
  LISA_CUDA(cudaMemcpyAsync(g->master, p.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice, s));
  LISA_TRY(guide_pack(*g, s));
  LISA_CUDA(cudaStreamSynchronize(s));
  static bool attr_set = false;
  if (!attr_set) {
    LISA_CUDA(cudaFuncSetAttribute(k_guide_train<SRC_RAW>, cudaFuncAttributeMaxDynamicSharedMemorySize, TRAIN_SMEM));
    LISA_CUDA(cudaFuncSetAttribute(k_guide_infer<SRC_RAW>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM));
    LISA_CUDA(cudaFuncSetAttribute(k_guide_infer<SRC_NEE>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM));
    attr_set = true;
  }
  out = std::move(g);
  return Status();
}

Status guide_launch_infer(GuideNet& g, const GuideSrc& src, int src_kind, float* out, uint32_t max_n, cudaStream_t s) {
  const uint32_t pairs = std::max<uint32_t>(1, (max_n + 255) / 256);  // two tiles of 128 per CTA
  const uint32_t grid = std::min<uint32_t>(pairs, (uint32_t)sm_count_current() * INFER_BLOCKS_PER_SM);
  if (src_kind == SRC_RAW)
    k_guide_infer<SRC_RAW><<<grid, INFER_THREADS, INFER_SMEM, s>>>(g.w_bf16, g.master, src, out, g.status);
  else
    k_guide_infer<SRC_NEE><<<grid, INFER_THREADS, INFER_SMEM, s>>>(g.w_bf16, g.master, src, out, g.status);
  LISA_CUDA(cudaGetLastError());
  return Status();
}

// Gradient of one batch: every training CTA writes its partial gradient and
// loss to its own slot of g.grad_part / g.loss_part (no atomics); the Adam
// step (or guide_launch_reduce) sums them.  With adam_follows the device
// step count advances for the Adam step launched next.
Status guide_launch_train(GuideNet& g, const GuideSrc& src, float inv_n, uint32_t max_n, cudaStream_t s,
                          bool adam_follows) {
  if (!g.grad_part) return Status::invalid("guide: no partial-gradient slots");
  const uint32_t tiles = std::max<uint32_t>(1, (max_n + 127) / 128);
  const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)sm_count_current());
  g.nparts = grid;
  uint32_t* bump = adam_follows ? g.d_step : nullptr;
  k_guide_train<SRC_RAW><<<grid, 128, TRAIN_SMEM, s>>>(g.w_bf16, g.master, src, inv_n, g.grad_part, g.loss_part,
                                                       g.status, bump);
  LISA_CUDA(cudaGetLastError());
  return Status();
}

// One wave's training rounds (k_guide_train_rounds), a cooperative launch
// of one CTA per SM; grid_bar (one word) is zeroed first.
Status guide_launch_train_rounds(GuideNet& g, const GuideSrc& src, int src_kind, uint32_t chunk, uint32_t rounds,
                                 float lr, uint32_t* grid_bar, cudaStream_t s, unsigned long long* sample_count) {
  static bool attr_set = false;
  if (!attr_set) {
    LISA_CUDA(cudaFuncSetAttribute(k_guide_train_rounds<SRC_GEOM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   TRAIN_SMEM));
    LISA_CUDA(cudaFuncSetAttribute(k_guide_train_rounds<SRC_RAW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   TRAIN_SMEM));
    attr_set = true;
  }
  LISA_CUDA(cudaMemsetAsync(grid_bar, 0, sizeof(uint32_t), s));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)sm_count_current());
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = TRAIN_SMEM;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (!g.grad_part) return Status::invalid("guide: no partial-gradient slots");  // one per SM
  if (src_kind == SRC_RAW)
    LISA_CUDA(cudaLaunchKernelEx(&cfg, k_guide_train_rounds<SRC_RAW>, g.w_bf16, g.master, g.adam_m, g.adam_v, src,
                                 chunk, rounds, lr, g.grad_part, g.loss_part, grid_bar, g.loss_last, g.d_step, g.status,
                                 sample_count));
  else
    LISA_CUDA(cudaLaunchKernelEx(&cfg, k_guide_train_rounds<SRC_GEOM>, g.w_bf16, g.master, g.adam_m, g.adam_v, src,
                                 chunk, rounds, lr, g.grad_part, g.loss_part, grid_bar, g.loss_last, g.d_step, g.status,
                                 sample_count));
  return Status();
}

// g.grads and g.loss = the sums of the last training launch's partials.
Status guide_launch_reduce(GuideNet& g, cudaStream_t s) {
  k_guide_reduce<<<(NPARAM + 255) / 256, 256, 0, s>>>(g.grad_part, g.loss_part, g.nparts, g.grads, g.loss);
  LISA_CUDA(cudaGetLastError());
  return Status();
}

Status guide_launch_adam(GuideNet& g, float lr, cudaStream_t s) {
  k_guide_adam<<<(4 * NPARAM + 255) / 256, 256, 0, s>>>(g.master, g.adam_m, g.adam_v, g.grad_part, g.loss_part, g.nparts,
                                                    g.loss_last, lr, g.d_step, g.status, g.w_bf16);
  LISA_CUDA(cudaGetLastError());
  return Status();
}

Status guide_check_status(GuideNet& g, cudaStream_t s) {
  uint32_t st = 0;
  LISA_CUDA(cudaMemcpyAsync(&st, g.status, sizeof(st), cudaMemcpyDeviceToHost, s));
  LISA_CUDA(cudaStreamSynchronize(s));
  if (st & (ST_GUIDE_NONFINITE << 1)) return Status(LISA_ERR_DEVICE, "guide: tensor-core wait timed out");
  if (st & ST_GUIDE_NONFINITE) return Status(LISA_ERR_DEVICE, "guide: non-finite gradient");
  return Status();
}

// Guided mode: one network per scene (sharing one set of partial-gradient
// slots), the kept training records, the emitter samples (physically based
// estimator) and the training batch.
Status guide_renderer_init(Renderer& r) {
  // samples per Adam step: a multiple of 128; 0 = one 128-sample tile per SM
  const uint32_t chunk = r.opts.guide_train_batch ? std::max<uint32_t>(128, (r.opts.guide_train_batch + 127) / 128 * 128)
                                                  : 128u * (uint32_t)sm_count_current();
  r.guide_chunk = chunk;
  // Adam steps of a wave: guide_steps_per_wave per 4 Mi paths, at least one
  r.guide_max_steps = std::max<uint32_t>(
      1u, (uint32_t)(((uint64_t)r.capacity * r.opts.guide_steps_per_wave + (1ull << 22) - 1) >> 22));
  const uint32_t B = chunk * r.guide_max_steps;
  r.guide_batch_cap = B;
  if (!(r.opts.guide_bsdf_fraction >= 0.0f && r.opts.guide_bsdf_fraction <= 1.0f))
    return Status::invalid("guide_bsdf_fraction must be in [0, 1]");
  r.guides.clear();
  const uint32_t slots = (uint32_t)sm_count_current();
  LISA_TRY(r.arena.alloc((void**)&r.guide_grad_part, sizeof(float) * (size_t)NPARAM * slots, "guide gradients"));
  LISA_TRY(r.arena.alloc((void**)&r.guide_loss_part, sizeof(float) * slots, "guide losses"));
  for (size_t s = 0; s < r.scenes.size(); ++s) {
    std::unique_ptr<GuideNet> g;
    LISA_TRY(guide_create(r.opts.seed * 7919u + (uint32_t)s, g, r.stream, false));
    g->grad_part = r.guide_grad_part;
    g->loss_part = r.guide_loss_part;
    r.scenes[s].guide = (int)s;
    r.guides.push_back(std::move(g));
  }
  LISA_TRY(guided_infer_setup());
  // kept training records: four times the batch, so that enough of them
  // carry radiance
  r.rec_cap = 4u * B;
  LISA_TRY(r.arena.alloc((void**)&r.rec_list, sizeof(float4) * 5ull * r.rec_cap, "guide records"));
  if (r.opts.estimator == LISA_ESTIMATOR_PHYSICAL)
    LISA_TRY(r.arena.alloc((void**)&r.nee_light, sizeof(float4) * 2ull * r.capacity, "emitter samples"));
  LISA_TRY(r.arena.alloc((void**)&r.guide_batch, sizeof(float4) * 4ull * B, "guide batch"));
  LISA_TRY(r.arena.alloc((void**)&r.guide_grid_bar, sizeof(uint32_t), "guide training barrier"));
  return Status();
}

}  // namespace lisa

// ===========================================================================
using namespace lisa;

static int gret(const Status& s) {
  set_last_error(s);
  return s.code;
}

// A barrier that nothing completes, waited on with an iteration limit: the
// time-out path of the tensor-core kernels (status bit, early exit) taken
// on purpose, with no fault and no unbounded wait.
static_assert((ST_GUIDE_NONFINITE << 1) == LISA_STATUS_WAIT_TIMEOUT, "time-out status bit");

__global__ void k_wait_timeout(uint32_t limit, uint32_t* status) {
  __shared__ uint64_t mbar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&mbar, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && !tc::mbar_wait(&mbar, 0, limit)) atomicOr(status, ST_GUIDE_NONFINITE << 1);
}

extern "C" {

int lisa_selftest_wait_timeout(uint32_t limit, uint32_t* status_word) {
  if (!status_word || limit == 0) return gret(Status::invalid("null argument or zero limit"));
  uint32_t* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(uint32_t));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return gret(Status(LISA_ERR_UNSUPPORTED, std::string("no CUDA device: ") + cudaGetErrorString(e)));
  }
  e = cudaMemset(d, 0, sizeof(uint32_t));
  if (e == cudaSuccess) {
    k_wait_timeout<<<1, 32>>>(limit, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(status_word, d, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return gret(Status::cuda(e, "wait self-test"));
  return gret(Status());
}

int lisa_guide_create(uint32_t seed, lisa_guide** out) {
  try {
    if (!out) return gret(Status::invalid("null argument"));
    std::unique_ptr<lisa_guide> g(new lisa_guide());
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return gret(Status(LISA_ERR_UNSUPPORTED, std::string("no CUDA device: ") + cudaGetErrorString(e)));
    }
    Status s = guide_create(seed, g->net, g->stream, true);
    if (!s.ok()) return gret(s);
    *out = g.release();
    return gret(Status());
  } catch (const std::exception& e) {
    return gret(Status(LISA_ERR_INVALID, e.what()));
  }
}

void lisa_guide_destroy(lisa_guide* g) {
  if (!g) return;
  if (g->stream) cudaStreamSynchronize(g->stream);
  g->net.reset();
  if (g->stream && g->owns_stream) cudaStreamDestroy(g->stream);
  delete g;
}

int lisa_guide_get_params(lisa_guide* g, float* params) {
  if (!g || !params) return gret(Status::invalid("null argument"));
  cudaError_t e = cudaMemcpyAsync(params, g->get().master, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  return gret(e == cudaSuccess ? Status() : Status::cuda(e, "get params"));
}

int lisa_guide_set_params(lisa_guide* g, const float* params) {
  if (!g || !params) return gret(Status::invalid("null argument"));
  cudaError_t e = cudaMemcpyAsync(g->get().master, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, g->stream);
  if (e != cudaSuccess) return gret(Status::cuda(e, "set params"));
  Status s = guide_pack(g->get(), g->stream);
  if (s.ok()) {
    e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) s = Status::cuda(e, "set params");
  }
  return gret(s);
}

int lisa_guide_forward(lisa_guide* g, const float* features, uint32_t n, float* out) {
  if (!g || (n && (!features || !out))) return gret(Status::invalid("null argument"));
  if (n == 0) return gret(Status());
  float *d_x = nullptr, *d_o = nullptr;
  auto run = [&]() -> Status {
    LISA_CUDA(cudaMalloc(&d_x, sizeof(float) * 64ull * n));
    LISA_CUDA(cudaMalloc(&d_o, sizeof(float) * 40ull * n));
    LISA_CUDA(cudaMemcpyAsync(d_x, features, sizeof(float) * 64ull * n, cudaMemcpyHostToDevice, g->stream));
    GuideSrc src;
    std::memset(&src, 0, sizeof(src));
    src.raw = d_x;
    src.n = n;
    LISA_TRY(guide_launch_infer(g->get(), src, SRC_RAW, d_o, n, g->stream));
    LISA_CUDA(cudaMemcpyAsync(out, d_o, sizeof(float) * 40ull * n, cudaMemcpyDeviceToHost, g->stream));
    return guide_check_status(g->get(), g->stream);
  };
  Status s = run();
  if (d_x) cudaFree(d_x);
  if (d_o) cudaFree(d_o);
  return gret(s);
}

int lisa_guide_train_step(lisa_guide* g, const float* features, const float* dirs, const float* weights, uint32_t n,
                          float lr, float* loss, float* grads) {
  if (!g || (n && (!features || !dirs || !weights))) return gret(Status::invalid("null argument"));
  if (n == 0) return gret(Status::invalid("empty batch"));
  float *d_x = nullptr, *d_d = nullptr, *d_w = nullptr;
  auto run = [&]() -> Status {
    LISA_CUDA(cudaMalloc(&d_x, sizeof(float) * 64ull * n));
    LISA_CUDA(cudaMalloc(&d_d, sizeof(float) * 3ull * n));
    LISA_CUDA(cudaMalloc(&d_w, sizeof(float) * n));
    LISA_CUDA(cudaMemcpyAsync(d_x, features, sizeof(float) * 64ull * n, cudaMemcpyHostToDevice, g->stream));
    LISA_CUDA(cudaMemcpyAsync(d_d, dirs, sizeof(float) * 3ull * n, cudaMemcpyHostToDevice, g->stream));
    LISA_CUDA(cudaMemcpyAsync(d_w, weights, sizeof(float) * n, cudaMemcpyHostToDevice, g->stream));
    GuideSrc src;
    std::memset(&src, 0, sizeof(src));
    src.raw = d_x;
    src.dirs = d_d;
    src.weights = d_w;
    src.n = n;
    LISA_TRY(guide_launch_train(g->get(), src, 1.0f / (float)n, n, g->stream, lr > 0.0f));
    LISA_TRY(guide_launch_reduce(g->get(), g->stream));
    if (loss) LISA_CUDA(cudaMemcpyAsync(loss, g->get().loss, sizeof(float), cudaMemcpyDeviceToHost, g->stream));
    if (grads)
      LISA_CUDA(cudaMemcpyAsync(grads, g->get().grads, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, g->stream));
    LISA_TRY(guide_check_status(g->get(), g->stream));
    if (lr > 0.0f) {
      LISA_TRY(guide_launch_adam(g->get(), lr, g->stream));
      LISA_TRY(guide_check_status(g->get(), g->stream));
    }
    return Status();
  };
  Status s = run();
  if (d_x) cudaFree(d_x);
  if (d_d) cudaFree(d_d);
  if (d_w) cudaFree(d_w);
  return gret(s);
}

int lisa_guide_train_steps(lisa_guide* g, const float* features, const float* dirs, const float* weights, uint32_t n,
                           uint32_t chunk, uint32_t steps, float lr, float* loss) {
  if (!g || !features || !dirs || !weights) return gret(Status::invalid("null argument"));
  if (n == 0 || steps == 0) return gret(Status::invalid("empty batch"));
  if (chunk == 0 || chunk % 128) return gret(Status::invalid("chunk must be a positive multiple of 128"));
  if (!(lr > 0.0f)) return gret(Status::invalid("lr must be positive"));
  float *d_x = nullptr, *d_d = nullptr, *d_w = nullptr;
  uint32_t* d_bar = nullptr;
  auto run = [&]() -> Status {
    LISA_CUDA(cudaMalloc(&d_x, sizeof(float) * 64ull * n));
    LISA_CUDA(cudaMalloc(&d_d, sizeof(float) * 3ull * n));
    LISA_CUDA(cudaMalloc(&d_w, sizeof(float) * n));
    LISA_CUDA(cudaMalloc(&d_bar, sizeof(uint32_t)));
    LISA_CUDA(cudaMemcpyAsync(d_x, features, sizeof(float) * 64ull * n, cudaMemcpyHostToDevice, g->stream));
    LISA_CUDA(cudaMemcpyAsync(d_d, dirs, sizeof(float) * 3ull * n, cudaMemcpyHostToDevice, g->stream));
    LISA_CUDA(cudaMemcpyAsync(d_w, weights, sizeof(float) * n, cudaMemcpyHostToDevice, g->stream));
    GuideSrc src;
    std::memset(&src, 0, sizeof(src));
    src.raw = d_x;
    src.dirs = d_d;
    src.weights = d_w;
    src.n = n;
    LISA_TRY(guide_launch_train_rounds(g->get(), src, SRC_RAW, chunk, steps, lr, d_bar, g->stream, nullptr));
    if (loss) LISA_CUDA(cudaMemcpyAsync(loss, g->get().loss_last, sizeof(float), cudaMemcpyDeviceToHost, g->stream));
    LISA_TRY(guide_check_status(g->get(), g->stream));
    return Status();
  };
  Status s = run();
  if (d_x) cudaFree(d_x);
  if (d_d) cudaFree(d_d);
  if (d_w) cudaFree(d_w);
  if (d_bar) cudaFree(d_bar);
  return gret(s);
}

}  // extern "C"

// Inference core of the guide network, shared by the standalone inference
// kernel (guide.cu) and the renderer's fused inference + guided-bounce
// kernels (wavefront.cu): parameter and packed-weight layouts, feature
// loading, and infer_tiles(), which runs the five layers on the tensor cores
// tile by tile and hands each thread its sample's 40 outputs.
//
// Network: 64 encoded inputs -> 4 x (64, ReLU) -> 40 outputs = 8 vMF lobes
// (guide_mix.cuh).  A CTA of 128 threads processes tiles of 128 samples:
// thread t owns row t of every activation tile and TMEM lane t of the
// accumulator.  One thread issues tcgen05.mma (M = 128, K = 16 per
// instruction), commits to an mbarrier and waits (bounded; a time-out sets a
// status bit), the block meets at a barrier, then every thread reads its
// accumulator row with tcgen05.ld.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "guide.cuh"
#include "guide_mix.cuh"
#include "lisa_device.cuh"
#include "tcgen05.cuh"

namespace lisa {

// ---- parameter layout (FP32 master) ------------------------------------------
constexpr int P_W = 0;                    // W1..W4: 4 x 64 x 64, then W5: 40 x 64
constexpr int P_W5 = 4 * 64 * 64;
constexpr int P_B = P_W5 + 40 * 64;       // b1..b4: 4 x 64, then b5: 40
constexpr int P_B5 = P_B + 4 * 64;
constexpr int NPARAM = P_B5 + 40;
static_assert(NPARAM == LISA_GUIDE_NUM_PARAMS, "parameter count");

// ---- packed BF16 weights: rows of 128 B, pre-swizzled in 8-row groups ------------
constexpr int R_FWD = 0;        // W1..W4 forward: 4 x 64 rows (row = output)
constexpr int R_W5 = 256;       // W5 forward: 48 rows (40 used)
constexpr int R_T = 304;        // W2^T..W5^T: 4 x 64 rows (row = input, K = output)
constexpr int R_TOTAL = 560;
constexpr int PACK_BYTES = R_TOTAL * 128;
constexpr int FWD_BYTES = R_T * 128;  // what inference needs

__device__ __forceinline__ uint16_t f2bf(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float bf2f(uint16_t h) { return __bfloat162float(__ushort_as_bfloat16(h)); }

template <int SRC>
__device__ __forceinline__ void load_features(const GuideSrc& s, uint32_t i, float* f) {
  if (SRC == SRC_RAW) {
    const float4* r = (const float4*)(s.raw + 64ull * i);
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const float4 x = __ldg(r + c);
      f[4 * c] = x.x;
      f[4 * c + 1] = x.y;
      f[4 * c + 2] = x.z;
      f[4 * c + 3] = x.w;
    }
  } else if (SRC == SRC_GEOM) {
    const float4 a = s.geom[4ull * i], b = s.geom[4ull * i + 1], c = s.geom[4ull * i + 2], d = s.geom[4ull * i + 3];
    guide::encode(s.bmin, s.bmax, a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, d.y, f);
  } else {
    const float4 a = s.nee_a[i], b = s.nee_b[i], c = s.nee_c[i];
    // view direction: towards where the ray came from
    const float il = rsqrtf(fmaxf(c.x * c.x + c.y * c.y + c.z * c.z, 1e-30f));
    // the emitter flag (path state, a random access) only where it is a feature
    const bool flag = !s.no_flag && __float_as_int(s.ps_att[__float_as_uint(a.w)].w) >= 0;
    guide::encode(s.bmin, s.bmax, a.x, a.y, a.z, b.x, b.y, b.z, -c.x * il, -c.y * il, -c.z * il, flag ? 1.0f : 0.0f,
                  f);
  }
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Brings sample i's feature rows into L2 ahead of load_features (emitter
// queue only: the other sources stream in order).
template <int SRC>
__device__ __forceinline__ void prefetch_features(const GuideSrc& s, uint32_t i) {
  if (SRC == SRC_NEE) {
    prefetch_l2(s.nee_a + i);
    prefetch_l2(s.nee_b + i);
    prefetch_l2(s.nee_c + i);
  }
}

// Writes 64 values as BF16 (round to nearest even) into row `row` of a
// swizzled tile, two values per conversion.
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);  // .x (low half) = lo
  return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ void store_row_bf16(uint8_t* tile, int row, const float* v) {
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    uint4 q;
    q.x = pack_bf16x2(v[8 * c + 0], v[8 * c + 1]);
    q.y = pack_bf16x2(v[8 * c + 2], v[8 * c + 3]);
    q.z = pack_bf16x2(v[8 * c + 4], v[8 * c + 5]);
    q.w = pack_bf16x2(v[8 * c + 6], v[8 * c + 7]);
    *(uint4*)(tile + row * 128 + ((c ^ (row & 7)) << 4)) = q;
  }
}

// relu(lo + blo), relu(hi + bhi) as BF16x2: one packed FP32 add (add.rn.f32x2,
// the same rounding as two scalar adds) and one converting ReLU
// (cvt.rn.relu.bf16x2.f32: negative sums become +0).
__device__ __forceinline__ uint32_t bias_relu_bf16x2(float lo, float hi, float blo, float bhi) {
  const float2 s = __fadd2_rn(make_float2(lo, hi), make_float2(blo, bhi));
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(s.y), "f"(s.x));  // first source -> upper half
  return d;
}

// Row `row` of a hidden layer's output tile: relu(acc + bias) as BF16 (the
// bias is 64 FP32 values in shared memory, 16-byte aligned).
__device__ __forceinline__ void store_row_bias_relu(uint8_t* tile, int row, const float* acc, const float* bias) {
  const float4* b4 = reinterpret_cast<const float4*>(bias);
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const float4 u = b4[2 * c], w = b4[2 * c + 1];
    uint4 q;
    q.x = bias_relu_bf16x2(acc[8 * c + 0], acc[8 * c + 1], u.x, u.y);
    q.y = bias_relu_bf16x2(acc[8 * c + 2], acc[8 * c + 3], u.z, u.w);
    q.z = bias_relu_bf16x2(acc[8 * c + 4], acc[8 * c + 5], w.x, w.y);
    q.w = bias_relu_bf16x2(acc[8 * c + 6], acc[8 * c + 7], w.z, w.w);
    *(uint4*)(tile + row * 128 + ((c ^ (row & 7)) << 4)) = q;
  }
}

// D = A(128 x 64) * B(N x 64)^T: four K = 16 steps, then a commit.
__device__ __forceinline__ void issue_layer(uint32_t d_tmem, const uint8_t* a, const uint8_t* b, uint32_t N,
                                            uint64_t* mbar) {
  const uint32_t sa = tc::smem_u32(a), sb = tc::smem_u32(b);
  const uint32_t idesc = tc::idesc_bf16_f32(128, N);
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) tc::mma_bf16(d_tmem, tc::sw128_desc(sa + 32 * k), tc::sw128_desc(sb + 32 * k), idesc, k);
  tc::mma_commit(mbar);
}

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return (uint8_t*)(((uintptr_t)p + 1023) & ~(uintptr_t)1023);
}

// ---------------------------------------------------------------------------------
// inference: the five layers, tile by tile

// + 1024 for the manual 1024-byte alignment, + 2 KB of slack after the last
// operand tile.  A CTA is two warpgroups sharing one copy of the weights,
// each with its own tile, accumulator (64 TMEM columns), mbarrier and MMA
// thread; two CTAs share an SM (2 x 74.8 KB of shared memory, 2 x 128 TMEM
// columns, <= 128 registers a thread): 16 warps and four tile pipelines per
// SM.
constexpr int INFER_SMEM = FWD_BYTES + 2 * 16384 + 1024 + 2048;
constexpr int INFER_THREADS = 256;
constexpr int INFER_BLOCKS_PER_SM = 2;

// Runs the network on samples [src.first, n) and calls epi(i, valid, o) in
// the 128 threads of a warpgroup for their samples i of each tile (valid =
// i < n; o = the 40 outputs, bias included); epi may use warp-collective
// operations.  pre(i) runs for each valid sample when its features are
// loaded, five layers before its epi: a place to start the epilogue's
// memory traffic (prefetches).  Needs INFER_SMEM bytes of dynamic shared
// memory and INFER_THREADS threads.
//
// The two warpgroups of a CTA run independent pipelines (named barriers,
// one per warpgroup): thread 0 of a warpgroup issues its tile's layer
// (tcgen05.mma, M = 128, K = 16 per instruction), every thread of the
// warpgroup waits for it on the warpgroup's mbarrier, reads its
// accumulator row with tcgen05.ld and writes the next layer's input row
// (bias, ReLU, BF16) over the tile in shared memory, and the warpgroup
// meets at its barrier before the next issue.  While one
// warpgroup runs an epilogue, the tensor core runs the other warpgroups'
// layers.
template <int SRC, class Pre, class Epi>
__device__ __forceinline__ void infer_tiles(const uint16_t* __restrict__ pack, const float* __restrict__ master,
                                            const GuideSrc& src, uint32_t* status, Pre&& pre, Epi&& epi) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* w = smem;
  __shared__ uint64_t mbar[2];  // one per warpgroup
  __shared__ uint64_t mbar_w;   // the packed weights' bulk copy
  __shared__ uint32_t tmem_base;
  __shared__ int failed[2];     // per warpgroup
  __shared__ int weights_failed;
  __shared__ __align__(16) float s_bias[4 * 64 + 48];
  const int tid = threadIdx.x, warp = tid >> 5, wg = tid >> 7, t = tid & 127;
  // samples [src.first, n)
  const uint32_t n = max(src.count ? min(*(volatile const uint32_t*)src.count, src.n) : src.n, src.first);
  const uint32_t ntiles = (n - src.first + 127) / 128;
  if (2 * blockIdx.x >= ntiles) return;
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::mbar_init(&mbar_w, 1);
    tc::fence_mbar_init();
    tc::bulk_load(w, pack, FWD_BYTES, &mbar_w);  // weights by TMA while the rest is set up
    failed[0] = failed[1] = 0;
    weights_failed = 0;
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base, 128);
  for (int k = tid; k < 4 * 64 + 48; k += INFER_THREADS) s_bias[k] = k < 4 * 64 + 40 ? __ldg(master + P_B + k) : 0.0f;
  if (tid == 0 && !tc::mbar_wait(&mbar_w, 0)) {
    atomicOr(status, ST_GUIDE_NONFINITE << 1);
    failed[0] = failed[1] = 1;
    weights_failed = 1;
  }
  tc::fence_smem_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base + 64u * wg;  // this warpgroup's accumulator columns
  const uint32_t lane_addr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  uint8_t* const act = smem + FWD_BYTES + 16384 * wg;
  const uint32_t bar_id = 1u + wg;
  auto wg_sync = [&]() { asm volatile("bar.sync %0, 128;" ::"r"(bar_id) : "memory"); };
  // parity of the warpgroup's next MMA completion; thread 0 of the
  // warpgroup: whether a committed MMA has not been waited for, and its parity
  uint32_t phase = 0, busy_parity = 0;
  bool busy = false;
  auto issue = [&](int l) {
    issue_layer(tmem, act, w + (l < 4 ? (R_FWD + 64 * l) : R_W5) * 128, l < 4 ? 64u : 48u, &mbar[wg]);
    busy = true;
    busy_parity = phase;
  };
  for (uint32_t tile = 2 * blockIdx.x + wg; tile < ntiles; tile += 2 * gridDim.x) {
    if (failed[wg]) break;  // read after a warpgroup barrier: uniform over the warpgroup
    const uint32_t i = src.first + tile * 128 + t;
    {
      float f[64];
      if (i < n) {
        load_features<SRC>(src, i, f);
        pre(i);
      } else {
#pragma unroll
        for (int q = 0; q < 64; ++q) f[q] = 0.0f;
      }
      store_row_bf16(act, t, f);
    }
    // the warpgroup's next tile's feature rows, while this one runs
    const uint32_t j = src.first + (tile + 2 * gridDim.x) * 128 + t;
    if (j < n) prefetch_features<SRC>(src, j);
    tc::fence_smem_async();
    tc::fence_before_sync();
    wg_sync();
    tc::fence_after_sync();
    if (t == 0) issue(0);
#pragma unroll 1
    for (int l = 0; l < 5; ++l) {
      // every thread waits for the layer's MMA itself (bounded; no barrier
      // to hand the completion on); a time-out reaches the others through
      // failed[wg] at the warpgroup's next barrier
      if (tc::mbar_wait(&mbar[wg], phase)) {
        if (t == 0) busy = false;
      } else {
        atomicOr(status, ST_GUIDE_NONFINITE << 1);
        failed[wg] = 1;
      }
      phase ^= 1u;
      tc::fence_after_sync();
      float acc[64];
      if (l < 4) {
        tc::tmem_ld16x<4>(lane_addr, acc);
        store_row_bias_relu(act, t, acc, s_bias + 64 * l);  // H_l over H_{l-1}
        tc::fence_smem_async();
        tc::fence_before_sync();
        wg_sync();
        tc::fence_after_sync();
        if (failed[wg]) break;
        if (t == 0) issue(l + 1);
      } else {
        tc::tmem_ld16x<3>(lane_addr, acc);
#pragma unroll
        for (int q = 0; q < 40; ++q) acc[q] += s_bias[4 * 64 + q];
        epi(i, i < n, acc);
      }
    }
    // the next tile rewrites the tile and the accumulator
    tc::fence_before_sync();
    wg_sync();
    tc::fence_after_sync();
  }
  // after a time-out, give an MMA still in flight a bounded chance to finish
  // before its TMEM is freed
  if (t == 0 && busy) tc::mbar_wait(&mbar[wg], busy_parity, 1u << 20);
  if (tid == 0 && weights_failed) tc::mbar_wait(&mbar_w, 0, 1u << 20);  // a late weight copy
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem_base, 128);
}

}  // namespace lisa

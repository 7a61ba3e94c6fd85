// GPU BVH construction for the triangle soup.
//
// Replaces the closed optixAccelBuild call of the reference
// (src/LiSA/src/optix_wrapper.cc:92-145).  Pipeline, all on the device:
//   1. per-triangle AABB and centroid, scene and centroid bounds
//   2. 30-bit Morton code of each centroid
//   3. stable LSD radix sort of (code, triangle) pairs: 4 passes of 8 bits,
//      tile histograms -> exclusive scan -> stable scatter (warp match-any
//      ranking), written here without a sort library
//   4. binary radix tree over the sorted codes (Karras, "Maximizing
//      Parallelism in the Construction of BVHs, Octrees, and k-d Trees",
//      HPG 2012), equal codes ordered by index
//   5. bottom-up AABBs with one atomic arrival counter per node
//   6. collapse into 8-wide nodes, level by level: each node adopts up to 8
//      descendants by repeatedly opening the child of largest surface area
//      (subtrees of <= 3 triangles become leaves), then stores its child
//      boxes quantised to 8 bits against a per-axis power-of-two grid,
//      rounded outward (compressed layout in the style of Ylitie, Karras,
//      Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed
//      Wide BVHs", HPG 2017).  Leaf triangles are copied into leaf order.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "lisa_device.cuh"
#include "lisa_internal.h"

namespace lisa {
namespace {

constexpr uint32_t LEAF_BIT = 0x80000000u;

__device__ __forceinline__ int f2ord(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__host__ __device__ __forceinline__ float ord2f(int i) {
#ifdef __CUDA_ARCH__
  return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
#else
  const int j = i >= 0 ? i : i ^ 0x7fffffff;
  float f;
  std::memcpy(&f, &j, 4);
  return f;
#endif
}

// bounds[0..2] = min scene xyz, [3..5] = max scene xyz, [6..8] min centroid,
// [9..11] max centroid, as order-preserving ints.
__global__ void k_prim_bounds(const float* __restrict__ v, uint32_t n, float4* __restrict__ lo,
                              float4* __restrict__ hi, int* bounds) {
  float mn[6], mx[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    mn[k] = __int_as_float(0x7f800000);
    mx[k] = -__int_as_float(0x7f800000);
  }
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* t = v + 9ull * i;
    float a[3], b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      a[k] = fminf(fminf(t[k], t[3 + k]), t[6 + k]);
      b[k] = fmaxf(fmaxf(t[k], t[3 + k]), t[6 + k]);
      const float c = 0.5f * (a[k] + b[k]);
      mn[k] = fminf(mn[k], a[k]);
      mx[k] = fmaxf(mx[k], b[k]);
      mn[3 + k] = fminf(mn[3 + k], c);
      mx[3 + k] = fmaxf(mx[3 + k], c);
    }
    lo[i] = make_float4(a[0], a[1], a[2], 0.0f);
    hi[i] = make_float4(b[0], b[1], b[2], 0.0f);
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
      mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      atomicMin(&bounds[k], f2ord(mn[k]));
      atomicMax(&bounds[3 + k], f2ord(mx[k]));
      atomicMin(&bounds[6 + k], f2ord(mn[3 + k]));
      atomicMax(&bounds[9 + k], f2ord(mx[3 + k]));
    }
  }
}

__device__ __forceinline__ uint32_t expand10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

#ifndef LISA_MORTON_SIZE_BITS
#define LISA_MORTON_SIZE_BITS 2
#endif

// Sort key: the triangle's size class above the 30-bit Morton code of its
// centroid (extended Morton codes, Vinkler, Bittner, Havran, HPG 2017), so
// large triangles -- walls, quads -- separate from the small ones near the
// root instead of overlapping every deep subtree.  Class 0 holds triangles
// whose box diagonal exceeds 1/8 of the scene's, then 1/64, 1/512.
__global__ void k_morton(const float4* __restrict__ lo, const float4* __restrict__ hi, uint32_t n,
                         const int* __restrict__ bounds, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = lo[i], b = hi[i];
  const float c[3] = {0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z)};
  uint32_t q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float cmin = ord2f(bounds[6 + k]), cmax = ord2f(bounds[9 + k]);
    const float ext = cmax - cmin;
    float u = ext > 0.0f ? (c[k] - cmin) / ext : 0.5f;
    u = fminf(fmaxf(u, 0.0f), 1.0f);
    q[k] = min((uint32_t)(u * 1024.0f), 1023u);
  }
  uint32_t key = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
#if LISA_MORTON_SIZE_BITS > 0
  float s2 = 0.0f, t2 = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float se = ord2f(bounds[3 + k]) - ord2f(bounds[k]);
    s2 += se * se;
  }
  t2 = (b.x - a.x) * (b.x - a.x) + (b.y - a.y) * (b.y - a.y) + (b.z - a.z) * (b.z - a.z);
  // diagonal ratio thresholds 1/8, 1/64, 1/512 on squared lengths
  const uint32_t cls = t2 * 64.0f > s2 ? 0u : (t2 * 4096.0f > s2 ? 1u : (t2 * 262144.0f > s2 ? 2u : 3u));
  key |= cls << 30;
#endif
  keys[i] = key;
  vals[i] = i;
}

// ---- radix sort -----------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;

__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                       uint32_t* __restrict__ hist, uint32_t num_tiles) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
  for (int k = 0; k < RS_ROUNDS; ++k) {
    const uint64_t idx = base + (uint64_t)k * RS_THREADS + threadIdx.x;
    if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * num_tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                          uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                          uint32_t n, int shift, const uint32_t* __restrict__ offs,
                                                          uint32_t num_tiles) {
  __shared__ uint32_t s_base[256];
  __shared__ uint32_t s_run[256];
  __shared__ uint32_t s_wc[RS_THREADS / 32][256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  s_base[tid] = offs[(uint64_t)tid * num_tiles + blockIdx.x];
  s_run[tid] = 0;
  const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
  const uint32_t lt = (1u << lane) - 1u;
  for (int r = 0; r < RS_ROUNDS; ++r) {
#pragma unroll
    for (int w = 0; w < RS_THREADS / 32; ++w) s_wc[w][tid] = 0;
    __syncthreads();
    const uint64_t idx = base + (uint64_t)r * RS_THREADS + tid;
    const bool valid = idx < n;
    const uint32_t key = valid ? kin[idx] : 0u;
    const uint32_t d = valid ? ((key >> shift) & 255u) : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & lt);
    if (valid && rank == 0) s_wc[warp][d] = __popc(peers);
    __syncthreads();
    uint32_t run = s_run[tid];
#pragma unroll
    for (int w = 0; w < RS_THREADS / 32; ++w) {
      const uint32_t c = s_wc[w][tid];
      s_wc[w][tid] = run;
      run += c;
    }
    s_run[tid] = run;
    __syncthreads();
    if (valid) {
      const uint32_t pos = s_base[d] + s_wc[warp][d] + rank;
      kout[pos] = key;
      vout[pos] = vin[idx];
    }
    __syncthreads();
  }
}

// ---- exclusive scan (in place) --------------------------------------------
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* total) {
  __shared__ uint32_t ws[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t s = lane < nw ? ws[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) ws[lane] = s;
  }
  __syncthreads();
  const uint32_t before = (warp > 0 ? ws[warp - 1] : 0u) + x - v;
  if (total) *total = ws[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_blocks(uint32_t* data, uint64_t m, uint32_t* sums) {
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK + (uint64_t)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    v[k] = (base + k < m) ? data[base + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t run = block_exclusive(s, &total);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    if (base + k < m) data[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_single(uint32_t* sums, uint32_t nb) {
  uint32_t carry = 0;
  for (uint32_t c0 = 0; c0 < nb; c0 += SCAN_CHUNK) {
    const uint32_t base = c0 + threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
      v[k] = (base + k < nb) ? sums[base + k] : 0u;
      s += v[k];
    }
    uint32_t total;
    uint32_t run = carry + block_exclusive(s, &total);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
      if (base + k < nb) sums[base + k] = run;
      run += v[k];
    }
    carry += total;
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_add(uint32_t* data, uint64_t m, const uint32_t* sums) {
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK + (uint64_t)threadIdx.x * SCAN_ITEMS;
  const uint32_t add = sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k)
    if (base + k < m) data[base + k] += add;
}

// ---- Karras radix tree ------------------------------------------------------
__device__ __forceinline__ int kdelta(const uint32_t* keys, int64_t n, int64_t i, int64_t j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = keys[i], b = keys[j];
  if (a == b) return 32 + __clz((uint32_t)(i ^ j));
  return __clz(a ^ b);
}

__global__ void k_karras(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ left,
                         uint32_t* __restrict__ right, uint32_t* __restrict__ first, uint32_t* __restrict__ last,
                         uint32_t* __restrict__ parent_int, uint32_t* __restrict__ parent_leaf) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)n - 1) return;
  const int64_t N = n;
  const int d = (kdelta(keys, N, i, i + 1) - kdelta(keys, N, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = kdelta(keys, N, i, i - d);
  int64_t lmax = 2;
  while (kdelta(keys, N, i, i + lmax * d) > dmin) lmax <<= 1;
  int64_t l = 0;
  for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
    if (kdelta(keys, N, i, i + (l + t) * d) > dmin) l += t;
  const int64_t j = i + l * d;
  const int dnode = kdelta(keys, N, i, j);
  int64_t s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (kdelta(keys, N, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int64_t gamma = i + s * d + (d < 0 ? -1 : 0);
  const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
  const uint32_t lc = (lo == gamma) ? (LEAF_BIT | (uint32_t)gamma) : (uint32_t)gamma;
  const uint32_t rc = (hi == gamma + 1) ? (LEAF_BIT | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
  left[i] = lc;
  right[i] = rc;
  first[i] = (uint32_t)lo;
  last[i] = (uint32_t)hi;
  if (lc & LEAF_BIT) parent_leaf[lc & ~LEAF_BIT] = (uint32_t)i; else parent_int[lc] = (uint32_t)i;
  if (rc & LEAF_BIT) parent_leaf[rc & ~LEAF_BIT] = (uint32_t)i; else parent_int[rc] = (uint32_t)i;
  if (i == 0) parent_int[0] = 0xffffffffu;
}

__device__ __forceinline__ void node_box(uint32_t c, const uint32_t* vals, const float4* plo, const float4* phi,
                                         const float4* ilo, const float4* ihi, float4& lo, float4& hi) {
  if (c & LEAF_BIT) {
    const uint32_t p = vals[c & ~LEAF_BIT];
    lo = plo[p];
    hi = phi[p];
  } else {
    lo = __ldcg(ilo + c);
    hi = __ldcg(ihi + c);
  }
}

__global__ void k_bottom_up(uint32_t n, const uint32_t* __restrict__ vals, const float4* __restrict__ plo,
                            const float4* __restrict__ phi, const uint32_t* __restrict__ parent_leaf,
                            const uint32_t* __restrict__ parent_int, const uint32_t* __restrict__ left,
                            const uint32_t* __restrict__ right, float4* ilo, float4* ihi, uint32_t* flags) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || n < 2) return;
  uint32_t p = parent_leaf[i];
  while (p != 0xffffffffu) {
    __threadfence();
    if (atomicAdd(&flags[p], 1u) == 0u) return;
    __threadfence();
    float4 a0, a1, b0, b1;
    node_box(left[p], vals, plo, phi, ilo, ihi, a0, a1);
    node_box(right[p], vals, plo, phi, ilo, ihi, b0, b1);
    __stcg(ilo + p, make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), 0.0f));
    __stcg(ihi + p, make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), 0.0f));
    p = parent_int[p];
  }
}

// ---- SAH refinement: treelet restructuring -----------------------------------
//
// One bottom-up pass over the binary LBVH (Karras & Aila, "Fast Parallel
// Construction of High-Quality Bounding Volume Hierarchies", HPG 2013): the
// thread that completes a node computes its box, primitive count and SAH
// cost, then takes the treelet of up to 7 leaves under it (grown by opening
// the treelet leaf of largest area) and rebuilds the treelet's internal
// nodes in the topology of least SAH cost, found by dynamic programming over
// the leaf subsets.  The treelet's leaves and everything below them stay as
// they are; every node keeps a box equal to the union of its children's.
// Node counts and costs overwrite the Karras ranges (first -> count,
// last -> cost bits), which the collapse no longer needs.

constexpr float SAH_CI = 1.2f;  // cost of a node visit relative to a triangle test
constexpr float SAH_CT = 1.0f;
constexpr int TL = 7;           // treelet leaves
// Subtrees of fewer primitives keep their LBVH topology (the 8-wide
// collapse flattens them).  Measured on the 1.31 M-triangle icosphere box
// and the 4.48 M-triangle sphere soup: 64 against 16 builds in 3.8 instead
// of 5.1 ms and 6.9 instead of 10.7 ms, with the same Mrays/s on the first
// and 0.4 % fewer on the second.
#ifndef LISA_TREELET_MIN_PRIMS
#define LISA_TREELET_MIN_PRIMS 64
#endif
constexpr uint32_t TREELET_MIN_PRIMS = LISA_TREELET_MIN_PRIMS;

__device__ __forceinline__ float4 box_min(float4 a, float4 b) {
  return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.0f);
}
__device__ __forceinline__ float4 box_max(float4 a, float4 b) {
  return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), 0.0f);
}
__device__ __forceinline__ float box_half_area(float4 lo, float4 hi) {
  const float x = hi.x - lo.x, y = hi.y - lo.y, z = hi.z - lo.z;
  return x * y + y * z + z * x;
}

struct SahTree {
  uint32_t n;
  const uint32_t* vals;
  const float4* plo;
  const float4* phi;
  uint32_t* parent_leaf;
  uint32_t* parent_int;
  uint32_t* left;
  uint32_t* right;
  float4* ilo;
  float4* ihi;
  uint32_t* count;  // per internal node: primitives below
  float* cost;      // per internal node: SAH cost of its subtree
  uint32_t* flags;
};

// box, count and cost of a child (leaf or internal node, already complete)
__device__ __forceinline__ void sah_child(const SahTree& t, uint32_t c, float4& lo, float4& hi, uint32_t& cnt,
                                          float& cost) {
  if (c & LEAF_BIT) {
    const uint32_t q = t.vals[c & ~LEAF_BIT];
    lo = t.plo[q];
    hi = t.phi[q];
    cnt = 1;
    cost = SAH_CT * box_half_area(lo, hi);
  } else {
    lo = __ldcg(t.ilo + c);
    hi = __ldcg(t.ihi + c);
    cnt = __ldcg(t.count + c);
    cost = __ldcg(t.cost + c);
  }
}

// Per-warp shared state of one treelet's restructuring.
struct TreeletSmem {
  float opt[1 << TL];        // best SAH cost of each subset of the treelet's leaves
  uint8_t split[1 << TL];    // its best partition (one side)
  float4 llo[TL], lhi[TL];   // leaf boxes
  float lcost[TL];
  uint32_t lcnt[TL];
  uint32_t leaf[TL], inner[TL - 2];
  int nl;
};

// Treelet restructuring (Karras and Aila, HPG 2013) of the subtree at
// `root`, by one warp: lane 0 grows the treelet (the largest-area leaf is
// expanded until TL leaves), the lanes then share the dynamic programme over
// the subsets of its leaves, one subset size per round (a subset's
// partitions only use smaller subsets), and lane 0 rebuilds the subtree when
// the best topology is cheaper.  Every subset's cost is computed by the same
// operations in the same order as a serial loop would.  All 32 lanes call
// it with the same root.
__device__ void treelet_optimize_warp(const SahTree& t, uint32_t root, TreeletSmem& s) {
  const int lane = threadIdx.x & 31;
  __syncwarp();  // the root's box, count and cost, just written by its lane, are visible to lane 0
  if (lane == 0) {
    int nl = 2, ni = 0;
    s.leaf[0] = __ldcg(t.left + root);
    s.leaf[1] = __ldcg(t.right + root);
    sah_child(t, s.leaf[0], s.llo[0], s.lhi[0], s.lcnt[0], s.lcost[0]);
    sah_child(t, s.leaf[1], s.llo[1], s.lhi[1], s.lcnt[1], s.lcost[1]);
    while (nl < TL) {
      int best = -1;
      float ba = -1.0f;
      for (int k = 0; k < nl; ++k) {
        if (s.leaf[k] & LEAF_BIT) continue;
        const float a = box_half_area(s.llo[k], s.lhi[k]);
        if (a > ba) {
          ba = a;
          best = k;
        }
      }
      if (best < 0) break;
      const uint32_t c = s.leaf[best];
      s.inner[ni++] = c;
      s.leaf[best] = __ldcg(t.left + c);
      s.leaf[nl] = __ldcg(t.right + c);
      sah_child(t, s.leaf[best], s.llo[best], s.lhi[best], s.lcnt[best], s.lcost[best]);
      sah_child(t, s.leaf[nl], s.llo[nl], s.lhi[nl], s.lcnt[nl], s.lcost[nl]);
      ++nl;
    }
    s.nl = nl;
  }
  __syncwarp();
  const int nl = s.nl;
  if (nl < 3) return;  // two leaves have one topology
  const uint32_t full = (1u << nl) - 1u;
  for (uint32_t sset = lane + 1; sset <= full; sset += 32)
    if ((sset & (sset - 1u)) == 0u) {
      s.opt[sset] = s.lcost[__ffs(sset) - 1];
      s.split[sset] = 0;
    }
  __syncwarp();
  for (int size = 2; size <= nl; ++size) {
    for (uint32_t sset = lane + 1; sset <= full; sset += 32) {
      if (__popc(sset) != size) continue;
      float4 lo = make_float4(3.4e38f, 3.4e38f, 3.4e38f, 0.0f), hi = make_float4(-3.4e38f, -3.4e38f, -3.4e38f, 0.0f);
      for (int k = 0; k < nl; ++k)
        if (sset & (1u << k)) {
          lo = box_min(lo, s.llo[k]);
          hi = box_max(hi, s.lhi[k]);
        }
      const uint32_t low = sset & (0u - sset), rest = sset ^ low;
      float best = s.opt[low] + s.opt[rest];
      uint32_t bp = low;
      // partitions (P, S \ P) with the lowest member in P, each once:
      // P = low + a nonempty proper subset of the rest
      for (uint32_t q = (rest - 1u) & rest; q; q = (q - 1u) & rest) {
        const uint32_t pset = q | low;
        const float c = s.opt[pset] + s.opt[sset ^ pset];
        if (c < best) {
          best = c;
          bp = pset;
        }
      }
      s.opt[sset] = SAH_CI * box_half_area(lo, hi) + best;
      s.split[sset] = (uint8_t)bp;
    }
    __syncwarp();
  }
  if (lane == 0 && s.opt[full] < __ldcg(t.cost + root) * (1.0f - 1e-6f)) {
    // rebuild: the root keeps its id, the other internal subsets reuse inner[]
    uint32_t st_set[TL], st_node[TL];
    int sp = 0, next = 0;
    st_set[sp] = full;
    st_node[sp++] = root;
    while (sp) {
      --sp;
      const uint32_t sset = st_set[sp], node = st_node[sp];
      const uint32_t part[2] = {s.split[sset], sset ^ (uint32_t)s.split[sset]};
      uint32_t ch[2];
      for (int h = 0; h < 2; ++h) {
        if ((part[h] & (part[h] - 1u)) == 0u) {
          ch[h] = s.leaf[__ffs(part[h]) - 1];
        } else {
          ch[h] = s.inner[next++];
          st_set[sp] = part[h];
          st_node[sp++] = ch[h];
        }
        if (ch[h] & LEAF_BIT) __stcg(t.parent_leaf + (ch[h] & ~LEAF_BIT), node);
        else __stcg(t.parent_int + ch[h], node);
      }
      __stcg(t.left + node, ch[0]);
      __stcg(t.right + node, ch[1]);
      float4 lo = make_float4(3.4e38f, 3.4e38f, 3.4e38f, 0.0f), hi = make_float4(-3.4e38f, -3.4e38f, -3.4e38f, 0.0f);
      uint32_t cnt = 0;
      for (int k = 0; k < nl; ++k)
        if (sset & (1u << k)) {
          lo = box_min(lo, s.llo[k]);
          hi = box_max(hi, s.lhi[k]);
          cnt += s.lcnt[k];
        }
      __stcg(t.ilo + node, lo);
      __stcg(t.ihi + node, hi);
      __stcg(t.count + node, cnt);
      __stcg(t.cost + node, s.opt[sset]);
    }
  }
  __syncwarp();
}

// Bottom-up pass: boxes, primitive counts and SAH costs of the internal
// nodes, one leaf per lane climbing to the root; the second lane to reach a
// node finishes it (the first stops there).  Nodes with enough primitives
// below are restructured by the whole warp, one lane's node at a time, so
// the restructuring's dynamic programme runs on 32 lanes.
constexpr int SAH_THREADS = 256;

__global__ void __launch_bounds__(SAH_THREADS) k_bottom_up_sah(SahTree t, int refine) {
  __shared__ TreeletSmem tls[SAH_THREADS / 32];
  TreeletSmem& tl = tls[threadIdx.x >> 5];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t p = (i < t.n && t.n >= 2) ? t.parent_leaf[i] : 0xffffffffu;
  bool active = p != 0xffffffffu;
  while (__any_sync(0xffffffffu, active)) {
    bool want = false;
    if (active) {
      __threadfence();
      if (atomicAdd(&t.flags[p], 1u) == 0u) {
        active = false;
      } else {
        __threadfence();
        float4 a0, a1, b0, b1;
        uint32_t ca, cb;
        float sa, sb;
        sah_child(t, __ldcg(t.left + p), a0, a1, ca, sa);
        sah_child(t, __ldcg(t.right + p), b0, b1, cb, sb);
        const float4 lo = box_min(a0, b0), hi = box_max(a1, b1);
        __stcg(t.ilo + p, lo);
        __stcg(t.ihi + p, hi);
        __stcg(t.count + p, ca + cb);
        __stcg(t.cost + p, SAH_CI * box_half_area(lo, hi) + sa + sb);
        want = refine && ca + cb >= TREELET_MIN_PRIMS;
      }
    }
    uint32_t m = __ballot_sync(0xffffffffu, want);
    while (m) {
      const int owner = __ffs(m) - 1;
      m &= m - 1;
      treelet_optimize_warp(t, __shfl_sync(0xffffffffu, p, owner), tl);
    }
    if (active) {
      p = __ldcg(t.parent_int + p);
      active = p != 0xffffffffu;
    }
  }
}

// ---- collapse to 8-wide compressed nodes -------------------------------------
struct CollapseArgs {
  uint32_t n;
  const uint32_t* vals;
  const float4* plo;
  const float4* phi;
  const float4* ilo;
  const float4* ihi;
  const uint32_t* left;
  const uint32_t* right;
  const uint32_t* count;  // primitives below each internal node
  const float* verts;
  const int32_t* mats;  // material per triangle, or null
  uint4* nodes;
  float4* tris;
  uint32_t* counters;  // [0] nodes, [1] tri slots
};

__device__ __forceinline__ uint32_t sub_count(const CollapseArgs& a, uint32_t c) {
  return (c & LEAF_BIT) ? 1u : a.count[c];
}
__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
  const float x = hi.x - lo.x, y = hi.y - lo.y, z = hi.z - lo.z;
  return x * y + y * z + z * x;
}

// Smallest e with 255 * 2^e >= ext, clamped to the normal float range.
__device__ int grid_exponent(double ext) {
  if (!(ext > 0.0)) return -126;
  int e;
  frexp(ext / 255.0, &e);  // ext/255 = m * 2^e, m in [0.5, 1)
  while (ldexp(255.0, e - 1) >= ext && e > -126) --e;
  while (ldexp(255.0, e) < ext) ++e;
  return max(-126, min(127, e));
}

// Collapse levels run as a fixed sequence of launches with no host round
// trip: level l reads its work count from levels[l] (written by level l-1)
// and appends the next level's work, counting it in levels[l+1]; a level
// with no work returns at once.
constexpr int COLLAPSE_LAUNCHES = 24;

__global__ void k_collapse_init(uint32_t* counters, uint32_t* levels, uint2* work0, uint2 root) {
  counters[0] = 1u;  // node 0 is the root
  counters[1] = 0u;
  for (int l = 0; l <= COLLAPSE_LAUNCHES + 1; ++l) levels[l] = l == 0 ? 1u : 0u;
  work0[0] = root;
}

__device__ void collapse_one(const CollapseArgs& a, uint2 item, uint2* __restrict__ next, uint32_t* next_count);

__global__ void k_collapse(CollapseArgs a, const uint2* __restrict__ work, const uint32_t* __restrict__ nwork_p,
                           uint2* __restrict__ next, uint32_t* next_count) {
  const uint32_t nwork = *nwork_p;
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nwork; w += gridDim.x * blockDim.x)
    collapse_one(a, work[w], next, next_count);
}

__device__ void collapse_one(const CollapseArgs& a, uint2 item, uint2* __restrict__ next, uint32_t* next_count) {
  const uint32_t dst = item.x, src = item.y;
  uint32_t cand[8];
  int nc;
  if (!(src & LEAF_BIT) && sub_count(a, src) > 3u) {
    cand[0] = a.left[src];
    cand[1] = a.right[src];
    nc = 2;
  } else {
    cand[0] = src;
    nc = 1;
  }
  float4 clo[8], chi[8];
  for (int k = 0; k < nc; ++k) node_box(cand[k], a.vals, a.plo, a.phi, a.ilo, a.ihi, clo[k], chi[k]);
  while (nc < 8) {
    int best = -1;
    float best_area = -1.0f;
    for (int k = 0; k < nc; ++k) {
      if ((cand[k] & LEAF_BIT) || sub_count(a, cand[k]) <= 3u) continue;
      const float ar = half_area(clo[k], chi[k]);
      if (ar > best_area) {
        best_area = ar;
        best = k;
      }
    }
    if (best < 0) break;
    const uint32_t c = cand[best];
    cand[best] = a.left[c];
    cand[nc] = a.right[c];
    node_box(cand[best], a.vals, a.plo, a.phi, a.ilo, a.ihi, clo[best], chi[best]);
    node_box(cand[nc], a.vals, a.plo, a.phi, a.ilo, a.ihi, clo[nc], chi[nc]);
    ++nc;
  }
  uint32_t num_int = 0, num_tri = 0;
  for (int k = 0; k < nc; ++k) {
    const uint32_t cnt = sub_count(a, cand[k]);
    if (cnt > 3u) ++num_int; else num_tri += cnt;
  }
  const uint32_t child_base = num_int ? atomicAdd(&a.counters[0], num_int) : 0u;
  const uint32_t tri_base = num_tri ? atomicAdd(&a.counters[1], num_tri) : 0u;
  // node frame
  float4 nlo = clo[0], nhi = chi[0];
  for (int k = 1; k < nc; ++k) {
    nlo.x = fminf(nlo.x, clo[k].x);
    nlo.y = fminf(nlo.y, clo[k].y);
    nlo.z = fminf(nlo.z, clo[k].z);
    nhi.x = fmaxf(nhi.x, chi[k].x);
    nhi.y = fmaxf(nhi.y, chi[k].y);
    nhi.z = fmaxf(nhi.z, chi[k].z);
  }
  const float p[3] = {nlo.x, nlo.y, nlo.z};
  const float ph[3] = {nhi.x, nhi.y, nhi.z};
  int e[3];
  for (int ax = 0; ax < 3; ++ax) e[ax] = grid_exponent((double)ph[ax] - (double)p[ax]);
  uint8_t qlo[3][8], qhi[3][8], meta[8];
  uint32_t imask = 0, rank = 0, toff = 0;
  for (int k = 0; k < 8; ++k) {
    meta[k] = 0;
    for (int ax = 0; ax < 3; ++ax) {
      qlo[ax][k] = 0;
      qhi[ax][k] = 0;
    }
  }
  for (int k = 0; k < nc; ++k) {
    const float lo3[3] = {clo[k].x, clo[k].y, clo[k].z};
    const float hi3[3] = {chi[k].x, chi[k].y, chi[k].z};
    for (int ax = 0; ax < 3; ++ax) {
      const double sc = ldexp(1.0, e[ax]);
      double ql = floor(((double)lo3[ax] - (double)p[ax]) / sc);
      double qh = ceil(((double)hi3[ax] - (double)p[ax]) / sc);
      ql = fmin(fmax(ql, 0.0), 255.0);
      qh = fmin(fmax(qh, 0.0), 255.0);
      while (ql > 0.0 && (double)p[ax] + ql * sc > (double)lo3[ax]) ql -= 1.0;
      while (qh < 255.0 && (double)p[ax] + qh * sc < (double)hi3[ax]) qh += 1.0;
      qlo[ax][k] = (uint8_t)ql;
      qhi[ax][k] = (uint8_t)qh;
    }
    const uint32_t cnt = sub_count(a, cand[k]);
    if (cnt > 3u) {
      imask |= 1u << k;
      meta[k] = (uint8_t)rank;
      const uint32_t slot = atomicAdd(next_count, 1u);
      next[slot] = make_uint2(child_base + rank, cand[k]);
      ++rank;
    } else {
      meta[k] = (uint8_t)((cnt << 5) | toff);
      // the (at most 3) primitives below, left to right
      uint32_t leaves[3], st[4];
      int nlv = 0, sp = 0;
      st[sp++] = cand[k];
      while (sp) {
        const uint32_t c = st[--sp];
        if (c & LEAF_BIT) {
          leaves[nlv++] = c & ~LEAF_BIT;
        } else {
          st[sp++] = a.right[c];
          st[sp++] = a.left[c];
        }
      }
      for (uint32_t q = 0; q < cnt; ++q) {
        const uint32_t prim = a.vals[leaves[q]];
        const float* t = a.verts + 9ull * prim;
        float4* o = a.tris + 3ull * (tri_base + toff + q);
        o[0] = make_float4(t[0], t[1], t[2], __int_as_float((int)prim));
        o[1] = make_float4(t[3], t[4], t[5], __int_as_float(a.mats ? a.mats[prim] : 0));
        o[2] = make_float4(t[6], t[7], t[8], 0.0f);
      }
      toff += cnt;
    }
  }
  auto pack4 = [](const uint8_t* b) {
    return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
  };
  uint4* np = a.nodes + 5ull * dst;
  np[0] = make_uint4(__float_as_uint(p[0]), __float_as_uint(p[1]), __float_as_uint(p[2]),
                     (uint32_t)(e[0] + 127) | ((uint32_t)(e[1] + 127) << 8) | ((uint32_t)(e[2] + 127) << 16) |
                         (imask << 24));
  np[1] = make_uint4(child_base, tri_base, pack4(meta), pack4(meta + 4));
  np[2] = make_uint4(pack4(qlo[0]), pack4(qlo[0] + 4), pack4(qlo[1]), pack4(qlo[1] + 4));
  np[3] = make_uint4(pack4(qlo[2]), pack4(qlo[2] + 4), pack4(qhi[0]), pack4(qhi[0] + 4));
  np[4] = make_uint4(pack4(qhi[1]), pack4(qhi[1] + 4), pack4(qhi[2]), pack4(qhi[2] + 4));
}

inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

}  // namespace

Status device_exclusive_scan(uint32_t* d, uint64_t m, uint32_t* tmp, cudaStream_t s) {
  const uint32_t nb = cdiv(m, SCAN_CHUNK);
  k_scan_blocks<<<nb, SCAN_THREADS, 0, s>>>(d, m, tmp);
  k_scan_single<<<1, SCAN_THREADS, 0, s>>>(tmp, nb);
  k_scan_add<<<nb, SCAN_THREADS, 0, s>>>(d, m, tmp);
  LISA_CUDA(cudaGetLastError());
  return Status();
}

// Sorts (keys, vals) by the low 32 bits of keys; stable.  Result in keys/vals.
Status device_radix_sort(uint32_t* keys, uint32_t* vals, uint32_t* keys2, uint32_t* vals2, uint32_t n,
                         uint32_t* hist, uint32_t* scan_tmp, int bits, cudaStream_t s) {
  const uint32_t tiles = cdiv(n, RS_TILE);
  uint32_t *ki = keys, *vi = vals, *ko = keys2, *vo = vals2;
  for (int shift = 0; shift < bits; shift += 8) {
    k_rs_hist<<<tiles, RS_THREADS, 0, s>>>(ki, n, shift, hist, tiles);
    LISA_TRY(device_exclusive_scan(hist, 256ull * tiles, scan_tmp, s));
    k_rs_scatter<<<tiles, RS_THREADS, 0, s>>>(ki, vi, ko, vo, n, shift, hist, tiles);
    LISA_CUDA(cudaGetLastError());
    std::swap(ki, ko);
    std::swap(vi, vo);
  }
  if (ki != keys) {
    LISA_CUDA(cudaMemcpyAsync(keys, ki, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    LISA_CUDA(cudaMemcpyAsync(vals, vi, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
  }
  return Status();
}

namespace {
template <class T>
Status take(ScratchSource& src, T** p, uint64_t count, const char* what) {
  void* q = nullptr;
  LISA_TRY(src.get(&q, std::max<uint64_t>(count * sizeof(T), 16), what));
  *p = (T*)q;
  return Status();
}
inline uint64_t al256(uint64_t b) { return (std::max<uint64_t>(b, 16) + 255) & ~255ull; }
}  // namespace

size_t bvh_temp_bytes(uint32_t n) {
  const uint64_t tiles = cdiv(n, RS_TILE);
  uint64_t b = 0;
  b += 4 * al256(16ull * n);                                   // plo phi ilo ihi
  b += 4 * al256(4ull * n);                                    // keys vals keys2 vals2
  b += al256(4ull * 256 * tiles) + al256(4ull * (cdiv(256ull * tiles, SCAN_CHUNK) + 16));
  b += 7 * al256(4ull * n);                                    // tree links and flags
  b += al256(16) + al256(48);                                  // counters, bounds
  b += al256(4ull * 32);                                       // collapse level counts
  b += 2 * al256(8ull * (n + 1));                              // collapse work lists
  return (size_t)b;
}

size_t bvh_output_bytes(uint32_t n) { return (size_t)(al256(80ull * (n + 1)) + al256(48ull * n)); }

Status build_bvh(const float* d_verts, uint32_t n, cudaStream_t s, ScratchSource& tmp, ScratchSource& out,
                 uint4** d_nodes, float4** d_tris, BvhBuildResult* info, const int32_t* d_mat, bool refine) {
  auto t0 = std::chrono::steady_clock::now();
  if (n == 0) {
    *d_nodes = nullptr;
    *d_tris = nullptr;
    info->num_nodes = 0;
    info->num_tri_slots = 0;
    info->depth = 0;
    for (int k = 0; k < 3; ++k) info->bmin[k] = info->bmax[k] = 0.0f;
    return Status();
  }
  float4 *plo, *phi, *ilo, *ihi;
  uint32_t *keys, *vals, *keys2, *vals2, *hist, *scan_tmp;
  uint32_t *left, *right, *first, *last, *par_int, *par_leaf, *flags, *counters;
  int* bounds;
  uint2 *work0, *work1;
  const uint32_t tiles = cdiv(n, RS_TILE);
  const char* w = "bvh build scratch";
  LISA_TRY(take(tmp, &plo, n, w));
  LISA_TRY(take(tmp, &phi, n, w));
  LISA_TRY(take(tmp, &ilo, n, w));
  LISA_TRY(take(tmp, &ihi, n, w));
  LISA_TRY(take(tmp, &keys, n, w));
  LISA_TRY(take(tmp, &vals, n, w));
  LISA_TRY(take(tmp, &keys2, n, w));
  LISA_TRY(take(tmp, &vals2, n, w));
  LISA_TRY(take(tmp, &hist, 256ull * tiles, w));
  LISA_TRY(take(tmp, &scan_tmp, cdiv(256ull * tiles, SCAN_CHUNK) + 16, w));
  LISA_TRY(take(tmp, &left, n, w));
  LISA_TRY(take(tmp, &right, n, w));
  LISA_TRY(take(tmp, &first, n, w));
  LISA_TRY(take(tmp, &last, n, w));
  LISA_TRY(take(tmp, &par_int, n, w));
  LISA_TRY(take(tmp, &par_leaf, n, w));
  LISA_TRY(take(tmp, &flags, n, w));
  LISA_TRY(take(tmp, &counters, 4, w));
  uint32_t* levels = nullptr;
  LISA_TRY(take(tmp, &levels, 32, w));
  LISA_TRY(take(tmp, &bounds, 12, w));
  LISA_TRY(take(tmp, &work0, n + 1, w));
  LISA_TRY(take(tmp, &work1, n + 1, w));

  int hb[12];
  for (int k = 0; k < 3; ++k) {
    hb[k] = 0x7fffffff;
    hb[3 + k] = (int)0x80000000;
    hb[6 + k] = 0x7fffffff;
    hb[9 + k] = (int)0x80000000;
  }
  LISA_CUDA(cudaMemcpyAsync(bounds, hb, sizeof(hb), cudaMemcpyHostToDevice, s));
  const int nblk = (int)std::min<uint32_t>(cdiv(n, 256), 4096);
  k_prim_bounds<<<nblk, 256, 0, s>>>(d_verts, n, plo, phi, bounds);
  k_morton<<<cdiv(n, 256), 256, 0, s>>>(plo, phi, n, bounds, keys, vals);
  LISA_CUDA(cudaGetLastError());
  LISA_TRY(device_radix_sort(keys, vals, keys2, vals2, n, hist, scan_tmp, 32, s));
  if (n > 1) {
    k_karras<<<cdiv(n - 1, 256), 256, 0, s>>>(keys, n, left, right, first, last, par_int, par_leaf);
    LISA_CUDA(cudaMemsetAsync(flags, 0, sizeof(uint32_t) * n, s));
    // boxes, counts and SAH costs bottom up, with treelet restructuring
    // unless refine is off; first/last become count/cost
    const SahTree st{n, vals, plo, phi, par_leaf, par_int, left, right, ilo, ihi, first, (float*)last, flags};
    k_bottom_up_sah<<<cdiv(n, SAH_THREADS), SAH_THREADS, 0, s>>>(st, refine ? 1 : 0);
    LISA_CUDA(cudaGetLastError());
  }
  // outputs
  uint4* nodes = nullptr;
  float4* tris = nullptr;
  LISA_TRY(take(out, &nodes, 5ull * (n + 1), "bvh nodes"));
  LISA_TRY(take(out, &tris, 3ull * n, "bvh triangles"));
  const uint2 root = make_uint2(0u, n > 1 ? 0u : LEAF_BIT);
  k_collapse_init<<<1, 1, 0, s>>>(counters, levels, work0, root);
  LISA_CUDA(cudaGetLastError());
  CollapseArgs a{n, vals, plo, phi, ilo, ihi, left, right, first, d_verts, d_mat, nodes, tris, counters};
  // a level holds at most one work item per 8-wide node, fewer than n/2
  int dev = 0, sms = 0;
  LISA_CUDA(cudaGetDevice(&dev));
  LISA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t cgrid = std::max<uint32_t>(1u, std::min<uint32_t>(cdiv(n / 2 + 1, 64), (uint32_t)sms * 16u));
  for (int l = 0; l < COLLAPSE_LAUNCHES; ++l)
    k_collapse<<<cgrid, 64, 0, s>>>(a, (l & 1) ? work1 : work0, levels + l, (l & 1) ? work0 : work1,
                                    levels + l + 1);
  LISA_CUDA(cudaGetLastError());
  uint32_t hc[2];
  uint32_t hl[COLLAPSE_LAUNCHES + 1];
  LISA_CUDA(cudaMemcpyAsync(hc, counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
  LISA_CUDA(cudaMemcpyAsync(hl, levels, sizeof(hl), cudaMemcpyDeviceToHost, s));
  LISA_CUDA(cudaMemcpyAsync(hb, bounds, sizeof(hb), cudaMemcpyDeviceToHost, s));
  LISA_CUDA(cudaStreamSynchronize(s));
  uint32_t depth = 0;
  while (depth < (uint32_t)COLLAPSE_LAUNCHES && hl[depth] > 0) ++depth;
  if (depth == (uint32_t)COLLAPSE_LAUNCHES && hl[COLLAPSE_LAUNCHES] > 0) {
    // a tree deeper than the fixed launches: the remaining levels, one host
    // round trip each (slot C holds the level's count, slot C+1 the next's)
    uint32_t* cur = levels + COLLAPSE_LAUNCHES;
    uint32_t nwork = hl[COLLAPSE_LAUNCHES];
    uint2 *wi = (COLLAPSE_LAUNCHES & 1) ? work1 : work0, *wo = (COLLAPSE_LAUNCHES & 1) ? work0 : work1;
    while (nwork > 0) {
      LISA_CUDA(cudaMemsetAsync(cur + 1, 0, sizeof(uint32_t), s));
      k_collapse<<<cdiv(nwork, 64), 64, 0, s>>>(a, wi, cur, wo, cur + 1);
      LISA_CUDA(cudaGetLastError());
      LISA_CUDA(cudaMemcpyAsync(cur, cur + 1, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
      LISA_CUDA(cudaMemcpyAsync(&nwork, cur + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      LISA_CUDA(cudaStreamSynchronize(s));
      std::swap(wi, wo);
      ++depth;
    }
    LISA_CUDA(cudaMemcpyAsync(hc, counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
    LISA_CUDA(cudaStreamSynchronize(s));
  }
  if (hc[1] != n) return Status(LISA_ERR_DEVICE, "bvh build: leaf triangle count mismatch");
  info->num_nodes = hc[0];
  info->num_tri_slots = hc[1];
  info->depth = depth;
  for (int k = 0; k < 3; ++k) {
    info->bmin[k] = ord2f(hb[k]);
    info->bmax[k] = ord2f(hb[3 + k]);
  }
  *d_nodes = nodes;
  *d_tris = tris;
  info->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return Status();
}

}  // namespace lisa

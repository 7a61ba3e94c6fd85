// Device-side data layout and the closest-hit traversal.
//
// HBM layout of one scene (all arrays 16-byte aligned, read with 128-bit
// loads):
//   nodes  : 8-wide compressed BVH nodes, 80 B = 5 x uint4 each
//              uint4 0: origin p.xyz (f32) | exponents ex,ey,ez (u8), imask (u8)
//              uint4 1: child_base | tri_base | meta[0..3] | meta[4..7]
//              uint4 2: qlo.x[8] | qlo.y[8]
//              uint4 3: qlo.z[8] | qhi.x[8]
//              uint4 4: qhi.y[8] | qhi.z[8]
//            child box = p + 2^(e-127) * q (per axis); imask bit i marks an
//            internal child at node child_base + meta[i]; a leaf child has
//            meta[i] = count<<5 | offset (count 1..3 triangles at
//            tri_base + offset); meta 0 and imask 0 = empty slot.
//   tris   : 3 x float4 per leaf triangle slot, in leaf order:
//            (v0.xyz, original triangle id as int bits),
//            (v1, its material if that is an emitter, else -1), (v2, 0)
//   prims  : 5 x float4 per original triangle (shading record):
//            (v0, n0.x) (v1, n0.y) (v2, n0.z) (n1, n2.x) (n2.y, n2.z, mat, 0)
//   mats   : DevMaterial, 48 B each
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "device_math.cuh"

namespace lisa {

enum : int { MAT_OPAQUE = 0, MAT_DIELECTRIC = 1, MAT_EMIT = 2 };

struct DevMaterial {
  float albedo[3];
  float roughness;
  float emission[3];
  float ior;
  int cls;
  float alpha;
  float light_pdf;  // physically based estimator: area pdf (luminance / total) of its emitters
  int pad;
};
static_assert(sizeof(DevMaterial) == 48, "DevMaterial layout");

constexpr float RAY_TMIN = 1e-4f;  // shader.cu:114,202
constexpr float RAY_TMAX = 1e16f;  // shader.cu:115,202
constexpr int NEE_TRIES = 30;      // shader.cu:199
// emissive triangles from which the emitter search uses their own BVH (with
// fewer, the bounds test of the emitter search is as selective)
constexpr uint32_t EMIT_BVH_MIN_TRIS = 32;
constexpr int TRAV_STACK = 64;

enum StatusBits : uint32_t {
  ST_STACK_OVERFLOW = 1u,
  ST_QUEUE_OVERFLOW = 2u,
  ST_BAD_WAVE = 4u,
  ST_GUIDE_NONFINITE = 8u,
  // 16: a bounded tensor-core wait ran out (LISA_STATUS_WAIT_TIMEOUT)
  ST_BOUNDS = 32u,  // bounds-checked builds: a BVH or triangle index out of range
};

// Bounds-checked builds (-DLISA_BOUNDS, a stand-in for a memory checker):
// node and triangle indices read from the BVH and the queue slots that
// appends reserve are checked before use; a bad one sets a status bit and
// the access is skipped.  Queue sizes are bounded by construction (one entry
// per path and depth), so in ordinary builds the checks compile away.

struct SceneDev {
  const uint4* nodes;
  const float4* tris;
  const float4* prims;
  const DevMaterial* mats;
  uint32_t num_prims;
  uint32_t num_nodes;
  uint32_t num_mats;
  float extent;  // bounding-box diagonal
  uint32_t width, height;
  uint32_t num_bounces;
  uint32_t pad0;
  float eye[3], U[3], V[3], W[3];
  float lens_radius;  // 0 = pinhole
  float focal_distance;
  float unitU[3], unitV[3], unitW[3];
  float bmin[3], bmax[3];  // scene bounds (guide encoding)
  // accumulation, one entry per pixel
  float4* acc_sum;   // Kahan sum (xyz)
  float4* acc_comp;  // Kahan compensation (xyz)
  double* acc_sq;    // 3 doubles: sum of squares
  double* acc_sum64; // 3 doubles: FP64 sum (accum_fp64 only, else null)
  uint32_t* pix_rng; // reference per-pixel stream state (LISA_RNG_PER_PIXEL)
  int32_t guide;     // guide slot of this scene (-1 = none)
  int32_t pad1;
  // physically based estimator: emitters, 4 float4 each --
  // (v0.xyz, area pdf) (e1 = v1-v0, material bits) (e2 = v2-v0, 0) (unit normal, 0)
  // -- and the CDF over area x luminance that picks them
  const float4* emit;
  const float* emit_cdf;
  uint32_t num_emit;
  uint32_t has_emit_box;     // the scene has emissive triangles, all inside emit_lo..emit_hi
  float emit_lo[3], emit_hi[3];
  // BVH over the emissive triangles alone (0 nodes = none): the emitter
  // search asks it first whether a ray meets an emitter at all
  const uint4* enodes;
  const float4* etris;
  uint32_t num_enodes;
  uint32_t num_etris;
};

// One group of a wave: `nplanes` consecutive sample planes of pixels
// [pix0, pix0+npix) of one scene.  slot = slot0 + m*npix + (p - pix0).
struct WaveGroup {
  uint32_t scene;
  uint32_t pix0, npix;
  uint32_t sample0, nplanes;
  uint32_t slot0;
  uint32_t acc0;  // prefix of npix over the wave's groups (accumulate index)
  uint32_t pad;
};
constexpr int MAX_GROUPS = 128;
struct WaveDesc {
  uint32_t num_groups;
  uint32_t paths;
  uint32_t acc_items;  // sum of npix
  uint32_t rng_mode;
  uint32_t seed;
  uint32_t pad[3];
  WaveGroup groups[MAX_GROUPS];
};

enum { HEAD_TRACE = 0, HEAD_SHADE = 1, HEAD_NEE = 2, HEAD_GUIDE = 3 };
struct WaveCtrl {
  uint32_t qcount[2];
  uint32_t nee_count;
  uint32_t train_count;
  uint32_t head[4];
  uint32_t status;
  uint32_t guided_count;  // guided vertices of the current wave
  uint32_t rec_count;     // training records kept in the current wave
  float drop_prob;        // probability of not keeping a guided vertex's record (0 = keep all)
  unsigned long long rays_primary;
  unsigned long long rays_bounce;
  unsigned long long rays_shadow;
  unsigned long long node_visits[2];  // [0] closest-hit stage, [1] emitter search
  unsigned long long tri_tests[2];
  unsigned long long nee_total;
  unsigned long long shadow_walked;   // emitter-search rays that walked the BVH
  unsigned long long infer_rows;      // emitter-queue entries the guide's inference ran on
  unsigned long long train_samples;   // samples of the guide's training steps
};

// ---------------------------------------------------------------------------
// Watertight ray/triangle test (Woop, Benthin, Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2013), evaluated with one rounding per
// operation and no FMA so the host oracle reproduces every hit bit for bit.

struct RayPre {
  float ox, oy, oz;
  float ix, iy, iz;  // 1/d per axis
  uint32_t k;        // shear axes: kx | ky << 2 | kz << 4
  float Sx, Sy, Sz;
  float slack;  // absolute slack on the best distance, in t units
  __device__ __forceinline__ int kx() const { return (int)(k & 3u); }
  __device__ __forceinline__ int ky() const { return (int)((k >> 2) & 3u); }
  __device__ __forceinline__ int kz() const { return (int)((k >> 4) & 3u); }
};

__device__ __forceinline__ float sel3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ RayPre ray_prepare(V3 o, V3 d, float extent) {
  RayPre r;
  r.ox = o.x;
  r.oy = o.y;
  r.oz = o.z;
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  int kx = kz + 1;
  if (kx == 3) kx = 0;
  int ky = kx + 1;
  if (ky == 3) ky = 0;
  const float dz = sel3(d.x, d.y, d.z, kz);
  if (dz < 0.0f) {
    const int t = kx;
    kx = ky;
    ky = t;
  }
  r.k = (uint32_t)kx | ((uint32_t)ky << 2) | ((uint32_t)kz << 4);
  r.Sx = fdiv(sel3(d.x, d.y, d.z, kx), dz);
  r.Sy = fdiv(sel3(d.x, d.y, d.z, ky), dz);
  // __frcp_rn is the correctly rounded 1/x, the same value as 1.0f/x: the
  // shear's 1/dz, and the node-culling reciprocal of that (dominant) axis
  r.Sz = __frcp_rn(dz);
  // The other two axes' reciprocals serve node culling only; __fdividef is
  // within 2 ulp there, which the slab padding covers (see trav_node).  A
  // zero or vanishing component takes a huge finite reciprocal of its sign
  // instead of infinity: the node test then keeps that axis's slab (the
  // ray's constant coordinate against the padded box) instead of turning it
  // into NaN and dropping it, which made such rays visit most of the tree.
  const float qx = ax > 1e-30f ? __fdividef(1.0f, d.x) : copysignf(1e30f, d.x);
  const float qy = ay > 1e-30f ? __fdividef(1.0f, d.y) : copysignf(1e30f, d.y);
  const float qz = az > 1e-30f ? __fdividef(1.0f, d.z) : copysignf(1e30f, d.z);
  r.ix = kz == 0 ? r.Sz : qx;
  r.iy = kz == 1 ? r.Sz : qy;
  r.iz = kz == 2 ? r.Sz : qz;
  // 2^-18 * extent / |d|max; a margin, so an approximate quotient will do
  r.slack = __fdividef(3.814697265625e-6f * extent, fmaxf(ax, fmaxf(ay, az)));
  return r;
}

// Returns t of the hit (or +inf).  prim_t < tbest test is the caller's.
__device__ __forceinline__ float intersect_tri(const RayPre& r, float4 a4, float4 b4, float4 c4, float tmin) {
  // translate to the ray origin
  const float ax_ = fsub(a4.x, r.ox), ay_ = fsub(a4.y, r.oy), az_ = fsub(a4.z, r.oz);
  const float bx_ = fsub(b4.x, r.ox), by_ = fsub(b4.y, r.oy), bz_ = fsub(b4.z, r.oz);
  const float cx_ = fsub(c4.x, r.ox), cy_ = fsub(c4.y, r.oy), cz_ = fsub(c4.z, r.oz);
  const int kx = r.kx(), ky = r.ky(), kz = r.kz();
  const float Akx = sel3(ax_, ay_, az_, kx), Aky = sel3(ax_, ay_, az_, ky), Akz = sel3(ax_, ay_, az_, kz);
  const float Bkx = sel3(bx_, by_, bz_, kx), Bky = sel3(bx_, by_, bz_, ky), Bkz = sel3(bx_, by_, bz_, kz);
  const float Ckx = sel3(cx_, cy_, cz_, kx), Cky = sel3(cx_, cy_, cz_, ky), Ckz = sel3(cx_, cy_, cz_, kz);
  // shear
  const float Axs = fsub(Akx, fmul(r.Sx, Akz)), Ays = fsub(Aky, fmul(r.Sy, Akz));
  const float Bxs = fsub(Bkx, fmul(r.Sx, Bkz)), Bys = fsub(Bky, fmul(r.Sy, Bkz));
  const float Cxs = fsub(Ckx, fmul(r.Sx, Ckz)), Cys = fsub(Cky, fmul(r.Sy, Ckz));
  // scaled barycentrics (edge functions)
  const float U = fsub(fmul(Cxs, Bys), fmul(Cys, Bxs));
  const float V = fsub(fmul(Axs, Cys), fmul(Ays, Cxs));
  const float W = fsub(fmul(Bxs, Ays), fmul(Bys, Axs));
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return __int_as_float(0x7f800000);
  const float det = fadd(fadd(U, V), W);
  if (det == 0.0f) return __int_as_float(0x7f800000);
  const float Az = fmul(r.Sz, Akz), Bz = fmul(r.Sz, Bkz), Cz = fmul(r.Sz, Ckz);
  const float T = fadd(fadd(fmul(U, Az), fmul(V, Bz)), fmul(W, Cz));
  const float t = fdiv(T, det);
  if (!(t > tmin)) return __int_as_float(0x7f800000);
  return t;
}

// ---------------------------------------------------------------------------
// Closest-hit traversal of the 8-wide compressed BVH, one node per step.
//
// Box tests are made conservative by padding each slab distance by
// 2^-20 (|c| + 255 |s|), which bounds the rounding of q*s + c with
// s = 2^e/d and c = (p-o)/d -- 1/d within 2 ulp, p-o, the product, the fma
// and the padding's own subtraction: about 9 * 2^-24 (|c| + 255 |s|) in all,
// against 16 * 2^-24 -- so the traversal never culls a box the exact ray
// enters.  Candidates are culled against best_t*(1+2^-16) + slack.
// Together with the lowest-index tie rule the result equals a brute-force
// scan with the same triangle test.
//
// The traversal is resumable: trav_step() processes one node -- its eight
// child boxes, then, in one flat loop, the triangles of the leaf children it
// hit -- and moves to the nearest internal child, pushing the others sorted
// by entry distance.  Kernels call it once per loop trip, so a lane whose
// ray finished can start another ray while the rest of its warp is still
// traversing.

struct TraceScene {
  const uint4* nodes;
  const float4* tris;
  uint32_t num_nodes;
  float extent;
#ifdef LISA_BOUNDS
  uint32_t num_tris;
#endif
};

__device__ __forceinline__ TraceScene trace_scene(const SceneDev& sc) {
  TraceScene t;
  t.nodes = sc.nodes;
  t.tris = sc.tris;
  t.num_nodes = sc.num_nodes;
  t.extent = sc.extent;
#ifdef LISA_BOUNDS
  t.num_tris = sc.num_prims;
#endif
  return t;
}

// The emissive triangles' own BVH, with the scene's extent (the ray set-up
// and so every triangle test are those of the scene's BVH).
__device__ __forceinline__ TraceScene trace_scene_emit(const SceneDev& sc) {
  TraceScene t;
  t.nodes = sc.enodes;
  t.tris = sc.etris;
  t.num_nodes = sc.num_enodes;
  t.extent = sc.extent;
#ifdef LISA_BOUNDS
  t.num_tris = sc.num_etris;
#endif
  return t;
}

constexpr uint32_t NODE_NONE = 0xffffffffu;

struct TravState {
  RayPre r;
  float tmin;
  // (best_t and best_prim start defined: a lane without a ray still joins
  // its warp's triangle pass, which reads them)
  float best_t = 0.0f;
  float cull;  // best_t * (1+2^-16) + slack
  int best_prim = -1;
  int best_mat;  // emitter material of the best hit, -1 if not an emitter (from the leaf triangle)
  uint32_t node;
  int sp;
  bool any;  // stop at the first non-emitter hit found (see trav_pop)
};

__device__ __forceinline__ float byte_f(uint32_t w, int b) { return (float)((w >> (8 * b)) & 0xffu); }

// Starts a ray; returns false when there is nothing to traverse (empty
// scene or zero direction), in which case the ray is a miss.  With `any`
// the traversal ends at the first hit it finds: best_prim then says only
// whether the segment (tmin, tmax) is blocked.
__device__ __forceinline__ bool trav_begin(TravState& s, const TraceScene& sc, V3 o, V3 d, float tmin, float tmax,
                                           bool any = false) {
  s.any = any;
  s.best_t = tmax;
  s.cull = tmax;
  s.best_prim = -1;
  s.tmin = tmin;
  s.sp = 0;
  s.node = 0;
  if (sc.num_nodes == 0 || is_zero(d)) return false;
  s.r = ray_prepare(o, d, sc.extent);
  return true;
}

// One node of the traversal, in three parts.  trav_node tests the node's
// eight child boxes, pushes the internal children it hits (with their entry
// distances) and returns, as a bitmask over the node's triangle slots, the
// triangles of the leaf children it hits.  The triangles are then tested,
// by the lane itself (trav_tris) or by its warp (trav_tris_warp), and
// trav_pop orders the pushed children and moves to the next node.
struct NodeWork {
  uint32_t tmask;     // triangle slots tri_base + bit index still to test
  uint32_t tri_base;
  int sp0;            // stack depth before this node's pushes
};

template <bool COUNT>
__device__ __forceinline__ NodeWork trav_node(TravState& s, const TraceScene& sc, uint2* stack, uint32_t& visits,
                                              uint32_t* status) {
  const RayPre& r = s.r;
#ifdef LISA_BOUNDS
  if (s.node >= sc.num_nodes) {  // end the ray
    if (status) atomicOr(status, ST_BOUNDS);
    NodeWork bad;
    bad.tmask = 0;
    bad.tri_base = 0;
    bad.sp0 = 0;
    s.sp = 0;
    return bad;
  }
#endif
  if (COUNT) ++visits;
  const uint4* np = sc.nodes + 5ull * s.node;
  const uint4 n0 = __ldg(np + 0);
  const uint4 n1 = __ldg(np + 1);
  const uint4 n2 = __ldg(np + 2);
  const uint4 n3 = __ldg(np + 3);
  const uint4 n4 = __ldg(np + 4);
  const float sx = __int_as_float((n0.w & 0xffu) << 23) * r.ix;
  const float sy = __int_as_float(((n0.w >> 8) & 0xffu) << 23) * r.iy;
  const float sz = __int_as_float(((n0.w >> 16) & 0xffu) << 23) * r.iz;
  const float cx = (__uint_as_float(n0.x) - r.ox) * r.ix;
  const float cy = (__uint_as_float(n0.y) - r.oy) * r.iy;
  const float cz = (__uint_as_float(n0.z) - r.oz) * r.iz;
  const float gx = 9.5367431640625e-7f * (fabsf(cx) + 255.0f * fabsf(sx));
  const float gy = 9.5367431640625e-7f * (fabsf(cy) + 255.0f * fabsf(sy));
  const float gz = 9.5367431640625e-7f * (fabsf(cz) + 255.0f * fabsf(sz));
  const float cnx = cx - gx, cfx = cx + gx;
  const float cny = cy - gy, cfy = cy + gy;
  const float cnz = cz - gz, cfz = cz + gz;
  const bool negx = r.ix < 0.0f, negy = r.iy < 0.0f, negz = r.iz < 0.0f;
  const uint32_t nx0 = negx ? n3.z : n2.x, nx1 = negx ? n3.w : n2.y;
  const uint32_t fx0 = negx ? n2.x : n3.z, fx1 = negx ? n2.y : n3.w;
  const uint32_t ny0 = negy ? n4.x : n2.z, ny1 = negy ? n4.y : n2.w;
  const uint32_t fy0 = negy ? n2.z : n4.x, fy1 = negy ? n2.w : n4.y;
  const uint32_t nz0 = negz ? n4.z : n3.x, nz1 = negz ? n4.w : n3.y;
  const uint32_t fz0 = negz ? n3.x : n4.z, fz1 = negz ? n3.y : n4.w;
  const uint32_t imask = n0.w >> 24;
  const uint32_t child_base = n1.x;
  NodeWork w;
  w.tri_base = n1.y;
  // child boxes: hit mask; internal children that are hit go straight onto
  // the stack with their entry distance (predicated stores, no branches)
  uint32_t hit = 0;
  w.sp0 = s.sp;
  int sp = w.sp0;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int b = c & 3;
    const float a0 = fmaf(byte_f(c < 4 ? nx0 : nx1, b), sx, cnx);
    const float a1 = fmaf(byte_f(c < 4 ? ny0 : ny1, b), sy, cny);
    const float a2 = fmaf(byte_f(c < 4 ? nz0 : nz1, b), sz, cnz);
    const float f0 = fmaf(byte_f(c < 4 ? fx0 : fx1, b), sx, cfx);
    const float f1 = fmaf(byte_f(c < 4 ? fy0 : fy1, b), sy, cfy);
    const float f2 = fmaf(byte_f(c < 4 ? fz0 : fz1, b), sz, cfz);
    const float tn = fmaxf(fmaxf(a0, a1), fmaxf(a2, s.tmin));
    const float tf = fminf(fminf(f0, f1), fminf(f2, s.cull));
    const bool h = tn <= tf;
    hit |= (h ? 1u : 0u) << c;
    if (h && ((imask >> c) & 1u) && sp < TRAV_STACK) {
      const uint32_t meta = ((c < 4 ? n1.z : n1.w) >> (8 * b)) & 0xffu;
      stack[sp++] = make_uint2(child_base + meta, __float_as_uint(tn));
    }
  }
  if (status && (imask & hit) && sp == TRAV_STACK && __popc(imask & hit) > sp - w.sp0)
    atomicOr(status, ST_STACK_OVERFLOW);
  s.sp = sp;
  // occupied slots: internal children and leaves with a non-zero meta byte
  uint32_t leafmask = 0;
#pragma unroll
  for (int c = 0; c < 8; ++c) leafmask |= ((((c < 4 ? n1.z : n1.w) >> (8 * (c & 3))) & 0xe0u) ? 1u : 0u) << c;
  leafmask &= ~imask & hit;
  // triangles of the hit leaves, as a bitmask over the node's triangle slots
  w.tmask = 0;
  while (leafmask) {
    const int c = __ffs(leafmask) - 1;
    leafmask &= leafmask - 1;
    const uint32_t meta = ((c < 4 ? n1.z : n1.w) >> (8 * (c & 3))) & 0xffu;
    w.tmask |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
  }
#ifdef LISA_BOUNDS
  if (w.tmask && w.tri_base + (31u - (uint32_t)__clz(w.tmask)) >= sc.num_tris) {
    if (status) atomicOr(status, ST_BOUNDS);
    w.tmask = 0;
  }
#endif
  return w;
}

// Keeps the hit (t, prim) if it is nearer, or as near with a lower
// triangle index (the brute-force tie rule).
__device__ __forceinline__ void trav_take(TravState& s, float t, int prim, int mat) {
  if (t < s.best_t || (t == s.best_t && prim < s.best_prim)) {
    s.best_t = t;
    s.best_prim = prim;
    s.best_mat = mat;
    s.cull = fmaf(t, 1.52587890625e-5f, t) + s.r.slack;
  }
}

// The lane tests its own triangles.
template <bool COUNT>
__device__ __forceinline__ void trav_tris(TravState& s, const TraceScene& sc, NodeWork w, uint32_t& tests) {
  while (w.tmask) {
    const int j = __ffs(w.tmask) - 1;
    w.tmask &= w.tmask - 1;
    const float4* tp = sc.tris + 3ull * (w.tri_base + (uint32_t)j);
    const float4 a = __ldg(tp + 0), bb = __ldg(tp + 1), cc = __ldg(tp + 2);
    if (COUNT) ++tests;
    trav_take(s, intersect_tri(s.r, a, bb, cc, s.tmin), __float_as_int(a.w), __float_as_int(bb.w));
  }
}

// Per-warp scratch of trav_tris_warp (shared memory).
struct TriPass {
  unsigned long long key[32];  // (t bits << 32 | triangle id) of each lane's best hit
  int mat[32];
  int owner[32];               // lane whose triangles start at this position of a pass
};

// The warp tests the triangles of all its lanes together, 32 at a time:
// the lanes' triangle lists are laid end to end (a prefix sum of their
// counts) and lane j of a pass takes the j-th triangle of the pass, with
// the owner's ray.  The owner's best hit is the minimum of the 64-bit keys
// (t, triangle id) -- t is positive, so its bits order as the float -- the
// same choice as the lane's own loop with its tie rule.  Called by all 32
// lanes; lanes without a ray pass w.tmask = 0.
template <bool COUNT>
__device__ __forceinline__ void trav_tris_warp(TravState& s, const TraceScene& sc, NodeWork w, uint32_t& tests,
                                               TriPass& tp) {
  const int lane = threadIdx.x & 31;
  const uint32_t cnt = __popc(w.tmask);
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  if (total == 0) return;
  // when no lane has more triangles than the passes a warp would need,
  // the lanes' own loops are cheaper than the exchange
  if (__reduce_max_sync(0xffffffffu, cnt) <= ((total + 31u) >> 5)) {
    if (cnt) trav_tris<COUNT>(s, sc, w, tests);
    return;
  }
  const uint32_t excl = incl - cnt;
  const unsigned long long key0 =
      ((unsigned long long)__float_as_uint(s.best_t) << 32) | (uint32_t)s.best_prim;
  tp.key[lane] = key0;
  for (uint32_t k0 = 0; k0 < total; k0 += 32) {
    // positions of this pass where a lane's list starts (the list holding
    // position 0 starts there too)
    const bool here = cnt && excl < k0 + 32 && excl + cnt > k0;
    const uint32_t pos = excl > k0 ? excl - k0 : 0u;
    if (here) tp.owner[pos] = lane;
    const uint32_t starts = __reduce_or_sync(0xffffffffu, here ? 1u << pos : 0u);
    __syncwarp();
    const uint32_t k = k0 + (uint32_t)lane;
    // the list holding position `lane`: the last start at or below it
    const int first = 31 - __clz(starts & (0xffffffffu >> (31 - lane)));
    const int o = tp.owner[first];
    const uint32_t o_excl = __shfl_sync(0xffffffffu, excl, o);
    uint32_t m = __shfl_sync(0xffffffffu, w.tmask, o);
    const uint32_t o_base = __shfl_sync(0xffffffffu, w.tri_base, o);
    RayPre r;
    r.ox = __shfl_sync(0xffffffffu, s.r.ox, o);
    r.oy = __shfl_sync(0xffffffffu, s.r.oy, o);
    r.oz = __shfl_sync(0xffffffffu, s.r.oz, o);
    r.k = __shfl_sync(0xffffffffu, s.r.k, o);
    r.Sx = __shfl_sync(0xffffffffu, s.r.Sx, o);
    r.Sy = __shfl_sync(0xffffffffu, s.r.Sy, o);
    r.Sz = __shfl_sync(0xffffffffu, s.r.Sz, o);
    const float tmin = __shfl_sync(0xffffffffu, s.tmin, o);
    const unsigned long long tris_p = __shfl_sync(0xffffffffu, (unsigned long long)sc.tris, o);
    const unsigned long long okey = __shfl_sync(0xffffffffu, key0, o);
    bool better = false;
    unsigned long long key = 0;
    int mat = 0;
    if (k < total) {
      // the (k - o_excl)-th remaining triangle of the owner's list
      for (uint32_t i = k - o_excl; i > 0; --i) m &= m - 1;
      const uint32_t j = (uint32_t)(__ffs(m) - 1);
      const float4* tq = (const float4*)tris_p + 3ull * (o_base + j);
      const float4 a = __ldg(tq + 0), bb = __ldg(tq + 1), cc = __ldg(tq + 2);
      if (COUNT) ++tests;
      const float t = intersect_tri(r, a, bb, cc, tmin);
      const int prim = __float_as_int(a.w);
      const float bt = __uint_as_float((uint32_t)(okey >> 32));
      const int bp = (int)(uint32_t)okey;
      if (t < bt || (t == bt && prim < bp)) {
        better = true;
        key = ((unsigned long long)__float_as_uint(t) << 32) | (uint32_t)prim;
        mat = __float_as_int(bb.w);
        atomicMin(&tp.key[o], key);
      }
    }
    __syncwarp();
    if (better && tp.key[o] == key) tp.mat[o] = mat;
    __syncwarp();
  }
  const unsigned long long best = tp.key[lane];
  if (best != key0) {
    s.best_t = __uint_as_float((uint32_t)(best >> 32));
    s.best_prim = (int)(uint32_t)best;
    s.best_mat = tp.mat[lane];
    s.cull = fmaf(s.best_t, 1.52587890625e-5f, s.best_t) + s.r.slack;
  }
  __syncwarp();
}

// Whether the ray may meet the box [lo, hi] inside (tmin, tmax): slab
// distances from the node-culling reciprocals, each widened by 2^-20 of
// their magnitude, which covers their roundings (conservative: a ray that
// meets the box is never rejected).
__device__ __forceinline__ bool box_may_hit(const RayPre& r, const float* lo, const float* hi, float tmin,
                                            float tmax) {
  const float ax = (lo[0] - r.ox) * r.ix, bx = (hi[0] - r.ox) * r.ix;
  const float ay = (lo[1] - r.oy) * r.iy, by = (hi[1] - r.oy) * r.iy;
  const float az = (lo[2] - r.oz) * r.iz, bz = (hi[2] - r.oz) * r.iz;
  const float gx = 9.5367431640625e-7f * (fabsf(ax) + fabsf(bx));
  const float gy = 9.5367431640625e-7f * (fabsf(ay) + fabsf(by));
  const float gz = 9.5367431640625e-7f * (fabsf(az) + fabsf(bz));
  const float tn = fmaxf(fmaxf(fminf(ax, bx) - gx, fminf(ay, by) - gy), fmaxf(fminf(az, bz) - gz, tmin));
  const float tf = fminf(fminf(fmaxf(ax, bx) + gx, fmaxf(ay, by) + gy), fminf(fmaxf(az, bz) + gz, tmax));
  return tn <= tf;
}

// Whether a ray from o along d may meet the scene's emissive triangles
// inside (RAY_TMIN, RAY_TMAX): box_may_hit against their padded bounds with
// the node-culling reciprocals (__fdividef, within 2 ulp; a huge finite
// value for a vanishing component), without the rest of a ray set-up.
// Conservative: false only when no emitter can be hit.
__device__ __forceinline__ bool emit_may_hit(const SceneDev& sc, V3 o, V3 d) {
  if (!sc.has_emit_box) return false;
  RayPre r;
  r.ox = o.x;
  r.oy = o.y;
  r.oz = o.z;
  r.ix = fabsf(d.x) > 1e-30f ? __fdividef(1.0f, d.x) : copysignf(1e30f, d.x);
  r.iy = fabsf(d.y) > 1e-30f ? __fdividef(1.0f, d.y) : copysignf(1e30f, d.y);
  r.iz = fabsf(d.z) > 1e-30f ? __fdividef(1.0f, d.z) : copysignf(1e30f, d.z);
  return box_may_hit(r, sc.emit_lo, sc.emit_hi, RAY_TMIN, RAY_TMAX);
}

// Conservative emit_may_hit for a hemisphere draw (x, y, z) of
// shoot_ray_hemisphere before it is normalised and flipped.  The draw,
// flipped by the sign of dot(N, draw), points along the same ray as the
// exact direction (a positive multiple, up to the direction's own
// rounding, which the slab padding covers); testing it on (0, inf) covers
// every point of (RAY_TMIN, RAY_TMAX) along the exact direction.  Where
// dot(N, draw) is too near zero for its sign to be certain (a few ulp of
// the exact dot would be), or not a number, the answer is "may hit".
__device__ __forceinline__ bool emit_may_hit_draw(const SceneDev& sc, V3 o, V3 N, float x, float y, float z) {
  if (!sc.has_emit_box) return false;
  const float s = N.x * x + N.y * y + N.z * z;
  if (!(fabsf(s) > 1e-5f * (fabsf(x) + fabsf(y) + fabsf(z)))) return true;
  const float f = s > 0.0f ? 1.0f : -1.0f;
  const float dx = f * x, dy = f * y, dz = f * z;
  RayPre r;
  r.ox = o.x;
  r.oy = o.y;
  r.oz = o.z;
  r.ix = fabsf(dx) > 1e-30f ? __fdividef(1.0f, dx) : copysignf(1e30f, dx);
  r.iy = fabsf(dy) > 1e-30f ? __fdividef(1.0f, dy) : copysignf(1e30f, dy);
  r.iz = fabsf(dz) > 1e-30f ? __fdividef(1.0f, dz) : copysignf(1e30f, dz);
  return box_may_hit(r, sc.emit_lo, sc.emit_hi, 0.0f, 3.0e38f);
}

// Whether the ray (o, d) may meet the box [lo, hi] inside (tmin, tmax),
// every step a single IEEE rounding so the host oracle takes the same
// decision bit for bit: slab distances with the correctly rounded 1/d (a
// huge finite value of d's sign for a zero component), each widened by
// 2^-20 of their magnitude.  Used where a ray is traced only for the
// emission it may reach: one that misses the emissive triangles' padded
// bounds would gather nothing, so it is not traced at all.
__device__ __forceinline__ bool box_may_hit_exact(V3 o, V3 d, const float* lo, const float* hi, float tmin,
                                                  float tmax) {
  const float dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z};
  float tn = tmin, tf = tmax;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float inv = dd[k] != 0.0f ? __frcp_rn(dd[k]) : copysignf(1e30f, dd[k]);
    const float a = fmul(fsub(lo[k], oo[k]), inv), b = fmul(fsub(hi[k], oo[k]), inv);
    const float g = fmul(9.5367431640625e-7f, fadd(fabsf(a), fabsf(b)));
    tn = fmaxf(tn, fsub(fminf(a, b), g));
    tf = fminf(tf, fadd(fmaxf(a, b), g));
  }
  return tn <= tf;
}

// Orders the children trav_node pushed by entry distance (nearest on top)
// and moves to the nearest child not culled.  Returns true when the
// traversal is finished.
__device__ __forceinline__ bool trav_pop(TravState& s, uint2* stack, int sp0) {
  // an any-hit traversal ends at its first hit that is not an emitter's (a
  // ray that cannot reach an emitter only finds such hits; the emitter
  // search's scene pass starts from an emitter hit and looks for a nearer
  // triangle, which cannot be an emitter's)
  if (s.any && s.best_prim >= 0 && s.best_mat < 0) return true;
  // (entry distances are positive, so their bit patterns order as floats)
  const int sp = s.sp;
  for (int i = sp0 + 1; i < sp; ++i) {
    const uint2 e = stack[i];
    int k = i;
    while (k > sp0 && stack[k - 1].y < e.y) {
      stack[k] = stack[k - 1];
      --k;
    }
    stack[k] = e;
  }
  while (s.sp > 0) {
    const uint2 e = stack[--s.sp];
    if (__uint_as_float(e.y) <= s.cull) {
      s.node = e.x;
      return false;
    }
  }
  return true;
}

// Processes one node with the lane's own triangle loop.  Returns true when
// the traversal is finished (s.best_prim / s.best_t hold the result,
// best_prim -1 on a miss).
template <bool COUNT>
__device__ __forceinline__ bool trav_step(TravState& s, const TraceScene& sc, uint2* stack, uint32_t& visits,
                                          uint32_t& tests, uint32_t* status) {
  const NodeWork w = trav_node<COUNT>(s, sc, stack, visits, status);
  trav_tris<COUNT>(s, sc, w, tests);
  return trav_pop(s, stack, w.sp0);
}

// The same step for a whole warp (all 32 lanes call it), the triangles
// tested by trav_tris_warp.  Returns true for an active lane whose
// traversal is finished; inactive lanes get false.
template <bool COUNT>
__device__ __forceinline__ bool trav_step_warp(bool active, TravState& s, const TraceScene& sc, uint2* stack,
                                               uint32_t& visits, uint32_t& tests, uint32_t* status, TriPass& tp) {
  NodeWork w;
  w.tmask = 0;
  w.tri_base = 0;
  w.sp0 = 0;
  if (active) w = trav_node<COUNT>(s, sc, stack, visits, status);
  trav_tris_warp<COUNT>(s, sc, w, tests, tp);
  return active && trav_pop(s, stack, w.sp0);
}

template <bool COUNT>
__device__ __forceinline__ void closest_hit(const TraceScene& sc, V3 o, V3 d, float tmin, float tmax, int& out_prim,
                                            float& out_t, uint32_t& visits, uint32_t& tests, uint32_t* status) {
  TravState s;
  uint2 stack[TRAV_STACK];
  if (trav_begin(s, sc, o, d, tmin, tmax)) {
    while (!trav_step<COUNT>(s, sc, stack, visits, tests, status)) {
    }
  }
  out_prim = s.best_prim;
  out_t = s.best_prim >= 0 ? s.best_t : __int_as_float(0x7f800000);
}

// Brute-force scan in original triangle order with the same test and tie
// rule (lowest index wins on equal t).
__device__ __forceinline__ void brute_hit(const SceneDev& sc, V3 o, V3 d, float tmin, float tmax, int& out_prim,
                                          float& out_t) {
  out_prim = -1;
  out_t = __int_as_float(0x7f800000);
  if (is_zero(d)) return;
  const RayPre r = ray_prepare(o, d, sc.extent);
  float best_t = tmax;
  int best = -1;
  for (uint32_t p = 0; p < sc.num_prims; ++p) {
    const float4* pr = sc.prims + 5ull * p;
    const float4 a = __ldg(pr + 0), b = __ldg(pr + 1), c = __ldg(pr + 2);
    const float t = intersect_tri(r, a, b, c, tmin);
    if (t < best_t) {
      best_t = t;
      best = (int)p;
    }
  }
  if (best >= 0) {
    out_prim = best;
    out_t = best_t;
  }
}

}  // namespace lisa

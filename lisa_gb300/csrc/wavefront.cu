// Wavefront path tracer: the reference estimator (src/LiSA/src/shader.cu)
// re-organised as stages over SoA queues instead of one OptiX thread per
// pixel.
//
//   raygen      one path per (scene, pixel, sample) slot          shader.cu:126-155
//   trace       closest hit of every queued ray (persistent warps) shader.cu:77-98
//   shade       per hit, by material class:                       shader.cu:211-255
//                 miss / emitter -> path ends (emitter adds Le*att)
//                 dielectric     -> Fresnel reflect / refract, next ray
//                 opaque         -> att *= albedo, enqueue emitter search
//   nee         up to 30 hemisphere rays per opaque vertex until one
//               returns the (stale) emitter, then the bounce          shader.cu:196-209,248-253
//   accumulate  per pixel, Kahan FP32 sum + FP64 sum of squares     shader.cu:156-166
//
// The persistent kernels take work with warp-aggregated atomics (one atomic
// per warp per refill); queue appends are warp-aggregated the same way.
// Counters that a stage consumes are reset by a stage that does not run
// concurrently with it (see the comments at each reset).
#include <algorithm>
#include <cstring>
#include <vector>

#include "guide.cuh"
#include "guide_mix.cuh"
#include "lisa_device.cuh"
#include "lisa_internal.h"
#include "wavefront.cuh"

#ifndef LISA_BSDF_HEADER
#define LISA_BSDF_HEADER "bsdfs/lambertian.cuh"
#endif
#include LISA_BSDF_HEADER
#include "guide_infer.cuh"
#include "physical.cuh"

namespace lisa {

constexpr uint32_t FULL = 0xffffffffu;

#ifndef LISA_NEE_MIN_BLOCKS
#define LISA_NEE_MIN_BLOCKS 6  // 6 x 128 threads per SM (80 registers; measured best of 6..8)
#endif
// Residency of the closest-hit and shade kernels: blocks per SM the
// compiler must fit (0 = its own register choice).  Measured: the closest-hit
// kernel at 8 (64 registers, no spills) is 4 % faster than at 7 (72); the
// shade kernel is fastest with its own choice (56 registers).
#ifndef LISA_TRACE_MIN_BLOCKS
#define LISA_TRACE_MIN_BLOCKS 8
#endif
#ifndef LISA_SHADE_MIN_BLOCKS
#define LISA_SHADE_MIN_BLOCKS 0
#endif
#if LISA_TRACE_MIN_BLOCKS > 0
#define LISA_TRACE_BOUNDS __launch_bounds__(128, LISA_TRACE_MIN_BLOCKS)
#else
#define LISA_TRACE_BOUNDS __launch_bounds__(128)
#endif
#if LISA_SHADE_MIN_BLOCKS > 0
#define LISA_SHADE_BOUNDS __launch_bounds__(256, LISA_SHADE_MIN_BLOCKS)
#else
#define LISA_SHADE_BOUNDS __launch_bounds__(256)
#endif
#ifndef LISA_NEE_PB_MIN_BLOCKS
#define LISA_NEE_PB_MIN_BLOCKS 7  // physically based emitter kernel: 7 x 128 threads per SM
#endif
#ifndef LISA_REFILL_IDLE
#define LISA_REFILL_IDLE 12  // default: idle lanes (of 32) that trigger a refill round
#endif

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Warp-aggregated reservation of `want ? 1 : 0` entries in *counter.  All 32
// lanes must call it.  Returns the lane's index (undefined if !want).
__device__ __forceinline__ uint32_t warp_reserve(uint32_t* counter, bool want) {
  const uint32_t mask = __ballot_sync(FULL, want);
  if (!mask) return 0;
  const int leader = __ffs(mask) - 1;
  const int lane = threadIdx.x & 31;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
  base = __shfl_sync(FULL, base, leader);
  return base + __popc(mask & lanemask_lt());
}

__device__ __forceinline__ void warp_add64(unsigned long long* c, uint32_t v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(c, (unsigned long long)v);
}

// Whether queue slot i, reserved by an append, lies inside the queue: always,
// by construction (one entry per path and depth); checked in bounds-checked
// builds, where a bad slot sets ST_QUEUE_OVERFLOW and the write is skipped.
__device__ __forceinline__ bool queue_fits(const WaveBufs& b, uint32_t i) {
#ifdef LISA_BOUNDS
  if (i < b.capacity) return true;
  atomicOr(&b.ctrl->status, ST_QUEUE_OVERFLOW);
  return false;
#else
  (void)b;
  (void)i;
  return true;
#endif
}

// The ray leaving a path's last vertex (physically based estimator) only
// gathers emission: it is traced only if it may meet the scene's emitters.
__device__ __forceinline__ bool final_ray_wanted(const SceneDev& sc, V3 p, V3 d) {
  return sc.has_emit_box && box_may_hit_exact(p, d, sc.emit_lo, sc.emit_hi, RAY_TMIN, RAY_TMAX);
}

__device__ __forceinline__ void warp_add32(uint32_t* c, uint32_t v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(c, v);
}

__device__ __forceinline__ V3 barycentric_normal(V3 p, const float4* pr) {
  // src/LiSA/src/maths.cu:33-56 (barycentrics re-derived from the hit point)
  const float4 r0 = __ldg(pr + 0), r1 = __ldg(pr + 1), r2 = __ldg(pr + 2), r3 = __ldg(pr + 3), r4 = __ldg(pr + 4);
  const V3 v1 = ld3(r0), v2 = ld3(r1), v3_ = ld3(r2);
  const V3 n1 = v3(r0.w, r1.w, r2.w);
  const V3 n2 = v3(r3.x, r3.y, r3.z);
  const V3 n3 = v3(r3.w, r4.x, r4.y);
  const V3 e1 = v2 - v1, e2 = v3_ - v1, i = p - v1;
  const float d00 = dot(e1, e1), d01 = dot(e1, e2), d11 = dot(e2, e2);
  const float d20 = dot(i, e1), d21 = dot(i, e2);
  const float denom = fsub(fmul(d00, d11), fmul(d01, d01));
  const float w = fdiv(fsub(fmul(d00, d21), fmul(d01, d20)), denom);
  const float v = fdiv(fsub(fmul(d11, d20), fmul(d01, d21)), denom);
  const float u = fsub(fsub(1.0f, v), w);
  return normalize((u * n1 + v * n2) + w * n3);
}

__device__ __forceinline__ int prim_material(const SceneDev& sc, int prim) {
  return __float_as_int(__ldg(sc.prims + 5ull * prim + 4).z);
}

__device__ __forceinline__ int find_group(const WaveDesc& w, uint32_t key, bool by_acc) {
  int lo = 0, hi = (int)w.num_groups - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const uint32_t b = by_acc ? w.groups[mid].acc0 : w.groups[mid].slot0;
    if (b <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// raygen (shader.cu:126-152) -- also resets the counters of depth 0

__global__ void k_raygen(WaveBufs b, const WaveDesc* __restrict__ wave) {
  const WaveDesc& w = *wave;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // nothing else runs during raygen
    b.ctrl->qcount[0] = w.paths;
    b.ctrl->qcount[1] = 0;
    b.ctrl->nee_count = 0;
    b.ctrl->head[HEAD_TRACE] = 0;
    b.ctrl->head[HEAD_SHADE] = 0;
    b.ctrl->head[HEAD_NEE] = 0;
    b.ctrl->guided_count = 0;
    b.ctrl->rec_count = 0;
    b.ctrl->train_count = 0;
    b.ctrl->rays_primary += w.paths;
  }
  for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < w.paths; slot += gridDim.x * blockDim.x) {
    const WaveGroup& g = w.groups[find_group(w, slot, false)];
    const SceneDev& sc = b.scenes[g.scene];
    const uint32_t off = slot - g.slot0;
    const uint32_t m = off / g.npix;
    const uint32_t pix = g.pix0 + (off - m * g.npix);
    const uint32_t sample = g.sample0 + m;
    const uint32_t x = pix % sc.width, y = pix / sc.width;
    uint32_t seed;
    if (w.rng_mode == LISA_RNG_PER_PIXEL) {
      seed = sc.pix_rng[pix];
    } else {
      seed = tea<16>(pix, tea<4>(sample, w.seed));
    }
    const float jx = rng11(seed);
    const float jy = rng11(seed);
    const float dx = fsub(fdiv(fadd(fmul(2.0f, (float)x), jx), (float)sc.width), 1.0f);
    const float dy = fsub(fdiv(fadd(fmul(2.0f, (float)y), jy), (float)sc.height), 1.0f);
    const V3 U = v3(sc.U[0], sc.U[1], sc.U[2]), V = v3(sc.V[0], sc.V[1], sc.V[2]), W = v3(sc.W[0], sc.W[1], sc.W[2]);
    V3 dir = normalize((dx * U + dy * V) + W);
    V3 org = v3(sc.eye[0], sc.eye[1], sc.eye[2]);
    if (sc.lens_radius > 0.0f) {
      // Thin lens (not in the reference, whose camera is a pinhole): the
      // pinhole ray meets the focal plane at distance focal_distance along
      // the view axis; the origin moves to a uniform point of the lens disk,
      // drawn by rejection from the square (trig-free, so the oracle draws
      // the same point bit for bit).
      const V3 wu = v3(sc.unitW[0], sc.unitW[1], sc.unitW[2]);
      const float tf = fdiv(sc.focal_distance, dot(dir, wu));
      const V3 focus = org + tf * dir;
      float lu, lv;
      do {
        lu = rng11(seed);
        lv = rng11(seed);
      } while (fadd(fmul(lu, lu), fmul(lv, lv)) > 1.0f);
      org = org + fmul(sc.lens_radius, lu) * v3(sc.unitU[0], sc.unitU[1], sc.unitU[2]) +
            fmul(sc.lens_radius, lv) * v3(sc.unitV[0], sc.unitV[1], sc.unitV[2]);
      dir = normalize(focus - org);
    }
    b.ro[0][slot] = make_float4(org.x, org.y, org.z, __uint_as_float(slot));
    b.rd[0][slot] = make_float4(dir.x, dir.y, dir.z, __uint_as_float(g.scene));
    // w: the stale emitter flag (compat, -1 = none) or the pdf of the last
    // diffuse bounce (physically based, 0 = camera or specular)
    b.ps_att[slot] = make_float4(1.0f, 1.0f, 1.0f, b.physical ? 0.0f : __int_as_float(-1));
    b.ps_col[slot] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float((g.scene << 24) | pix));
    b.ps_rng[slot] = seed;
  }
}

// ---------------------------------------------------------------------------
// closest hit of the queued rays: each lane traverses one node per loop trip
// and takes the next ray as soon as its own is done (warp-aggregated fetch).

template <bool COUNT>
__global__ void LISA_TRACE_BOUNDS k_trace(WaveBufs b, int depth) {
  const int q = depth & 1;
  const uint32_t count = *(volatile uint32_t*)&b.ctrl->qcount[q];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // shade/nee of this depth have not started; the previous depth's
    // consumers of these counters have finished
    b.ctrl->qcount[q ^ 1] = 0;
    b.ctrl->nee_count = 0;
    b.ctrl->head[HEAD_SHADE] = 0;
    b.ctrl->head[HEAD_NEE] = 0;
    if (depth > 0) b.ctrl->rays_bounce += count;
  }
  const int lane = threadIdx.x & 31;
  const uint32_t lt = lanemask_lt();
  uint2 stack[TRAV_STACK];
  TravState s;
  TraceScene ts;
  uint32_t ray = 0, visits = 0, tests = 0;
  bool active = false, exhausted = false;
  __shared__ TriPass tri_pass[4];
  TriPass& tp = tri_pass[threadIdx.x >> 5];
  while (true) {
    // take new rays only once enough lanes are idle (see k_nee)
    if (__popc(__ballot_sync(FULL, active)) <= (int)b.refill_busy_max) {
      const bool need = !active && !exhausted;
      const uint32_t nmask = __ballot_sync(FULL, need);
      if (nmask) {
        const int leader = __ffs(nmask) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&b.ctrl->head[HEAD_TRACE], (uint32_t)__popc(nmask));
        base = __shfl_sync(FULL, base, leader);
        if (need) {
          ray = base + __popc(nmask & lt);
          if (ray < count) {
            const float4 o = b.ro[q][ray], d = b.rd[q][ray];
            ts = trace_scene(b.scenes[__float_as_uint(d.w)]);
            active = trav_begin(s, ts, ld3(o), ld3(d), RAY_TMIN, RAY_TMAX);
            if (!active) b.hit[ray] = make_int2(-1, 0x7f800000);
          } else {
            exhausted = true;
          }
        }
      }
      if (!__any_sync(FULL, active || !exhausted)) break;
    }
    if (trav_step_warp<COUNT>(active, s, ts, stack, visits, tests, &b.ctrl->status, tp)) {
      b.hit[ray] = make_int2(s.best_prim, s.best_prim >= 0 ? __float_as_int(s.best_t) : 0x7f800000);
      active = false;
    }
  }
  if (COUNT) {
    warp_add64(&b.ctrl->node_visits[0], visits);
    warp_add64(&b.ctrl->tri_tests[0], tests);
  }
}

// ---------------------------------------------------------------------------
// shade: emitter / miss / dielectric / opaque (shader.cu:189-194,211-255)

template <bool PHYS>
__global__ void LISA_SHADE_BOUNDS k_shade(WaveBufs b, int depth) {
  const int q = depth & 1;
  const uint32_t count = *(volatile uint32_t*)&b.ctrl->qcount[q];
  if (blockIdx.x == 0 && threadIdx.x == 0) b.ctrl->head[HEAD_TRACE] = 0;  // trace of this depth is done
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  for (uint32_t base = gw * 32; base < count; base += warps * 32) {
    const uint32_t i = base + lane;
    bool want_ray = false, want_nee = false;
    V3 p = v3(0.0f), nd = v3(0.0f), N = v3(0.0f), d = v3(0.0f);
    uint32_t slot = 0;
    int mat_idx = 0;
    uint32_t scene = 0;
    if (i < count) {
      const int2 h = b.hit[i];
      const float4 o4 = b.ro[q][i];
      const float4 d4 = b.rd[q][i];
      slot = __float_as_uint(o4.w);
      scene = __float_as_uint(d4.w);
      if (h.x >= 0) {  // a miss adds the background, 0 (optix_wrapper.cc:354-356), and ends the path
        const SceneDev& sc = b.scenes[scene];
        mat_idx = prim_material(sc, h.x);
        const DevMaterial& m = sc.mats[mat_idx];
        float4 att = b.ps_att[slot];
        if (m.cls == MAT_EMIT) {
          // color += Le * att; done (shader.cu:216-218)
          const float4 col = b.ps_col[slot];
          V3 le = v3(m.emission[0], m.emission[1], m.emission[2]) * ld3(att);
          if (PHYS && att.w > 0.0f) {
            // reached by a diffuse bounce: power-heuristic weight against
            // the emitter sampler's density for this direction
            const float prev = att.w;
            const float t = __int_as_float(h.y);
            const float4* pr = sc.prims + 5ull * h.x;
            const V3 v0 = ld3(pr[0]);
            const V3 cr = cross3(ld3(pr[1]) - v0, ld3(pr[2]) - v0);
            const V3 n = cr * fdiv(1.0f, fsqrt(dot(cr, cr)));
            const float cos_y = fabsf(dot(n, ld3(d4)));
            float w = 0.0f;
            if (cos_y > 0.0f) {
              const float pl = fdiv(fmul(m.light_pdf, fmul(t, t)), cos_y);
              w = fdiv(fmul(prev, prev), fadd(fmul(prev, prev), fmul(pl, pl)));
            }
            le = le * w;
          }
          const V3 c = ld3(col) + le;
          b.ps_col[slot] = make_float4(c.x, c.y, c.z, col.w);
        } else if (!PHYS || depth < (int)sc.num_bounces) {
          // (physically based: the ray leaving the last vertex only gathers
          // the emission it reaches, so any other hit ends the path)
          d = ld3(d4);
          const float t = __int_as_float(h.y);
          p = ld3(o4) + t * d;
          N = barycentric_normal(p, sc.prims + 5ull * h.x);
          // the reference estimator traces num_bounces rays; the physically
          // based one also the ray leaving its last vertex
          const bool last = !PHYS && depth + 1 >= (int)sc.num_bounces;
          if (m.cls == MAT_DIELECTRIC) {
            float cosI = dot(d, N);
            float eta;
            V3 nrm;
            V3 a = ld3(att);
            if (cosI < 0.0f) {
              cosI = -cosI;
              eta = fdiv(1.0f, m.ior);
              nrm = N;
            } else {
              a = a * v3(m.albedo[0], m.albedo[1], m.albedo[2]);
              eta = m.ior;
              nrm = -N;
            }
            uint32_t seed = b.ps_rng[slot];
            if (eta == 1.0f) {
              nd = d;
            } else if (PHYS) {
              // total internal reflection reflects; Schlick's term takes the
              // cosine on the less dense side (the transmitted one on exit)
              const float cost2 = fsub(1.0f, fmul(fmul(eta, eta), fsub(1.0f, fmul(cosI, cosI))));
              if (cost2 <= 0.0f) {
                nd = reflect(d, nrm);
              } else if (rnd(seed) <= bsdf::BTDF(eta > 1.0f ? fsqrt(cost2) : cosI, eta)) {
                nd = reflect(d, nrm);
              } else {
                nd = bsdf::refract(cosI, d, nrm, eta);
              }
            } else if (rnd(seed) <= bsdf::BTDF(cosI, eta)) {
              nd = reflect(d, nrm);
            } else {
              // a zero direction (total internal reflection) is traced as a miss
              nd = bsdf::refract(cosI, d, nrm, eta);
            }
            b.ps_rng[slot] = seed;
            b.ps_att[slot] = make_float4(a.x, a.y, a.z, PHYS ? 0.0f : att.w);
            want_ray = !last && !is_zero(nd);
            if (PHYS && want_ray && depth + 1 == (int)sc.num_bounces) want_ray = final_ray_wanted(sc, p, nd);
          } else {
            const V3 a = ld3(att) * v3(m.albedo[0], m.albedo[1], m.albedo[2]);
            b.ps_att[slot] = make_float4(a.x, a.y, a.z, att.w);
            want_nee = true;
          }
        }
      }
    }
    const uint32_t ri = warp_reserve(&b.ctrl->qcount[q ^ 1], want_ray);
    if (want_ray && queue_fits(b, ri)) {
      b.ro[q ^ 1][ri] = make_float4(p.x, p.y, p.z, __uint_as_float(slot));
      b.rd[q ^ 1][ri] = make_float4(nd.x, nd.y, nd.z, __uint_as_float(scene));
    }
    const uint32_t ni = warp_reserve(&b.ctrl->nee_count, want_nee);
    if (want_nee && queue_fits(b, ni)) {
      b.nee_a[ni] = make_float4(p.x, p.y, p.z, __uint_as_float(slot));
      b.nee_b[ni] = make_float4(N.x, N.y, N.z, __int_as_float(mat_idx));
      b.nee_c[ni] = make_float4(d.x, d.y, d.z, __uint_as_float(scene));
    }
  }
}

// ---------------------------------------------------------------------------
// emitter search + bounce (shader.cu:196-209, 248-253; lambertian.cu:7-22)
//
// Each lane owns one opaque vertex at a time and runs a small state machine:
// start a shadow ray (hemisphere draw), traverse one BVH node per loop trip,
// and when the ray ends apply the reference's occlusion programs; after an
// emitter is seen (or 30 rays) it draws the bounce, writes the path state,
// appends the continuation ray and takes the next vertex.  Lanes advance
// independently, so a warp stays full while its vertices need between 1 and
// 30 rays of different lengths.

// Guided bounce at an opaque vertex with roughness 1, where the reference
// draws hemi(N) (lambertian.cu:7-13): one-sample MIS between that sampler
// (probability c) and the guide's vMF mixture.  The path continues with
// weight p_hemi(w) / (c p_hemi(w) + (1-c) q_guide(w)), so the estimator's
// expectation is unchanged; directions below the surface get weight 0.
__device__ __forceinline__ V3 guided_bounce(const float* o, V3 N, uint32_t& seed, float c, float& weight) {
  guide::Lobe L[guide::LOBES];
  guide::decode(o, L);
  V3 w;
  if (rnd(seed) < c) {
    w = bsdf::shoot_ray_hemisphere(N, seed);
  } else {
    const float u0 = rnd(seed), u1 = rnd(seed), u2 = rnd(seed);
    guide::mix_sample(L, u0, u1, u2, w.x, w.y, w.z);
  }
  const float ph = guide::hemi_pdf(N.x, N.y, N.z, w.x, w.y, w.z);
  const float q = c * ph + (1.0f - c) * guide::mix_pdf(L, w.x, w.y, w.z);
  weight = (ph > 0.0f && q > 0.0f && isfinite(q)) ? ph / q : 0.0f;
  return w;
}

template <bool COUNT, bool GUIDED = false>
__global__ void __launch_bounds__(128, LISA_NEE_MIN_BLOCKS) k_nee(WaveBufs b, int depth) {
  const int q = depth & 1;
  const uint32_t count = *(volatile uint32_t*)&b.ctrl->nee_count;
  const int lane = threadIdx.x & 31;
  const uint32_t lt = lanemask_lt();
  uint2 stack[TRAV_STACK];
  TravState s;
  TraceScene ts;
  const SceneDev* sc = nullptr;
  bool have = false, exhausted = false, ray_active = false;
  uint32_t entry = 0, slot = 0, tries = 0, seed = 0;
  int stale = -1, mat_idx = 0;
  // the vertex position lives in the shadow ray's origin (s.r.o*)
  V3 N = v3(0.0f), dir = v3(0.0f);
  s.r.ox = s.r.oy = s.r.oz = 0.0f;
  uint32_t shadow = 0, walked = 0, visits = 0, tests = 0;
  bool pending = false;  // a finished shadow ray not yet evaluated
  bool emit_pass = false;  // the finished traversal was of the emitters' own BVH
  // LCG jumps over j tries (3 draws each), j = 0..31, for the warp's
  // search of the next try that needs a traversal
  __shared__ uint2 s_jump[32];
  if (threadIdx.x < 32) {
    const LcgJump j = lcg_jump(3u * threadIdx.x);
    s_jump[threadIdx.x] = make_uint2(j.a, j.c);
  }
  __syncthreads();
  __shared__ TriPass tri_pass[4];
  TriPass& tp = tri_pass[threadIdx.x >> 5];
  while (true) {
    // Bookkeeping (evaluate finished rays, finish and fetch vertices, start
    // rays) runs only once enough lanes are idle, so its divergent code is
    // shared by many lanes; otherwise the warp keeps traversing.
    const uint32_t busy = __ballot_sync(FULL, ray_active);
    if (__popc(busy) <= (int)b.refill_busy_max) {
      bool want_ray = false;
      V3 nd = v3(0.0f);
      if (pending && emit_pass) {
        // A try with the flag unset matters only if its closest hit is an
        // emitter.  The emitters' BVH gave the nearest emitter on the ray
        // (if none, the try is inconsequential: evaluated as a miss); the
        // scene's BVH, started from that hit as the best so far, keeps it
        // unless a triangle is nearer (or as near with a lower index) --
        // the same closest hit as one traversal of the whole scene.  Such a
        // triangle is not an emitter's, so that pass ends at the first one.
        emit_pass = false;
        if (s.best_prim >= 0) {
          const float te = s.best_t;
          const int pe = s.best_prim, me = s.best_mat;
          ts = trace_scene(*sc);
          ray_active = trav_begin(s, ts, v3(s.r.ox, s.r.oy, s.r.oz), dir, RAY_TMIN, RAY_TMAX);
          s.best_t = te;
          s.best_prim = pe;
          s.best_mat = me;
          s.cull = fmaf(te, 1.52587890625e-5f, te) + s.r.slack;
          s.any = true;
          ++walked;
          pending = !ray_active;
        }
      }
      if (pending) {
        pending = false;
        if (s.best_prim >= 0) {
          // the occlusion hit program marks a hit only on an emitter and
          // otherwise leaves the flag as it was (shader.cu:177-184)
          if (s.best_mat >= 0) stale = s.best_mat;
        } else {
          stale = -1;  // miss (shader.cu:172-175)
        }
        const bool lit = stale >= 0;
        if (lit || ++tries == (uint32_t)NEE_TRIES) {
          const float4 at = b.ps_att[slot];
          const V3 att = ld3(at);
          if (lit) {
            const DevMaterial& em = sc->mats[stale];
            const float brdf = bsdf::BRDF(N, dir, sc->mats[mat_idx]);
            const float4 c = b.ps_col[slot];
            const V3 col = ld3(c) + (v3(em.emission[0], em.emission[1], em.emission[2]) * brdf) * att;
            b.ps_col[slot] = make_float4(col.x, col.y, col.z, c.w);
          }
          if (GUIDED && sc->mats[mat_idx].roughness == 1.0f) {
            // the bounce of a guided vertex is drawn by k_guided_infer,
            // after the guide has seen the emitter flag this search left
            want_ray = false;
          } else {
            const V3 D = ld3(b.nee_c[entry]);
            // the bounce is drawn at every vertex, the last one included, so
            // the per-pixel stream advances exactly as in the reference
            nd = bsdf::bounce(D, N, seed, sc->mats[mat_idx]);
            want_ray = depth + 1 < (int)sc->num_bounces && !is_zero(nd);
          }
          b.ps_rng[slot] = seed;
          b.ps_att[slot] = make_float4(att.x, att.y, att.z, __int_as_float(stale));
          have = false;
        }
      }
      const uint32_t ri = warp_reserve(&b.ctrl->qcount[q ^ 1], want_ray);
      if (want_ray && queue_fits(b, ri)) {
        b.ro[q ^ 1][ri] = make_float4(s.r.ox, s.r.oy, s.r.oz, __uint_as_float(slot));
        b.rd[q ^ 1][ri] = make_float4(nd.x, nd.y, nd.z, __uint_as_float((uint32_t)(sc - b.scenes)));
      }
      const bool need = !have && !exhausted;
      const uint32_t nmask = __ballot_sync(FULL, need);
      if (nmask) {
        const int leader = __ffs(nmask) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&b.ctrl->head[HEAD_NEE], (uint32_t)__popc(nmask));
        base = __shfl_sync(FULL, base, leader);
        if (need) {
          entry = base + __popc(nmask & lt);
          if (entry < count) {
            const float4 a4 = b.nee_a[entry], b4 = b.nee_b[entry];
            s.r.ox = a4.x;
            s.r.oy = a4.y;
            s.r.oz = a4.z;
            slot = __float_as_uint(a4.w);
            N = ld3(b4);
            mat_idx = __float_as_int(b4.w);
            stale = __float_as_int(b.ps_att[slot].w);
            seed = b.ps_rng[slot];
            sc = b.scenes + __float_as_uint(__ldg(&b.nee_c[entry].w));
            ts = trace_scene(*sc);
            tries = 0;
            have = true;
          } else {
            exhausted = true;
          }
        }
      }
      if (!__any_sync(FULL, have)) break;
      // The next try of a vertex.  A ray that cannot reach an emitter can
      // only miss (the flag is cleared) or hit something else (the flag is
      // kept): with the flag unset, neither lights the vertex nor changes
      // the flag, so such a try is counted and its traversal skipped -- the
      // search's outcome, the flag it leaves and the seed after it are those
      // of tracing every try.  With the flag set, a ray that cannot reach an
      // emitter is traced to its first hit only (a hit lights the vertex
      // with the flag's emitter, a miss clears it); a ray that may reach one
      // is traced to its closest hit.
      //
      // For the vertices whose flag is unset, the warp finds the next try
      // that may reach an emitter together: the LCG jumps to the state
      // before each later try, so lane j tests try `tries + j` of one
      // vertex (a conservative test on the unnormalised draw), and the first
      // lane that may (or the vertex's last try) sets where the vertex goes
      // on.  The tries before it are passed over without their directions.
      const bool search = have && !ray_active && !pending && stale < 0;
      uint32_t smask = __ballot_sync(FULL, search);
      uint32_t skipped = 0;
      while (smask) {
        const int owner = __ffs(smask) - 1;
        smask &= smask - 1;
        const uint32_t s0 = __shfl_sync(FULL, seed, owner);
        const uint32_t t0 = __shfl_sync(FULL, tries, owner);
        const V3 po = v3(__shfl_sync(FULL, s.r.ox, owner), __shfl_sync(FULL, s.r.oy, owner),
                         __shfl_sync(FULL, s.r.oz, owner));
        const V3 no = v3(__shfl_sync(FULL, N.x, owner), __shfl_sync(FULL, N.y, owner), __shfl_sync(FULL, N.z, owner));
        const SceneDev* so = (const SceneDev*)__shfl_sync(FULL, (unsigned long long)sc, owner);
        const uint32_t t = t0 + (uint32_t)lane;
        bool cand = t + 1 == (uint32_t)NEE_TRIES;
        if (t + 1 < (uint32_t)NEE_TRIES) {
          const uint2 j = s_jump[lane];
          uint32_t st = j.x * s0 + j.y;
          const float hx = rng11(st);
          const float hy = rng11(st);
          const float hz = rng11(st);
          cand = emit_may_hit_draw(*so, po, no, hx, hy, hz);
        }
        // the vertex's last try is always a candidate, so a lane is found
        const int first = __ffs(__ballot_sync(FULL, cand)) - 1;
        if (lane == owner) {
          const uint2 j = s_jump[first];
          seed = j.x * seed + j.y;
          tries = t0 + (uint32_t)first;
          skipped = (uint32_t)first;
        }
      }
      if (have && !ray_active && !pending) {
        const V3 p = v3(s.r.ox, s.r.oy, s.r.oz);
        shadow += skipped + 1;
        const float hx = rng11(seed);
        const float hy = rng11(seed);
        const float hz = rng11(seed);
        dir = bsdf::hemisphere_direction(N, hx, hy, hz);
        const bool capable = emit_may_hit(*sc, p, dir);
        if (!capable && stale < 0) {
          s.best_prim = -1;  // an inconsequential try: evaluated as a miss
          pending = true;
        } else {
          // with the flag unset, a ray that may reach an emitter first asks
          // the emitters' own BVH (scenes with more than a few emitter
          // triangles; with a few, the bounds test above is as selective)
          emit_pass = stale < 0 && sc->num_etris >= EMIT_BVH_MIN_TRIS;
          ts = emit_pass ? trace_scene_emit(*sc) : trace_scene(*sc);
          ray_active = trav_begin(s, ts, p, dir, RAY_TMIN, RAY_TMAX);
          if (ray_active) {
            s.any = !capable;
            ++walked;
          } else {
            emit_pass = false;
          }
          pending = !ray_active;  // nothing to traverse: a miss
        }
      }
    }
    if (trav_step_warp<COUNT>(ray_active, s, ts, stack, visits, tests, &b.ctrl->status, tp)) {
      ray_active = false;
      pending = true;
    }
  }
  warp_add64(&b.ctrl->rays_shadow, shadow);
  warp_add64(&b.ctrl->shadow_walked, walked);
  if (COUNT) {
    warp_add64(&b.ctrl->node_visits[1], visits);
    warp_add64(&b.ctrl->tri_tests[1], tests);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    b.ctrl->head[HEAD_TRACE] = 0;
    b.ctrl->nee_total += count;
  }
}

// Training records of guided vertices, in two halves so that the slot's
// atomic is in flight while the vertex is finished.  record_reserve keeps a
// vertex's record with probability 1 - drop (decided by a hash of slot,
// depth and the wave's salt, not by the path's stream; drop =
// ctrl->drop_prob, read once per launch), warp-aggregated over the lanes
// that call it, and returns the record index or ~0u; record_write fills it.
__device__ __forceinline__ uint32_t record_reserve(const WaveBufs& b, int depth, float drop, uint32_t slot,
                                                   bool want) {
  if (b.rec_cap == 0) return ~0u;  // a wave that does not train keeps no records
  const float u = (float)(tea<4>(slot * 16u + (uint32_t)depth, b.rec_salt) >> 8) * (1.0f / 16777216.0f);
  const bool keep = want && u >= drop;
  const uint32_t active = __activemask();
  const uint32_t mask = __ballot_sync(active, keep);
  if (!mask) return ~0u;
  const int leader = __ffs(mask) - 1;
  const int lane = threadIdx.x & 31;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&b.ctrl->rec_count, (uint32_t)__popc(mask));
  base = __shfl_sync(active, base, leader);
  const uint32_t k = base + __popc(mask & lanemask_lt());
  return keep && k < b.rec_cap ? k : ~0u;
}

__device__ __forceinline__ void record_write(const WaveBufs& b, uint32_t k, uint32_t slot, float flag, float4 r0,
                                             float4 r1, float4 r2, float4 r3, V3 c0) {
  if (k == ~0u) return;
  float4* rec = b.rec_list + 4ull * k;
  rec[0] = r0;
  rec[1] = r1;
  rec[2] = r2;
  rec[3] = r3;
  b.rec_col[k] = make_float4(c0.x, c0.y, c0.z, __uint_as_float((slot << 1) | (flag != 0.0f ? 1u : 0u)));
}

// ---------------------------------------------------------------------------
// Guided bounces, in the epilogue of the guide's inference (k_guided_infer):
// thread t holds the 40 network outputs of emitter-queue entry i in
// registers and finishes that vertex, so the outputs never reach HBM.
//
// Reference estimator: the opaque vertices with roughness 1, whose bounce
// k_nee deferred until the guide had seen the emitter flag its search left,
// with a training record per vertex (the radiance later gathered along the
// new direction, over the throughput after the bounce, is the incident
// radiance).  Returns whether a continuation ray (p, nd) is wanted.
__device__ __forceinline__ bool guided_compat_vertex(const WaveBufs& b, int depth, float drop, uint32_t i,
                                                     const float* o, V3& p, V3& nd, uint32_t& slot, uint32_t& scene,
                                                     uint32_t& guided_n) {
  const float4 a4 = b.nee_a[i], b4 = b.nee_b[i], c4 = b.nee_c[i];
  slot = __float_as_uint(a4.w);
  scene = __float_as_uint(c4.w);
  const SceneDev& sc = b.scenes[scene];
  if (sc.mats[__float_as_int(b4.w)].roughness != 1.0f) return false;  // bounced in k_nee
  const uint32_t rk = record_reserve(b, depth, drop, slot, true);
  const float4 cw = b.ps_col[slot];
  p = ld3(a4);
  const V3 N = ld3(b4);
  const V3 D = ld3(c4);
  uint32_t seed = b.ps_rng[slot];
  const float4 at = b.ps_att[slot];
  const int stale = __float_as_int(at.w);
  float weight;
  nd = guided_bounce(o, N, seed, b.bsdf_fraction, weight);
  const V3 att = ld3(at) * weight;
  const float il = rsqrtf(fmaxf(dot(D, D), 1e-30f));
  record_write(b, rk, slot, stale >= 0 ? 1.0f : 0.0f, make_float4(p.x, p.y, p.z, weight),
              make_float4(N.x, N.y, N.z, nd.x), make_float4(-D.x * il, -D.y * il, -D.z * il, nd.y),
              make_float4(att.x, att.y, att.z, nd.z), ld3(cw));
  b.ps_rng[slot] = seed;
  b.ps_att[slot] = make_float4(att.x, att.y, att.z, at.w);
  ++guided_n;
  return depth + 1 < (int)sc.num_bounces && weight > 0.0f;
}

// ---------------------------------------------------------------------------
// physically based estimator at opaque vertices (opt-in; no reference
// counterpart).  Emitter sampling: one shadow ray toward a point of an
// emitter picked by area x luminance (two-sided emitters), weighted against
// the bounce's density by the power heuristic.  Bounce: the diffuse lobe
// with probability = roughness (cosine-weighted), else a mirror; the
// throughput keeps the albedo applied by k_shade.  ps_att.w carries the
// solid-angle density of the last diffuse bounce (0 after a camera ray or a
// specular event) for the weight at an emitter hit (k_shade<true>).
//
// Plain mode finishes each vertex here.  Guided mode (SPLIT) only traces the
// shadow ray and leaves (direction, density, cosine, emitter material,
// visibility) in nee_light; k_guided_infer weighs it with the guide's density
// and draws the bounce once the guide's inference has run.

template <bool COUNT, bool SPLIT>
__global__ void __launch_bounds__(128, LISA_NEE_PB_MIN_BLOCKS) k_nee_pb(WaveBufs b, int depth) {
  const int q = depth & 1;
  const uint32_t count = *(volatile uint32_t*)&b.ctrl->nee_count;
  const int lane = threadIdx.x & 31;
  const uint32_t lt = lanemask_lt();
  uint2 stack[TRAV_STACK];
  TravState s;
  TraceScene ts;
  const SceneDev* sc = nullptr;
  bool have = false, exhausted = false, ray_active = false, pending = false, shadow = false;
  uint32_t entry = 0, slot = 0, seed = 0;
  int mat_idx = 0, em_m = 0;
  V3 Ns = v3(0.0f), wi = v3(0.0f);  // the vertex position lives in s.r.o*
  float pl = 0.0f, cos_x = 0.0f;
  s.r.ox = s.r.oy = s.r.oz = 0.0f;
  uint32_t nshadow = 0, visits = 0, tests = 0;
  __shared__ TriPass tri_pass[4];
  TriPass& tp = tri_pass[threadIdx.x >> 5];
  while (true) {
    const uint32_t busy = __ballot_sync(FULL, ray_active);
    if (__popc(busy) <= (int)b.refill_busy_max) {
      bool want_ray = false;
      V3 nd = v3(0.0f);
      if (pending) {
        pending = false;
        const bool lit = shadow && s.best_prim < 0;
        if (SPLIT) {
          b.nee_light[2ull * entry] = make_float4(wi.x, wi.y, wi.z, pl);
          b.nee_light[2ull * entry + 1] = make_float4(cos_x, __int_as_float(em_m), lit ? 1.0f : 0.0f, 0.0f);
          b.ps_rng[slot] = seed;
        } else {
          const DevMaterial& m = sc->mats[mat_idx];
          const float r = m.roughness;
          const float4 at = b.ps_att[slot];
          const V3 att = ld3(at);
          if (lit) {
            const DevMaterial& em = sc->mats[em_m];
            const float fcos = fmul(r, fdiv(cos_x, PI_F));
            // power heuristic against the bounce (traced at every vertex, the
            // last one's for the emission it reaches only)
            const float wl = fdiv(fmul(pl, pl), fadd(fmul(pl, pl), fmul(fcos, fcos)));
            const float4 c = b.ps_col[slot];
            const V3 col =
                ld3(c) + ((att * v3(em.emission[0], em.emission[1], em.emission[2])) * fdiv(fcos, pl)) * wl;
            b.ps_col[slot] = make_float4(col.x, col.y, col.z, c.w);
          }
          float prev = 0.0f;
          if (r >= 1.0f || (r > 0.0f && rnd(seed) < r)) {
            nd = cosine_dir(Ns, seed);
            prev = fmul(r, fdiv(dot(Ns, nd), PI_F));
          } else {
            nd = reflect(ld3(b.nee_c[entry]), Ns);
          }
          want_ray = !is_zero(nd);
          if (want_ray && depth + 1 == (int)sc->num_bounces)
            want_ray = final_ray_wanted(*sc, v3(s.r.ox, s.r.oy, s.r.oz), nd);
          b.ps_rng[slot] = seed;
          b.ps_att[slot] = make_float4(att.x, att.y, att.z, prev);
        }
        have = false;
      }
      const uint32_t ri = warp_reserve(&b.ctrl->qcount[q ^ 1], want_ray);
      if (want_ray && queue_fits(b, ri)) {
        b.ro[q ^ 1][ri] = make_float4(s.r.ox, s.r.oy, s.r.oz, __uint_as_float(slot));
        b.rd[q ^ 1][ri] = make_float4(nd.x, nd.y, nd.z, __uint_as_float((uint32_t)(sc - b.scenes)));
      }
      const bool need = !have && !exhausted;
      const uint32_t nmask = __ballot_sync(FULL, need);
      if (nmask) {
        const int leader = __ffs(nmask) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&b.ctrl->head[HEAD_NEE], (uint32_t)__popc(nmask));
        base = __shfl_sync(FULL, base, leader);
        if (need) {
          entry = base + __popc(nmask & lt);
          if (entry < count) {
            const float4 a4 = b.nee_a[entry], b4 = b.nee_b[entry];
            const V3 p = ld3(a4);
            s.r.ox = p.x;
            s.r.oy = p.y;
            s.r.oz = p.z;
            slot = __float_as_uint(a4.w);
            const V3 N = ld3(b4);
            mat_idx = __float_as_int(b4.w);
            seed = b.ps_rng[slot];
            const float4 c4 = b.nee_c[entry];
            sc = b.scenes + __float_as_uint(c4.w);
            ts = trace_scene(*sc);
            Ns = dot(N, ld3(c4)) < 0.0f ? N : -N;  // faces the incoming ray
            have = true;
            shadow = false;
            wi = v3(0.0f);
            pl = cos_x = 0.0f;
            em_m = 0;
            if (sc->mats[mat_idx].roughness > 0.0f && sc->num_emit > 0) {
              V3 y;
              const uint32_t k = sample_emitter(*sc, seed, y);
              const V3 w = y - p;
              const float d2 = dot(w, w);
              const float dist = fsqrt(d2);
              wi = w * fdiv(1.0f, dist);
              cos_x = dot(Ns, wi);
              const float cos_y = fabsf(dot(ld3(__ldg(sc->emit + 4ull * k + 3)), wi));
              if (cos_x > 0.0f && cos_y > 0.0f && dist > 0.0f) {
                pl = fdiv(fmul(__ldg(sc->emit + 4ull * k).w, d2), cos_y);
                em_m = __float_as_int(__ldg(sc->emit + 4ull * k + 1).w);
                shadow = true;
                ++nshadow;
                // stop short of the emitter itself; any blocker will do
                ray_active = trav_begin(s, ts, p, wi, RAY_TMIN, fmul(dist, 0.9990234375f), true);
              }
            }
            pending = !ray_active;  // no shadow ray, or nothing to traverse
          } else {
            exhausted = true;
          }
        }
      }
      if (!__any_sync(FULL, have)) break;
    }
    if (trav_step_warp<COUNT>(ray_active, s, ts, stack, visits, tests, &b.ctrl->status, tp)) {
      ray_active = false;
      pending = true;
    }
  }
  warp_add64(&b.ctrl->rays_shadow, nshadow);
  warp_add64(&b.ctrl->shadow_walked, nshadow);  // every shadow ray of this estimator is traced
  if (COUNT) {
    warp_add64(&b.ctrl->node_visits[1], visits);
    warp_add64(&b.ctrl->tri_tests[1], tests);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    b.ctrl->head[HEAD_TRACE] = 0;
    b.ctrl->nee_total += count;
  }
}

// Physically based estimator: the emitter sample of k_nee_pb weighed
// against the guided density, then the bounce -- the diffuse lobe by
// one-sample MIS between cosine sampling (probability c) and the guide's
// mixture, q = c cos/pi + (1-c) q_guide, throughput x (cos/pi) / q -- with a
// training record per diffuse bounce.
__device__ __forceinline__ bool guided_pb_vertex(const WaveBufs& b, int depth, float drop, uint32_t i, const float* o,
                                                 V3& p, V3& nd, uint32_t& slot, uint32_t& scene, uint32_t& guided_n) {
  const float c = b.bsdf_fraction;
  const float4 a4 = b.nee_a[i], b4 = b.nee_b[i], c4 = b.nee_c[i];
  p = ld3(a4);
  slot = __float_as_uint(a4.w);
  scene = __float_as_uint(c4.w);
  const V3 N = ld3(b4);
  const V3 D = ld3(c4);
  const V3 Ns = dot(N, D) < 0.0f ? N : -N;
  const float4 cw = b.ps_col[slot];
  const SceneDev& sc = b.scenes[scene];
  const float r = sc.mats[__float_as_int(b4.w)].roughness;
  V3 att = ld3(b.ps_att[slot]);
  V3 col = ld3(cw);
  uint32_t seed = b.ps_rng[slot];
  // the lobe choice is the stream's first draw at this vertex, as when the
  // bounce is drawn in k_nee_pb; decided first so that the training
  // record's slot is reserved while the mixture is evaluated
  const bool diffuse = r >= 1.0f || (r > 0.0f && rnd(seed) < r);
  const uint32_t rk = record_reserve(b, depth, drop, slot, diffuse);
  guide::Lobe L[guide::LOBES];
  guide::decode(o, L);
  const float4 l0 = b.nee_light[2ull * i], l1 = b.nee_light[2ull * i + 1];
  if (l1.z != 0.0f) {
    const float pl = l0.w, cos_x = l1.x;
    const DevMaterial& em = sc.mats[__float_as_int(l1.y)];
    // (fast reciprocals: the guided bounce's densities need no bit-exact
    // agreement with the oracle, only the same values for sampling and weight)
    const float fcos = r * cos_x * (1.0f / PI_F);
    const float pb = r * (c * (cos_x * (1.0f / PI_F)) + (1.0f - c) * guide::mix_pdf(L, l0.x, l0.y, l0.z));
    const float wl = __fdividef(pl * pl, pl * pl + pb * pb);
    col = col + ((att * v3(em.emission[0], em.emission[1], em.emission[2])) * __fdividef(fcos, pl)) * wl;
  }
  float prev = 0.0f;
  bool want;
  if (diffuse) {
    if (rnd(seed) < c) {
      nd = cosine_dir(Ns, seed);
    } else {
      const float u0 = rnd(seed), u1 = rnd(seed), u2 = rnd(seed);
      guide::mix_sample(L, u0, u1, u2, nd.x, nd.y, nd.z);
    }
    const float cs = dot(Ns, nd);
    const float pc = cs > 0.0f ? cs * (1.0f / PI_F) : 0.0f;
    const float qm = c * pc + (1.0f - c) * guide::mix_pdf(L, nd.x, nd.y, nd.z);
    const float weight = (pc > 0.0f && qm > 0.0f && isfinite(qm)) ? __fdividef(pc, qm) : 0.0f;
    att = att * weight;
    prev = r * qm;
    want = weight > 0.0f;
    const float il = rsqrtf(fmaxf(dot(D, D), 1e-30f));
    record_write(b, rk, slot, 0.0f, make_float4(p.x, p.y, p.z, weight), make_float4(N.x, N.y, N.z, nd.x),
                make_float4(-D.x * il, -D.y * il, -D.z * il, nd.y), make_float4(att.x, att.y, att.z, nd.z), col);
    ++guided_n;
  } else {
    nd = reflect(D, Ns);
    want = true;
  }
  if (want && depth + 1 == (int)sc.num_bounces) want = final_ray_wanted(sc, p, nd);
  b.ps_col[slot] = make_float4(col.x, col.y, col.z, cw.w);
  b.ps_rng[slot] = seed;
  b.ps_att[slot] = make_float4(att.x, att.y, att.z, prev);
  return want;
}

// The guide's inference on the emitter queue of this depth, fused with the
// guided bounces of those vertices (tensor-core layers, guide_infer.cuh;
// bounce in the last layer's epilogue).
template <bool PHYS>
__global__ void __launch_bounds__(INFER_THREADS, INFER_BLOCKS_PER_SM) k_guided_infer(const uint16_t* __restrict__ pack,
                                                                           const float* __restrict__ master,
                                                                           GuideSrc src, uint32_t* status, WaveBufs b,
                                                                           int depth) {
  const int q = depth & 1;
  uint32_t guided_n = 0;
  const float drop = b.ctrl->drop_prob;  // written by the last wave's record collection
  // the path state and emitter sample that the guided bounce reads, brought
  // into L2 while the five layers run
  auto pre = [&](uint32_t i) {
    const uint32_t slot = __float_as_uint(b.nee_a[i].w);
    prefetch_l2(b.ps_col + slot);
    prefetch_l2(b.ps_rng + slot);
    if (PHYS) {
      prefetch_l2(b.ps_att + slot);  // (the reference estimator's flag feature has loaded it)
      prefetch_l2(b.nee_light + 2ull * i);
    }
  };
  infer_tiles<SRC_NEE>(pack, master, src, status, pre, [&](uint32_t i, bool valid, const float* o) {
    bool want = false;
    V3 p = v3(0.0f), nd = v3(0.0f);
    uint32_t slot = 0, scene = 0;
    if (valid) {
      if (PHYS) want = guided_pb_vertex(b, depth, drop, i, o, p, nd, slot, scene, guided_n);
      else want = guided_compat_vertex(b, depth, drop, i, o, p, nd, slot, scene, guided_n);
    }
    const uint32_t ri = warp_reserve(&b.ctrl->qcount[q ^ 1], want);
    if (want && queue_fits(b, ri)) {
      b.ro[q ^ 1][ri] = make_float4(p.x, p.y, p.z, __uint_as_float(slot));
      b.rd[q ^ 1][ri] = make_float4(nd.x, nd.y, nd.z, __uint_as_float(scene));
    }
  });
  warp_add32(&b.ctrl->guided_count, guided_n);
  if (blockIdx.x == 0 && threadIdx.x == 0) b.ctrl->infer_rows += *(volatile uint32_t*)&b.ctrl->nee_count;
}

// ---------------------------------------------------------------------------
// accumulate: per pixel, the wave's samples in sample order

__global__ void k_accumulate(WaveBufs b, const WaveDesc* __restrict__ wave) {
  const WaveDesc& w = *wave;
  for (uint32_t item = blockIdx.x * blockDim.x + threadIdx.x; item < w.acc_items; item += gridDim.x * blockDim.x) {
    const WaveGroup& g = w.groups[find_group(w, item, true)];
    const SceneDev& sc = b.scenes[g.scene];
    const uint32_t pix = g.pix0 + (item - g.acc0);
    float4 s = sc.acc_sum[pix], c = sc.acc_comp[pix];
    double* sq = sc.acc_sq + 3ull * pix;
    double q0 = sq[0], q1 = sq[1], q2 = sq[2];
    double m0 = 0, m1 = 0, m2 = 0;
    if (sc.acc_sum64) {
      m0 = sc.acc_sum64[3ull * pix];
      m1 = sc.acc_sum64[3ull * pix + 1];
      m2 = sc.acc_sum64[3ull * pix + 2];
    }
    uint32_t last_slot = 0;
    for (uint32_t m = 0; m < g.nplanes; ++m) {
      const uint32_t slot = g.slot0 + m * g.npix + (pix - g.pix0);
      last_slot = slot;
      const float4 v = b.ps_col[slot];
      // Kahan: y = v - c; t = s + y; c = (t - s) - y; s = t
      float y, t;
      y = fsub(v.x, c.x); t = fadd(s.x, y); c.x = fsub(fsub(t, s.x), y); s.x = t;
      y = fsub(v.y, c.y); t = fadd(s.y, y); c.y = fsub(fsub(t, s.y), y); s.y = t;
      y = fsub(v.z, c.z); t = fadd(s.z, y); c.z = fsub(fsub(t, s.z), y); s.z = t;
      q0 = __dadd_rn(q0, __dmul_rn((double)v.x, (double)v.x));
      q1 = __dadd_rn(q1, __dmul_rn((double)v.y, (double)v.y));
      q2 = __dadd_rn(q2, __dmul_rn((double)v.z, (double)v.z));
      if (sc.acc_sum64) {
        m0 = __dadd_rn(m0, (double)v.x);
        m1 = __dadd_rn(m1, (double)v.y);
        m2 = __dadd_rn(m2, (double)v.z);
      }
    }
    sc.acc_sum[pix] = s;
    sc.acc_comp[pix] = c;
    sq[0] = q0;
    sq[1] = q1;
    sq[2] = q2;
    if (sc.acc_sum64) {
      sc.acc_sum64[3ull * pix] = m0;
      sc.acc_sum64[3ull * pix + 1] = m1;
      sc.acc_sum64[3ull * pix + 2] = m2;
    }
    if (w.rng_mode == LISA_RNG_PER_PIXEL) sc.pix_rng[pix] = b.ps_rng[last_slot];
  }
}

// ---------------------------------------------------------------------------
// guide training samples from the wave's kept records
//
// Each record holds the radiance the path had gathered when the vertex was
// left (c0) and the throughput after its bounce (a1); with the path's final
// radiance c, the radiance that arrived along the sampled direction is
// L = (c - c0) / a1.  The training weight is mean(L) * p_bsdf / q, the
// importance weight of the Neural Importance Sampling loss; records with
// weight 0 carry no gradient and are skipped.  At most `cap` samples go to
// the batch.  The keep probability of the next wave's records is set from
// this wave's guided-vertex count, aiming at 90 % of the record capacity.

__global__ void k_guide_collect(WaveBufs b, float4* __restrict__ batch, uint32_t cap) {
  const uint32_t total = *(volatile uint32_t*)&b.ctrl->guided_count;
  const uint32_t nrec = min(*(volatile uint32_t*)&b.ctrl->rec_count, b.rec_cap);
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t end = (nrec + 31u) & ~31u;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < end; k += stride) {
    bool want = false;
    float4 r0, r1, r2, r3, r4;
    float wt = 0.0f;
    if (k < nrec) {
      r4 = b.rec_col[k];
      const float4 col = b.ps_col[__float_as_uint(r4.w) >> 1];
      // no channel gained radiance after the vertex: every term below is
      // <= 0 (or not a number), so the record is not wanted -- its other
      // four float4 are not read
      if (col.x > r4.x || col.y > r4.y || col.z > r4.z) {
        const float4* rec = b.rec_list + 4ull * k;
        r0 = rec[0];
        r1 = rec[1];
        r2 = rec[2];
        r3 = rec[3];
        float l = 0.0f;
        int nl = 0;
        if (r3.x > 0.0f) { l += (col.x - r4.x) / r3.x; ++nl; }
        if (r3.y > 0.0f) { l += (col.y - r4.y) / r3.y; ++nl; }
        if (r3.z > 0.0f) { l += (col.z - r4.z) / r3.z; ++nl; }
        wt = nl ? l / (float)nl * r0.w : 0.0f;
        want = wt > 0.0f && isfinite(wt);
      }
    }
    const uint32_t i = warp_reserve(&b.ctrl->train_count, want);
    if (want && i < cap) {
      float4* o = batch + 4ull * i;
      o[0] = make_float4(r0.x, r0.y, r0.z, r1.x);
      o[1] = make_float4(r1.y, r1.z, r2.x, r2.y);
      o[2] = make_float4(r2.z, r1.w, r2.w, r3.w);
      o[3] = make_float4(fminf(wt, 1e4f), (float)(__float_as_uint(r4.w) & 1u), 0.0f, 0.0f);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const float keep = total ? fminf(1.0f, 0.9f * (float)b.rec_cap / (float)total) : 1.0f;
    b.ctrl->drop_prob = 1.0f - keep;
  }
}

__global__ void k_init_pixrng(uint32_t* rng, uint32_t npix, uint32_t subframe) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x)
    rng[p] = tea<16>(p, subframe);  // shader.cu:141
}

// ---------------------------------------------------------------------------
// tone map (src/cuda/helpers.h:35-62) and the PPM payload
// (src/sutil/sutil.cpp:533-553: rows flipped, alpha dropped)

__device__ __forceinline__ unsigned char quantize8(float x) {
  x = clampf(x, 0.0f, 1.0f);
  return (unsigned char)min((unsigned)(x * 256.0f), 255u);
}
__device__ __forceinline__ float to_srgb(float c) {
  const float inv_gamma = 1.0f / 2.4f;
  return c < 0.0031308f ? fmul(12.92f, c) : fsub(fmul(1.055f, powf(c, inv_gamma)), 0.055f);
}

__global__ void k_tonemap(const float4* __restrict__ sum, uint32_t npix, float inv_n, uint32_t width,
                          uint32_t height, float* rgb32, uchar4* rgba8, unsigned char* ppm) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    const float4 s = sum[p];
    const float r = fmul(s.x, inv_n), g = fmul(s.y, inv_n), bl = fmul(s.z, inv_n);
    if (rgb32) {
      rgb32[3ull * p] = r;
      rgb32[3ull * p + 1] = g;
      rgb32[3ull * p + 2] = bl;
    }
    const unsigned char R = quantize8(to_srgb(clampf(r, 0.0f, 1.0f)));
    const unsigned char G = quantize8(to_srgb(clampf(g, 0.0f, 1.0f)));
    const unsigned char B = quantize8(to_srgb(clampf(bl, 0.0f, 1.0f)));
    if (rgba8) rgba8[p] = make_uchar4(R, G, B, 255);
    if (ppm) {
      const uint32_t x = p % width, y = p / width;
      const uint64_t o = 3ull * ((uint64_t)(height - 1 - y) * width + x);
      ppm[o] = R;
      ppm[o + 1] = G;
      ppm[o + 2] = B;
    }
  }
}

// ---------------------------------------------------------------------------
// traversal hooks: closest hit / brute force / counting pass of given rays

template <bool COUNT>
__global__ void __launch_bounds__(128) k_trace_rays(const SceneDev* __restrict__ scd, const float* __restrict__ rays,
                                                   uint32_t n, int32_t* prim, float* tout, WaveCtrl* ctrl) {
  // the same warp-wide traversal step as the wavefront kernels (whole
  // warps run each round: `total` is a multiple of 32, as is the stride)
  uint32_t visits = 0, tests = 0;
  __shared__ TriPass tri_pass[4];
  TriPass& tp = tri_pass[threadIdx.x >> 5];
  uint2 stack[TRAV_STACK];
  const TraceScene ts = trace_scene(*scd);
  const uint32_t total = ((n + 31) / 32) * 32;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    TravState s;
    bool active = false;
    if (i < n) {
      const float* r = rays + 8ull * i;
      active = trav_begin(s, ts, v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6]), r[3], r[7]);
    }
    while (__any_sync(FULL, active))
      if (trav_step_warp<COUNT>(active, s, ts, stack, visits, tests, &ctrl->status, tp)) active = false;
    if (i < n) {
      if (prim) prim[i] = s.best_prim;
      if (tout) tout[i] = s.best_prim >= 0 ? s.best_t : __int_as_float(0x7f800000);
    }
  }
  if (COUNT) {
    warp_add64(&ctrl->node_visits[0], visits);
    warp_add64(&ctrl->tri_tests[0], tests);
  }
}

__global__ void k_brute_rays(const SceneDev* __restrict__ scd, const float* __restrict__ rays, uint32_t n,
                             int32_t* prim, float* tout) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* r = rays + 8ull * i;
    int hp;
    float ht;
    brute_hit(*scd, v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6]), r[3], r[7], hp, ht);
    prim[i] = hp;
    tout[i] = ht;
  }
}

// ---------------------------------------------------------------------------
// host side

// Host view of one planned wave.
struct WaveLaunch {
  uint32_t bounces;  // depth of its deepest scene
  int scene;         // scene of its first group (the only one of a guided wave)
  bool guided;       // the guide samples this wave's bounces
  bool train;        // guided wave: train the guide after it
  bool warm;         // guided wave: warm-up, sample the BSDF only
  uint32_t steps;    // guided wave: Adam steps after it, in proportion to its paths
};

namespace {

// Guided mode guides the scenes with at least guide_min_spp samples per
// pixel, one scene per wave so one network runs its inference, each wave
// holding at most guide_spp_per_wave planes (or as many as make 1 Mi paths,
// for small images) so the guide trains in between; the other scenes are
// packed into plain waves after them.
bool scene_guided(const Renderer& r, uint32_t s) {
  return r.opts.mode == LISA_MODE_GUIDED && r.scenes[s].params.num_samples >= r.opts.guide_min_spp;
}

void plan_waves(Renderer& r, const std::vector<uint32_t>& spp, const std::vector<uint64_t>& sample_base,
                std::vector<WaveDesc>& waves, std::vector<WaveLaunch>& wave_launch) {
  const uint32_t W = r.capacity;
  const bool per_pixel = r.opts.rng == LISA_RNG_PER_PIXEL;
  waves.clear();
  wave_launch.clear();
  WaveDesc cur;
  std::memset(&cur, 0, sizeof(cur));
  uint32_t cur_b = 0;
  bool cur_guided = false;
  auto close = [&]() {
    if (cur.num_groups == 0) return;
    cur.rng_mode = r.opts.rng;
    cur.seed = r.opts.seed;
    waves.push_back(cur);
    // guide_steps_per_wave steps per 4 Mi paths, at least one
    const uint32_t steps = cur_guided ? std::min<uint32_t>(r.guide_max_steps, std::max<uint32_t>(
                                            1u, (uint32_t)(((uint64_t)cur.paths * r.opts.guide_steps_per_wave +
                                                            (1ull << 21)) >> 22)))
                                      : 0u;
    wave_launch.push_back(WaveLaunch{cur_b, (int)cur.groups[0].scene, cur_guided, false, false, steps});
    std::memset(&cur, 0, sizeof(cur));
    cur_b = 0;
  };
  auto add = [&](uint32_t s, uint32_t pix0, uint32_t npix, uint32_t sample0, uint32_t k) {
    WaveGroup& g = cur.groups[cur.num_groups++];
    g.scene = s;
    g.pix0 = pix0;
    g.npix = npix;
    g.sample0 = sample0;
    g.nplanes = k;
    g.slot0 = cur.paths;
    g.acc0 = cur.acc_items;
    cur.paths += k * npix;
    cur.acc_items += npix;
    cur_b = std::max(cur_b, r.scenes[s].params.num_bounces);
  };
  for (int pass = 0; pass < 2; ++pass) {
    const bool one_scene = pass == 0;  // pass 0: guided scenes, pass 1: the rest
    cur_guided = one_scene;
    for (uint32_t s = 0; s < r.scenes.size(); ++s) {
      if (scene_guided(r, s) != one_scene) continue;
      const uint32_t npix = r.scenes[s].npix;
      const uint32_t max_planes =
          one_scene && r.opts.guide_spp_per_wave && npix
              ? std::max<uint32_t>(r.opts.guide_spp_per_wave, ((1u << 20) + npix - 1) / npix)
              : UINT32_MAX;
      uint32_t planes = spp[s];
      uint32_t j = (uint32_t)sample_base[s];
      if (npix == 0 || r.scenes[s].params.num_bounces == 0) continue;
      if (one_scene) close();
      bool scene_in_cur = false;
      while (planes > 0) {
        const uint32_t room = W - cur.paths;
        if (cur.num_groups == MAX_GROUPS || (per_pixel && scene_in_cur)) {
          close();
          scene_in_cur = false;
          continue;
        }
        if (npix <= room) {
          uint32_t k = std::min(std::min(planes, room / npix), max_planes);
          if (per_pixel) k = 1;
          add(s, 0, npix, j, k);
          scene_in_cur = true;
          planes -= k;
          j += k;
          if (one_scene) {
            close();
            scene_in_cur = false;
          }
        } else if (cur.paths == 0) {
          for (uint32_t p0 = 0; p0 < npix; p0 += W) {
            add(s, p0, std::min(W, npix - p0), j, 1);
            close();
          }
          planes -= 1;
          j += 1;
          scene_in_cur = false;
        } else {
          close();
          scene_in_cur = false;
        }
      }
    }
    close();
  }
}

WaveBufs make_bufs(Renderer& r) {
  WaveBufs b;
  std::memset(&b, 0, sizeof(b));
  b.ro[0] = r.ro[0];
  b.ro[1] = r.ro[1];
  b.rd[0] = r.rd[0];
  b.rd[1] = r.rd[1];
  b.hit = r.hit;
  b.ps_att = r.ps_att;
  b.ps_col = r.ps_col;
  b.ps_rng = r.ps_rng;
  b.nee_a = r.nee_a;
  b.nee_b = r.nee_b;
  b.nee_c = r.nee_c;
  b.ctrl = r.ctrl;
  b.scenes = r.d_scenes;
  b.capacity = r.capacity;
  b.refill_busy_max = 32u - (r.opts.refill_idle ? std::min<uint32_t>(r.opts.refill_idle, 32u) : LISA_REFILL_IDLE);
  b.physical = r.opts.estimator == LISA_ESTIMATOR_PHYSICAL;
  b.rec_list = r.rec_list;
  b.rec_col = r.rec_list ? r.rec_list + 4ull * r.rec_cap : nullptr;
  b.rec_cap = r.rec_cap;
  b.nee_light = r.nee_light;
  b.bsdf_fraction = r.opts.guide_bsdf_fraction;
  return b;
}

struct StageTimer {
  Renderer& r;
  bool on;
  bool capturing = false;  // inside stream capture: record external event nodes
  size_t next = 0;
  std::vector<std::pair<int, std::pair<size_t, size_t>>> marks;  // stage, (start ev, end ev)
  explicit StageTimer(Renderer& rr, bool enable) : r(rr), on(enable) {}
  Status ev(size_t* idx) {
    if (next >= r.ev_pool.size()) {
      cudaEvent_t e;
      LISA_CUDA(cudaEventCreate(&e));
      r.ev_pool.push_back(e);
    }
    *idx = next++;
    if (capturing)
      LISA_CUDA(cudaEventRecordWithFlags(r.ev_pool[*idx], r.stream, cudaEventRecordExternal));
    else
      LISA_CUDA(cudaEventRecord(r.ev_pool[*idx], r.stream));
    return Status();
  }
};

}  // namespace

// Dynamic shared memory of the fused inference kernels.
Status guided_infer_setup() {
  LISA_CUDA(cudaFuncSetAttribute(k_guided_infer<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM));
  LISA_CUDA(cudaFuncSetAttribute(k_guided_infer<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, INFER_SMEM));
  return Status();
}

Status guide_collect(Renderer& r, int, uint32_t cap, cudaStream_t s) {
  WaveBufs b = make_bufs(r);
  k_guide_collect<<<r.sm_count * 8, 256, 0, s>>>(b, r.guide_batch, cap);
  LISA_CUDA(cudaGetLastError());
  return Status();
}

// Stage indices of the timer: 0 trace, 1 shade, 2 emitter search, 3 other,
// 4 guide inference, 5 guide training (sample collection, training, Adam).
Status launch_wave_sequence(Renderer& r, const std::vector<WaveLaunch>& waves, lisa_render_stats* st,
                            StageTimer* tm) {
  WaveBufs b = make_bufs(r);
  uint32_t launches[5] = {0, 0, 0, 0, 0};  // trace, shade, nee, guide, total
  auto stage = [&](int which, auto&& fn) -> Status {
    size_t e0 = 0, e1 = 0;
    if (tm && tm->on) LISA_TRY(tm->ev(&e0));
    LISA_TRY(fn());
    LISA_CUDA(cudaGetLastError());
    if (tm && tm->on) {
      LISA_TRY(tm->ev(&e1));
      tm->marks.push_back({which, {e0, e1}});
    }
    if (which < 3) launches[which]++;
    if (which == 4 || which == 5) launches[3]++;
    launches[4]++;
    return Status();
  };
  const int acc_blocks = r.sm_count * 8;
  const bool counting = r.opts.count_traversal != 0;
  const bool guided_mode = r.opts.mode == LISA_MODE_GUIDED;
  const bool physical = r.opts.estimator == LISA_ESTIMATOR_PHYSICAL;
  for (size_t wv = 0; wv < waves.size(); ++wv) {
    const WaveDesc* wd = r.d_waves + wv;
    GuideSrc infer_src, train_src;
    GuideNet* net = nullptr;
    const bool guided = guided_mode && waves[wv].guided;
    if (guided) {
      const SceneGpu& sg = r.scenes[waves[wv].scene];
      net = r.guides[sg.guide].get();
      std::memset(&infer_src, 0, sizeof(infer_src));
      infer_src.nee_a = r.nee_a;
      infer_src.nee_b = r.nee_b;
      infer_src.nee_c = r.nee_c;
      infer_src.ps_att = r.ps_att;
      infer_src.count = &r.ctrl->nee_count;
      infer_src.n = r.capacity;
      infer_src.no_flag = physical ? 1u : 0u;
      for (int k = 0; k < 3; ++k) {
        infer_src.bmin[k] = sg.bvh.bmin[k];
        infer_src.bmax[k] = sg.bvh.bmax[k];
      }
      train_src = infer_src;
      train_src.nee_a = train_src.nee_b = train_src.nee_c = nullptr;
      train_src.geom = r.guide_batch;
      train_src.count = &r.ctrl->train_count;
      train_src.n = r.guide_batch_cap;
    }
    LISA_TRY(stage(3, [&] {
      k_raygen<<<r.sm_count * 8, 256, 0, r.stream>>>(b, wd);
      return Status();
    }));
    // the physically based estimator traces one more ray per path, the one
    // leaving its last vertex, for the emission it reaches (no vertex)
    const uint32_t depths = waves[wv].bounces + (physical ? 1u : 0u);
    for (uint32_t d = 0; d < depths; ++d) {
      LISA_TRY(stage(0, [&] {
        if (counting) k_trace<true><<<r.trace_blocks, r.trace_threads, 0, r.stream>>>(b, (int)d);
        else k_trace<false><<<r.trace_blocks, r.trace_threads, 0, r.stream>>>(b, (int)d);
        return Status();
      }));
      LISA_TRY(stage(1, [&] {
        if (physical) k_shade<true><<<r.shade_blocks, r.shade_threads, 0, r.stream>>>(b, (int)d);
        else k_shade<false><<<r.shade_blocks, r.shade_threads, 0, r.stream>>>(b, (int)d);
        return Status();
      }));
      if (d == waves[wv].bounces) break;  // the emission-only depth has no vertices
      // the guide draws the bounces of the first guide_max_depth vertices
      // of a path (0 = all); deeper ones sample the BSDF (and, with the
      // reference estimator, never the last one, whose bounce is not traced)
      const bool guided_d = guided && (physical || d + 1 < waves[wv].bounces) &&
                            (r.opts.guide_max_depth == 0 || d < r.opts.guide_max_depth);
      LISA_TRY(stage(2, [&] {
        const dim3 g(physical ? r.nee_pb_blocks : r.nee_blocks), t(r.nee_threads);
        if (physical) {
          if (guided_d) {
            if (counting) k_nee_pb<true, true><<<g, t, 0, r.stream>>>(b, (int)d);
            else k_nee_pb<false, true><<<g, t, 0, r.stream>>>(b, (int)d);
          } else {
            if (counting) k_nee_pb<true, false><<<g, t, 0, r.stream>>>(b, (int)d);
            else k_nee_pb<false, false><<<g, t, 0, r.stream>>>(b, (int)d);
          }
        } else if (guided_d) {
          if (counting) k_nee<true, true><<<g, t, 0, r.stream>>>(b, (int)d);
          else k_nee<false, true><<<g, t, 0, r.stream>>>(b, (int)d);
        } else {
          if (counting) k_nee<true><<<g, t, 0, r.stream>>>(b, (int)d);
          else k_nee<false><<<g, t, 0, r.stream>>>(b, (int)d);
        }
        return Status();
      }));
      if (guided_d) {
        LISA_TRY(stage(4, [&] {
          WaveBufs bw = b;  // warm-up waves sample the BSDF only (c = 1)
          if (waves[wv].warm) bw.bsdf_fraction = 1.0f;
          bw.rec_salt = (uint32_t)(r.guide_waves_done + wv) * 2654435761u + 17u;
          if (!waves[wv].train) bw.rec_cap = 0;
          const uint32_t grid = std::min<uint32_t>((r.capacity + 255) / 256, (uint32_t)(r.sm_count * INFER_BLOCKS_PER_SM));
          if (physical)
            k_guided_infer<true><<<grid, INFER_THREADS, INFER_SMEM, r.stream>>>(net->w_bf16, net->master, infer_src, net->status,
                                                                       bw, (int)d);
          else
            k_guided_infer<false><<<grid, INFER_THREADS, INFER_SMEM, r.stream>>>(net->w_bf16, net->master, infer_src, net->status,
                                                                        bw, (int)d);
          return Status();
        }));
      }
    }
    LISA_TRY(stage(3, [&] {
      k_accumulate<<<acc_blocks, 256, 0, r.stream>>>(b, wd);
      return Status();
    }));
    if (guided && waves[wv].train) {
      const uint32_t steps = waves[wv].steps;
      LISA_TRY(stage(5, [&] { return guide_collect(r, (int)wv, steps * r.guide_chunk, r.stream); }));
      // one Adam step per slice of the collected samples, all in one
      // cooperative launch
      LISA_TRY(stage(5, [&] {
        return guide_launch_train_rounds(*net, train_src, SRC_GEOM, r.guide_chunk, steps, r.opts.guide_lr, r.guide_grid_bar,
                                         r.stream, &r.ctrl->train_samples);
      }));
    }
  }
  if (st) {
    st->launches_trace += launches[0];
    st->launches_shade += launches[1];
    st->launches_nee += launches[2];
    st->launches_guide += launches[3];
    st->launches_total += launches[4];
  }
  return Status();
}

Status renderer_render(Renderer& r, uint32_t spp_req, bool progressive, lisa_render_stats* st) {
  lisa_render_stats local;
  std::memset(&local, 0, sizeof(local));
  std::vector<uint32_t> spp(r.scenes.size());
  std::vector<uint64_t> base(r.scenes.size());
  for (size_t s = 0; s < r.scenes.size(); ++s) {
    spp[s] = progressive ? spp_req : r.scenes[s].params.num_samples;
    base[s] = r.scenes[s].next_sample;
  }
  std::vector<WaveDesc> waves;
  std::vector<WaveLaunch> wb;
  plan_waves(r, spp, base, waves, wb);
  const bool guided = r.opts.mode == LISA_MODE_GUIDED;
  // warm-up and training flags count the guided waves of each scene (its
  // guide); a scene's Adam steps stop at guide_train_steps
  std::vector<uint64_t> scene_waves(r.scenes.size(), 0), scene_steps(r.scenes.size(), 0);
  if (guided)
    for (size_t i = 0; i < wb.size(); ++i) {
      if (!wb[i].guided) continue;
      const int sc = wb[i].scene;
      const uint64_t k = r.scenes[sc].guide_waves_done + scene_waves[sc]++;
      const uint64_t done = r.scenes[sc].guide_steps_done + scene_steps[sc];
      if (r.opts.guide_train_steps)
        wb[i].steps = (uint32_t)std::min<uint64_t>(wb[i].steps, done < r.opts.guide_train_steps
                                                                    ? r.opts.guide_train_steps - done
                                                                    : 0);
      wb[i].train = (r.opts.guide_train_waves == 0 || k < r.opts.guide_train_waves) && wb[i].steps > 0;
      if (!wb[i].train) wb[i].steps = 0;
      scene_steps[sc] += wb[i].steps;
      wb[i].warm = k < r.opts.guide_warmup_waves;
    }
  if (waves.size() > r.wave_capacity) {
    if (r.d_waves) cudaFree(r.d_waves);
    r.d_waves = nullptr;
    LISA_CUDA(cudaMalloc(&r.d_waves, sizeof(WaveDesc) * waves.size()));
    r.wave_capacity = (uint32_t)waves.size();
  }
  if (!waves.empty())
    LISA_CUDA(cudaMemcpyAsync(r.d_waves, waves.data(), sizeof(WaveDesc) * waves.size(), cudaMemcpyHostToDevice,
                              r.stream));
  // reset ray counters
  LISA_CUDA(cudaMemsetAsync(r.ctrl, 0, sizeof(WaveCtrl), r.stream));
  if (r.opts.rng == LISA_RNG_PER_PIXEL) {
    for (auto& s : r.scenes) {
      const uint32_t subframe = progressive ? s.subframe : 0u;
      k_init_pixrng<<<r.sm_count * 4, 256, 0, r.stream>>>(s.pix_rng, s.npix, subframe);
    }
    LISA_CUDA(cudaGetLastError());
  }
  cudaEvent_t e0, e1;
  LISA_CUDA(cudaEventCreate(&e0));
  LISA_CUDA(cudaEventCreate(&e1));
  LISA_CUDA(cudaEventRecord(e0, r.stream));
  StageTimer tm(r, r.opts.stage_timing != 0);
  Status s;
  if (r.opts.use_graph && !wb.empty()) {
    // one graph per launch-sequence shape; the wave table it reads is
    // refreshed above, outside the graph
    std::vector<uint64_t> key;
    for (const WaveLaunch& w : wb)
      key.push_back(((uint64_t)w.steps << 40) | ((uint64_t)w.bounces << 32) | ((uint64_t)w.scene << 3) |
                    ((uint64_t)w.guided << 2) | ((uint64_t)w.warm << 1) | w.train);
    key.push_back(r.opts.count_traversal);
    key.push_back(r.opts.stage_timing);
    key.push_back((uint64_t)(uintptr_t)r.d_waves);
    if (key != r.graph_key || !r.graph_exec) {
      if (tm.on) {  // create the timing events before capture begins
        size_t need = 0;
        for (const WaveLaunch& w : wb) need += 2ull * (5ull * (w.bounces + 1) + 6 + 2ull * w.steps);
        while (r.ev_pool.size() < need) {
          cudaEvent_t e;
          LISA_CUDA(cudaEventCreate(&e));
          r.ev_pool.push_back(e);
        }
      }
      if (r.graph_exec) cudaGraphExecDestroy(r.graph_exec);
      r.graph_exec = nullptr;
      r.graph_key.clear();
      cudaGraph_t g = nullptr;
      LISA_CUDA(cudaStreamBeginCapture(r.stream, cudaStreamCaptureModeThreadLocal));
      lisa_render_stats counts;
      std::memset(&counts, 0, sizeof(counts));
      tm.capturing = true;
      s = launch_wave_sequence(r, wb, &counts, &tm);
      tm.capturing = false;
      const cudaError_t ce = cudaStreamEndCapture(r.stream, &g);
      if (s.ok() && ce != cudaSuccess) s = Status::cuda(ce, "cudaStreamEndCapture");
      if (s.ok()) {
        const cudaError_t ie = cudaGraphInstantiate(&r.graph_exec, g, 0);
        if (ie != cudaSuccess) s = Status::cuda(ie, "cudaGraphInstantiate");
      }
      if (g) cudaGraphDestroy(g);
      if (s.ok()) {
        r.graph_key = key;
        r.graph_marks = tm.marks;
        r.graph_launches[0] = counts.launches_trace;
        r.graph_launches[1] = counts.launches_shade;
        r.graph_launches[2] = counts.launches_nee;
        r.graph_launches[3] = counts.launches_total;
        r.graph_launches[4] = counts.launches_guide;
      }
    }
    if (s.ok()) {
      tm.marks = r.graph_marks;
      local.launches_trace = r.graph_launches[0];
      local.launches_shade = r.graph_launches[1];
      local.launches_nee = r.graph_launches[2];
      local.launches_total = r.graph_launches[3];
      local.launches_guide = r.graph_launches[4];
      const cudaError_t le = cudaGraphLaunch(r.graph_exec, r.stream);
      if (le != cudaSuccess) s = Status::cuda(le, "cudaGraphLaunch");
    }
  } else {
    s = launch_wave_sequence(r, wb, &local, &tm);
  }
  LISA_CUDA(cudaEventRecord(e1, r.stream));
  if (!s.ok()) {
    cudaStreamSynchronize(r.stream);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return s;
  }
  WaveCtrl hc;
  LISA_CUDA(cudaMemcpyAsync(&hc, r.ctrl, sizeof(hc), cudaMemcpyDeviceToHost, r.stream));
  LISA_CUDA(cudaStreamSynchronize(r.stream));
  float ms = 0.0f;
  LISA_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (tm.on) {
    for (auto& m : tm.marks) {
      float t = 0.0f;
      LISA_CUDA(cudaEventElapsedTime(&t, r.ev_pool[m.second.first], r.ev_pool[m.second.second]));
      if (m.first == 0) local.ms_trace += t;
      else if (m.first == 1) local.ms_shade += t;
      else if (m.first == 2) local.ms_nee += t;
      else if (m.first == 4) {
        local.ms_guide += t;
        local.ms_guide_infer += t;
      } else if (m.first == 5) {
        local.ms_guide += t;
        local.ms_guide_train += t;
      }
      else local.ms_other += t;
    }
  }
  for (size_t k = 0; k < r.scenes.size(); ++k) {
    r.scenes[k].samples_done += spp[k];
    r.scenes[k].next_sample += spp[k];
    if (progressive) r.scenes[k].subframe++;
  }
  if (guided) {
    r.guide_waves_done += wb.size();
    for (size_t k = 0; k < r.scenes.size(); ++k) {
      r.scenes[k].guide_waves_done += scene_waves[k];
      r.scenes[k].guide_steps_done += scene_steps[k];
    }
    for (auto& g : r.guides) LISA_TRY(guide_check_status(*g, r.stream));
    for (size_t k = wb.size(); k-- > 0;) {
      if (!wb[k].guided) continue;
      float l = 0.0f;  // loss of the last guided wave's scene
      LISA_CUDA(cudaMemcpy(&l, r.guides[r.scenes[wb[k].scene].guide]->loss_last, sizeof(float),
                           cudaMemcpyDeviceToHost));
      local.guide_loss = l;
      break;
    }
  }
  local.rays_primary = hc.rays_primary;
  local.rays_bounce = hc.rays_bounce;
  local.rays_shadow = hc.rays_shadow;
  local.paths = hc.rays_primary;
  local.samples_total = r.scenes.empty() ? 0 : r.scenes[0].samples_done;
  local.ms_device = ms;
  local.device_status = hc.status;
  local.nee_vertices = hc.nee_total;
  local.node_visits_trace = hc.node_visits[0];
  local.tri_tests_trace = hc.tri_tests[0];
  local.node_visits_nee = hc.node_visits[1];
  local.tri_tests_nee = hc.tri_tests[1];
  local.shadow_traversals = hc.shadow_walked;
  local.guide_infer_rows = hc.infer_rows;
  local.guide_train_samples = hc.train_samples;
  if (st) *st = local;
  if (hc.status) return Status(LISA_ERR_DEVICE, "device status word " + std::to_string(hc.status));
  return Status();
}

Status renderer_reset(Renderer& r) {
  for (auto& s : r.scenes) {
    LISA_CUDA(cudaMemsetAsync(s.acc_sum, 0, sizeof(float4) * s.npix, r.stream));
    LISA_CUDA(cudaMemsetAsync(s.acc_comp, 0, sizeof(float4) * s.npix, r.stream));
    LISA_CUDA(cudaMemsetAsync(s.acc_sq, 0, sizeof(double) * 3 * s.npix, r.stream));
    if (s.acc_sum64) LISA_CUDA(cudaMemsetAsync(s.acc_sum64, 0, sizeof(double) * 3 * s.npix, r.stream));
    s.samples_done = 0;
    s.next_sample = s.sample_offset;
    s.subframe = 0;
  }
  LISA_CUDA(cudaStreamSynchronize(r.stream));
  return Status();
}

Status renderer_get_image(Renderer& r, int scene, float* rgb32, uint8_t* rgba8, double* var, double* mean64) {
  if (scene < 0 || scene >= (int)r.scenes.size()) return Status::invalid("scene index out of range");
  SceneGpu& s = r.scenes[scene];
  const uint32_t npix = s.npix;
  const double n = (double)s.samples_done;
  float* d_rgb = nullptr;
  uchar4* d_rgba = nullptr;
  if (rgb32 || var) LISA_CUDA(dev_alloc((void**)&d_rgb, sizeof(float) * 3 * std::max<uint32_t>(npix, 1)));
  if (rgba8) LISA_CUDA(dev_alloc((void**)&d_rgba, sizeof(uchar4) * std::max<uint32_t>(npix, 1)));
  const float inv_n = n > 0 ? (float)(1.0 / n) : 0.0f;
  if (npix) {
    k_tonemap<<<r.sm_count * 4, 256, 0, r.stream>>>(s.acc_sum, npix, inv_n, s.params.width, s.params.height, d_rgb,
                                                     d_rgba, nullptr);
    LISA_CUDA(cudaGetLastError());
  }
  // the mean goes straight to the caller's buffer unless the FP64 figures
  // below need it on the host as well
  const bool direct = rgb32 && !var && !mean64;
  std::vector<float> h_rgb;
  if (d_rgb && direct) {
    LISA_CUDA(cudaMemcpyAsync(rgb32, d_rgb, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost, r.stream));
  } else if (d_rgb) {
    h_rgb.resize(3ull * npix);
    LISA_CUDA(cudaMemcpyAsync(h_rgb.data(), d_rgb, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost, r.stream));
  }
  if (rgba8) LISA_CUDA(cudaMemcpyAsync(rgba8, d_rgba, sizeof(uchar4) * npix, cudaMemcpyDeviceToHost, r.stream));
  std::vector<double> sq, m64;
  if (var) {
    sq.resize(3ull * npix);
    LISA_CUDA(cudaMemcpyAsync(sq.data(), s.acc_sq, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost, r.stream));
  }
  if ((mean64 || var) && s.acc_sum64) {
    m64.resize(3ull * npix);
    LISA_CUDA(
        cudaMemcpyAsync(m64.data(), s.acc_sum64, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost, r.stream));
  }
  LISA_CUDA(cudaStreamSynchronize(r.stream));
  dev_free(d_rgb);
  dev_free(d_rgba);
  // The mean is the float Kahan sum over n (mean of the samples); rgb32 row 0
  // is the bottom row like the reference accum_buffer.
  if (rgb32 && !direct) std::memcpy(rgb32, h_rgb.data(), sizeof(float) * 3 * npix);
  if (mean64) {
    if (s.acc_sum64) {
      for (size_t i = 0; i < 3ull * npix; ++i) mean64[i] = n > 0 ? m64[i] / n : 0.0;
    } else {
      for (size_t i = 0; i < 3ull * npix; ++i) mean64[i] = (double)h_rgb[i];
    }
  }
  if (var) {
    for (size_t i = 0; i < 3ull * npix; ++i) {
      const double mu = s.acc_sum64 ? (n > 0 ? m64[i] / n : 0.0) : (double)h_rgb[i];
      double v = n > 1 ? (sq[i] / n - mu * mu) * n / (n - 1.0) : 0.0;
      var[i] = v > 0 ? v : 0.0;
    }
  }
  return Status();
}

Status renderer_get_ppm(Renderer& r, int scene, uint8_t* rgb8) {
  if (scene < 0 || scene >= (int)r.scenes.size()) return Status::invalid("scene index out of range");
  SceneGpu& s = r.scenes[scene];
  const uint32_t npix = s.npix;
  if (npix == 0) return Status();
  unsigned char* d = nullptr;
  LISA_CUDA(dev_alloc((void**)&d, 3ull * npix));
  const float inv_n = s.samples_done > 0 ? (float)(1.0 / (double)s.samples_done) : 0.0f;
  k_tonemap<<<r.sm_count * 4, 256, 0, r.stream>>>(s.acc_sum, npix, inv_n, s.params.width, s.params.height, nullptr,
                                                   nullptr, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(rgb8, d, 3ull * npix, cudaMemcpyDeviceToHost, r.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(r.stream);
  else cudaStreamSynchronize(r.stream);
  dev_free(d);
  if (e != cudaSuccess) return Status::cuda(e, "ppm payload");
  return Status();
}

Status launch_trace_closest(const SceneDev* d_scene, WaveCtrl* d_ctrl, const float* d_rays, uint32_t n,
                            int32_t* d_prim, float* d_t, cudaStream_t s, int sm_count, bool brute) {
  if (n == 0) return Status();
  LISA_CUDA(cudaMemsetAsync(d_ctrl, 0, sizeof(WaveCtrl), s));
  const uint32_t blocks = std::min<uint32_t>((n + 127) / 128, (uint32_t)sm_count * 16);
  if (brute) {
    k_brute_rays<<<blocks, 128, 0, s>>>(d_scene, d_rays, n, d_prim, d_t);
  } else {
    k_trace_rays<false><<<blocks, 128, 0, s>>>(d_scene, d_rays, n, d_prim, d_t, d_ctrl);
  }
  LISA_CUDA(cudaGetLastError());
  uint32_t status = 0;
  LISA_CUDA(cudaMemcpyAsync(&status, &d_ctrl->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  LISA_CUDA(cudaStreamSynchronize(s));
  if (status) return Status(LISA_ERR_DEVICE, "device status word " + std::to_string(status));
  return Status();
}

Status trace_rays(Renderer& r, const float* d_rays, uint32_t n, int32_t* d_prim, float* d_t, cudaStream_t s,
                  bool brute) {
  if (r.scenes.empty()) return Status::invalid("renderer has no scene");
  return launch_trace_closest(r.d_scenes, r.ctrl, d_rays, n, d_prim, d_t, s, r.sm_count, brute);
}

Status trace_count(Renderer& r, const float* d_rays, uint32_t n, uint64_t* visits, uint64_t* tests) {
  LISA_CUDA(cudaMemsetAsync(r.ctrl, 0, sizeof(WaveCtrl), r.stream));
  if (n)
    k_trace_rays<true><<<std::min<uint32_t>((n + 127) / 128, r.sm_count * 16), 128, 0, r.stream>>>(
        r.d_scenes, d_rays, n, nullptr, nullptr, r.ctrl);
  LISA_CUDA(cudaGetLastError());
  WaveCtrl hc;
  LISA_CUDA(cudaMemcpyAsync(&hc, r.ctrl, sizeof(hc), cudaMemcpyDeviceToHost, r.stream));
  LISA_CUDA(cudaStreamSynchronize(r.stream));
  *visits = hc.node_visits[0];
  *tests = hc.tri_tests[0];
  return Status();
}

Status configure_launch(Renderer& r) {
  int occ = 0;
  const int tthreads = r.opts.threads_per_block ? (int)r.opts.threads_per_block : 128;
  LISA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_trace<false>, tthreads, 0));
  int bps = r.opts.blocks_per_sm ? (int)r.opts.blocks_per_sm : std::max(occ, 1);
  bps = std::min(bps, std::max(occ, 1));
  r.trace_threads = tthreads;
  r.trace_blocks = r.sm_count * bps;
  LISA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_nee<false>, tthreads, 0));
  bps = r.opts.blocks_per_sm ? (int)r.opts.blocks_per_sm : std::max(occ, 1);
  bps = std::min(bps, std::max(occ, 1));
  r.nee_threads = tthreads;
  r.nee_blocks = r.sm_count * bps;
  // the physically based emitter kernel has its own register budget
  LISA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_nee_pb<false, false>, tthreads, 0));
  bps = r.opts.blocks_per_sm ? (int)r.opts.blocks_per_sm : std::max(occ, 1);
  bps = std::min(bps, std::max(occ, 1));
  r.nee_pb_blocks = r.sm_count * bps;
  LISA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_shade<false>, 256, 0));
  r.shade_threads = 256;
  r.shade_blocks = r.sm_count * std::max(occ, 1);
  return Status();
}

}  // namespace lisa

// Sampling routines of the physically based estimator (an opt-in mode with
// no reference counterpart; the reference estimator is the default).
//
// Every float step is one IEEE rounding in a fixed order (device_math.cuh),
// and the oracle restates the same steps, so paths agree bit for bit.
#pragma once

#include "device_math.cuh"
#include "lisa_device.cuh"

namespace lisa {

constexpr float PI_F = 3.14159265358979323846f;

__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
  return v3(fsub(fmul(a.y, b.z), fmul(a.z, b.y)), fsub(fmul(a.z, b.x), fmul(a.x, b.z)),
            fsub(fmul(a.x, b.y), fmul(a.y, b.x)));
}

// Orthonormal basis around a unit vector (Duff, Burgess, Christensen, Hery,
// Kensler, Liani, Villemin, "Building an Orthonormal Basis, Revisited",
// JCGT 2017).
__device__ __forceinline__ void onb(V3 n, V3& t, V3& b) {
  const float sign = copysignf(1.0f, n.z);
  const float a = fdiv(-1.0f, fadd(sign, n.z));
  const float bb = fmul(fmul(n.x, n.y), a);
  t = v3(fadd(1.0f, fmul(fmul(fmul(sign, n.x), n.x), a)), fmul(sign, bb), -fmul(sign, n.x));
  b = v3(bb, fadd(sign, fmul(fmul(n.y, n.y), a)), -n.y);
}

// Cosine-weighted direction about the unit vector n (density cos / pi): a
// uniform point of the unit disk by rejection -- at most 16 pairs, then the
// centre -- lifted to the hemisphere (Malley's method).  No trigonometry, so
// the host restatement reproduces it exactly.
__device__ __forceinline__ V3 cosine_dir(V3 n, uint32_t& seed) {
  float x = 0.0f, y = 0.0f, r2 = 0.0f;
  for (int k = 0; k < 16; ++k) {
    x = rng11(seed);
    y = rng11(seed);
    r2 = fadd(fmul(x, x), fmul(y, y));
    if (r2 < 1.0f) break;
  }
  if (!(r2 < 1.0f)) x = y = r2 = 0.0f;
  const float z = fsqrt(fmaxf(0.0f, fsub(1.0f, r2)));
  V3 t, b;
  onb(n, t, b);
  return normalize((x * t + y * b) + z * n);
}

// A point y of an emitter chosen with probability area x luminance / total
// (first CDF entry above u0), uniform on the triangle.  Returns the emitter.
__device__ __forceinline__ uint32_t sample_emitter(const SceneDev& sc, uint32_t& seed, V3& y) {
  const float u0 = rnd(seed), u1 = rnd(seed), u2 = rnd(seed);
  uint32_t lo = 0, hi = sc.num_emit - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (u0 < __ldg(sc.emit_cdf + mid)) hi = mid;
    else lo = mid + 1;
  }
  const float4* e = sc.emit + 4ull * lo;
  const float a = fsqrt(u1);
  const float bu = fmul(a, fsub(1.0f, u2)), bv = fmul(a, u2);
  y = ld3(__ldg(e)) + (bu * ld3(__ldg(e + 1)) + bv * ld3(__ldg(e + 2)));
  return lo;
}

}  // namespace lisa

// Lambertian-with-roughness BSDF plug-in: the default of the interchangeable
// BSDF interface.
//
// A BSDF plug-in is a header that defines, in namespace lisa::bsdf,
//   V3    bounce(V3 ray_dir, V3 N, uint32_t& seed, const DevMaterial& m)
//   float BRDF(V3 N, V3 L, const DevMaterial& m)
//   float BTDF(float cosI, float eta)
// exactly the three functions LiSA's shader expects from a BSDF file
// (src/LiSA/src/bsdfs/lambertian.cu:7-27, included textually by
// src/LiSA/src/shader.cu:4).  The wavefront shading kernels include the
// header named by LISA_BSDF_HEADER (this one by default), so swapping the
// BSDF is a rebuild with -DLISA_BSDF_HEADER="bsdfs/other.cuh".
//
// Semantics follow the reference:
//   bounce = lerp(reflect(D, N), hemi(N), roughness), not renormalised;
//   BRDF   = NdotL * NdotL / pi with NdotL clamped to [0,1];
//   BTDF   = Schlick's Fresnel term with the incident cosine.
// The reference evaluates pow(x,2) and pow(x,5) with the math library; here
// they are repeated products, so the host oracle reproduces them exactly.
#pragma once

#include "../device_math.cuh"
#include "../lisa_device.cuh"

namespace lisa {
namespace bsdf {

// Uniform point of the cube [-1,1)^3, normalised, flipped into N's
// hemisphere (src/LiSA/src/maths.cu:10-15).  Draws x, then y, then z.
__device__ __forceinline__ V3 hemisphere_direction(V3 N, float x, float y, float z) {
  const V3 r = normalize(v3(x, y, z));
  return faceforward(r, N, r);
}
__device__ __forceinline__ V3 shoot_ray_hemisphere(V3 N, uint32_t& seed) {
  const float x = rng11(seed);
  const float y = rng11(seed);
  const float z = rng11(seed);
  return hemisphere_direction(N, x, y, z);
}

// Schlick (src/LiSA/src/maths.cu:17-20)
__device__ __forceinline__ float fresnel(float cosT, float eta) {
  const float r = fdiv(fsub(1.0f, eta), fadd(1.0f, eta));
  const float R0 = fmul(r, r);
  const float x = fsub(1.0f, cosT);
  const float x5 = fmul(fmul(fmul(fmul(x, x), x), x), x);
  return fadd(R0, fmul(fsub(1.0f, R0), x5));
}

// Refraction; the zero vector on total internal reflection
// (src/LiSA/src/maths.cu:22-30).
__device__ __forceinline__ V3 refract(float cosI, V3 d, V3 N, float eta) {
  const float cost2 = fsub(1.0f, fmul(fmul(eta, eta), fsub(1.0f, fmul(cosI, cosI))));
  const float k = fsub(fmul(eta, cosI), fsqrt(fabsf(cost2)));
  const V3 t = eta * d + k * N;
  return t * (cost2 > 0.0f ? 1.0f : 0.0f);
}

__device__ __forceinline__ V3 bounce(V3 ray_dir, V3 N, uint32_t& seed, const DevMaterial& m) {
  const V3 r = reflect(ray_dir, N);
  const V3 h = shoot_ray_hemisphere(N, seed);
  return lerp(r, h, m.roughness);
}

__device__ __forceinline__ float BRDF(V3 N, V3 L, const DevMaterial&) {
  const float NdotL = clampf(dot(N, L), 0.0f, 1.0f);
  const float sample_prob = fdiv(NdotL, 3.14159265358979323846f);
  return fmul(NdotL, sample_prob);
}

__device__ __forceinline__ float BTDF(float cosI, float eta) { return fresnel(cosI, eta); }

}  // namespace bsdf
}  // namespace lisa

// Device math for the estimator: float3 helpers whose every operation is a
// single IEEE-754 round-to-nearest step (__fadd_rn, __fmul_rn, ...), so the
// compiler never contracts a*b+c into an FMA.  The CPU oracle evaluates the
// same expressions in the same order with FP contraction off, which makes a
// path traced here and the same path traced on the host agree bit for bit.
//
// The vector helpers follow the semantics of the SDK helpers LiSA uses
// (src/sutil/vec_math.h: dot :521-524, cross :527-530, normalize :539-543
// as v * (1/sqrt(dot)), reflect :552-555, faceforward :561-564, lerp
// :494-497, clamp :509-512), the RNG follows src/cuda/random.h:31-67.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lisa {

// ---- scalar, one rounding each ------------------------------------------
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }

struct V3 {
  float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 v3(float s) { return V3{s, s, s}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)}; }
__device__ __forceinline__ V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return V3{fmul(a.x, b.x), fmul(a.y, b.y), fmul(a.z, b.z)}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return V3{fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return V3{fmul(s, a.x), fmul(s, a.y), fmul(s, a.z)}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return V3{fdiv(a.x, s), fdiv(a.y, s), fdiv(a.z, s)}; }

// ((a.x*b.x + a.y*b.y) + a.z*b.z)
__device__ __forceinline__ float dot(V3 a, V3 b) {
  return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z));
}
__device__ __forceinline__ V3 normalize(V3 v) {
  // the correctly rounded reciprocal: the value of 1.0f / x
  const float inv = __frcp_rn(fsqrt(dot(v, v)));
  return v * inv;
}
// i - (2*n)*dot(n,i)
__device__ __forceinline__ V3 reflect(V3 i, V3 n) { return i - (2.0f * n) * dot(n, i); }
// n * copysign(1, dot(i, nref))
__device__ __forceinline__ V3 faceforward(V3 n, V3 i, V3 nref) { return n * copysignf(1.0f, dot(i, nref)); }
// a + t*(b-a)
__device__ __forceinline__ V3 lerp(V3 a, V3 b, float t) { return a + t * (b - a); }
__device__ __forceinline__ float clampf(float f, float a, float b) { return fmaxf(a, fminf(f, b)); }
__device__ __forceinline__ bool is_zero(V3 v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }

__device__ __forceinline__ V3 ld3(float4 f) { return V3{f.x, f.y, f.z}; }

// ---- RNG (src/cuda/random.h:31-67, src/LiSA/src/maths.cu:6-8) -----------
template <unsigned N>
__host__ __device__ __forceinline__ uint32_t tea(uint32_t v0, uint32_t v1) {
  uint32_t s0 = 0;
#pragma unroll
  for (unsigned n = 0; n < N; n++) {
    s0 += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  return v0;
}
// 24-bit LCG step; value in [0, 2^24)
__device__ __forceinline__ uint32_t lcg(uint32_t& prev) {
  prev = 1664525u * prev + 1013904223u;
  return prev & 0x00FFFFFFu;
}
// [0, 1): exact (24-bit integer times 2^-24; the same value as the quotient
// by 2^24 that the reference computes)
__device__ __forceinline__ float rnd(uint32_t& s) { return fmul((float)lcg(s), 5.9604644775390625e-8f); }
// [-1, 1): rnd*2 - 1
__device__ __forceinline__ float rng11(uint32_t& s) { return fsub(fmul(rnd(s), 2.0f), 1.0f); }

// k LCG steps at once: the state after them is a * state + c (mod 2^32),
// with a = A^k and c = C (A^(k-1) + ... + A + 1) for the step's A and C.
struct LcgJump {
  uint32_t a, c;
};
__device__ __forceinline__ LcgJump lcg_jump(uint32_t k) {
  LcgJump j{1u, 0u};
  for (uint32_t i = 0; i < k; ++i) {
    j.a *= 1664525u;
    j.c = j.c * 1664525u + 1013904223u;
  }
  return j;
}

}  // namespace lisa

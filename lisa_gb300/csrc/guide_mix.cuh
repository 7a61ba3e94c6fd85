// Path-guide math shared by the sampler (wavefront.cu) and the training
// kernels (guide.cu): input encoding, decoding of the 40 network outputs
// into an 8-lobe von Mises-Fisher mixture, its pdf, sampling and the
// gradient of the training loss, and the pdf of the reference's hemisphere
// sampler.
//
// vMF lobe on the sphere: f(w) = k / (2 pi (1 - e^{-2k})) exp(k (mu.w - 1)),
// sampled with the numerically stable inversion of Jakob, "Numerically
// stable sampling of the von Mises Fisher distribution on S^2" (2012).
// Loss of one sample (Mueller et al., "Neural Importance Sampling", 2019):
// -weight * log q_guide(w), weight = L(w) p_bsdf(w) / q(w).
#pragma once

#include "device_math.cuh"

namespace lisa {
namespace guide {

constexpr int LOBES = 8;
constexpr int NOUT = 40;
constexpr int NIN = 64;
constexpr float KAPPA_LO = -4.0f, KAPPA_HI = 8.0f;  // kappa = exp(raw), raw clamped

// Input features (64): sin(2^k pi x) of the position normalised to the
// scene box, twelve octaves k = -3..8, for x, y, z (36); the normalised
// position mapped to [-1, 1] (3); the shading normal (3); the view
// direction (3); their dot product (1); the estimator's emitter flag after
// this vertex's emitter search (1: an emitter was seen and the flag is
// set, shader.cu:177-184), which changes what a bounce will gather; zeros
// (17).
__device__ __forceinline__ void encode(const float* bmin, const float* bmax, float px, float py, float pz, float nx,
                                       float ny, float nz, float vx, float vy, float vz, float flag, float* f) {
  const float p[3] = {px, py, pz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float ext = bmax[a] - bmin[a];
    const float u = ext > 0.0f ? fminf(fmaxf(__fdividef(p[a] - bmin[a], ext), 0.0f), 1.0f) : 0.5f;
    // one fast sine/cosine (absolute error ~2^-21 on [0, pi/8]), then the
    // double-angle recurrence for the higher octaves (the error doubles per
    // octave: ~2^-10 at the last, still under the inputs' BF16 precision)
    float sn, cs;
    __sincosf(u * 0.39269908169872414f, &sn, &cs);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      f[3 * k + a] = sn;
      const float s2 = 2.0f * sn * cs, c2 = (cs - sn) * (cs + sn);
      sn = s2;
      cs = c2;
    }
    f[36 + a] = 2.0f * u - 1.0f;
  }
  f[39] = nx;
  f[40] = ny;
  f[41] = nz;
  f[42] = vx;
  f[43] = vy;
  f[44] = vz;
  f[45] = nx * vx + ny * vy + nz * vz;
  f[46] = flag;
#pragma unroll
  for (int i = 47; i < 64; ++i) f[i] = 0.0f;
}

struct Lobe {
  float mx, my, mz;  // unit mean direction
  float kappa;
  float w;           // mixture weight
  float norm;        // |raw mu|
  float nk;          // vMF normalisation kappa / (2 pi (1 - e^{-2 kappa}))
};

// 1 - e^{-t} for t >= 0: a three-term series below 0.05 (relative error
// under 1e-6 there), else 1 - __expf(-t) (its cancellation costs at most
// 5 bits at t = 0.05).
__device__ __forceinline__ float one_minus_exp_neg(float t) {
  return t < 0.05f ? t * (1.0f - t * (0.5f - t * (1.0f / 6.0f))) : 1.0f - __expf(-t);
}

// Decodes the 40 raw outputs: per lobe (mu xyz, kappa, logit).  Fast
// intrinsics throughout: sampling and density read the same decoded lobes,
// so their small errors change which mixture is used, not the estimator's
// expectation.
__device__ __forceinline__ void decode(const float* o, Lobe* L) {
  float mx = -1e30f;
#pragma unroll
  for (int k = 0; k < LOBES; ++k) mx = fmaxf(mx, o[5 * k + 4]);
  float z = 0.0f;
#pragma unroll
  for (int k = 0; k < LOBES; ++k) {
    const float e = __expf(o[5 * k + 4] - mx);
    L[k].w = e;
    z += e;
  }
  const float iz = __fdividef(1.0f, z);
#pragma unroll
  for (int k = 0; k < LOBES; ++k) {
    const float ax = o[5 * k], ay = o[5 * k + 1], az = o[5 * k + 2];
    const float n2 = fmaxf(ax * ax + ay * ay + az * az, 1e-12f);
    const float in = rsqrtf(n2);
    L[k].mx = ax * in;
    L[k].my = ay * in;
    L[k].mz = az * in;
    L[k].norm = n2 * in;
    const float kap = __expf(fminf(fmaxf(o[5 * k + 3], KAPPA_LO), KAPPA_HI));
    L[k].kappa = kap;
    // the vMF normalisation, once per lobe, not per evaluation
    L[k].nk = __fdividef(kap, 6.28318530717958647692f * one_minus_exp_neg(2.0f * kap));
    L[k].w *= iz;
  }
}

// vMF density at unit w.
__device__ __forceinline__ float vmf_pdf(const Lobe& l, float wx, float wy, float wz) {
  const float c = l.mx * wx + l.my * wy + l.mz * wz;
  return l.nk * __expf(l.kappa * (c - 1.0f));
}

__device__ __forceinline__ float mix_pdf(const Lobe* L, float wx, float wy, float wz) {
  float q = 0.0f;
#pragma unroll
  for (int k = 0; k < LOBES; ++k) q += L[k].w * vmf_pdf(L[k], wx, wy, wz);
  return q;
}

// Sample the mixture with three uniforms in [0,1).
__device__ __forceinline__ void mix_sample(const Lobe* L, float u0, float u1, float u2, float& wx, float& wy,
                                           float& wz) {
  // the first lobe whose cumulative weight exceeds u0 (the last one if
  // none does), picked by selects so that L stays in registers
  Lobe l = L[LOBES - 1];
  float acc = 0.0f;
  bool found = false;
#pragma unroll
  for (int k = 0; k < LOBES - 1; ++k) {
    acc += L[k].w;
    const bool take = !found && u0 < acc;
    if (take) l = L[k];
    found = found || take;
  }
  const float k = l.kappa;
  // cos of the angle to mu: 1 + log(u1 + (1-u1) e^{-2k}) / k  (kappa <= e^5
  // keeps e^{-2k} representable enough; the clamp guards u1 = 0)
  const float ww = fminf(fmaxf(1.0f + __fdividef(__logf(u1 + (1.0f - u1) * __expf(-2.0f * k)), k), -1.0f), 1.0f);
  const float st = sqrtf(fmaxf(0.0f, 1.0f - ww * ww));
  float sp, cp;
  sincospif(2.0f * u2, &sp, &cp);
  // orthonormal basis around mu (Duff et al. 2017)
  const float sgn = copysignf(1.0f, l.mz);
  const float a = -1.0f / (sgn + l.mz);
  const float b = l.mx * l.my * a;
  const float t1x = 1.0f + sgn * l.mx * l.mx * a, t1y = sgn * b, t1z = -sgn * l.mx;
  const float t2x = b, t2y = sgn + l.my * l.my * a, t2z = -l.my;
  wx = ww * l.mx + st * (cp * t1x + sp * t2x);
  wy = ww * l.my + st * (cp * t1y + sp * t2y);
  wz = ww * l.mz + st * (cp * t1z + sp * t2z);
}

// Density of the reference hemisphere sampler (maths.cu:10-15): a uniform
// point of the cube [-1,1)^3, normalised, flipped into N's hemisphere:
// p(w) = 1 / (12 max_i |w_i|^3) for N.w > 0, w unit.
__device__ __forceinline__ float hemi_pdf(float nx, float ny, float nz, float wx, float wy, float wz) {
  if (nx * wx + ny * wy + nz * wz <= 0.0f) return 0.0f;
  const float m = fmaxf(fabsf(wx), fmaxf(fabsf(wy), fabsf(wz)));
  return __fdividef(1.0f, 12.0f * m * m * m);
}

// Gradient of  -wt * log q(w)  with respect to the 40 raw outputs o; also
// returns the loss term.  wt already includes any batch normalisation.
__device__ __forceinline__ float loss_grad(const float* o, float wx, float wy, float wz, float wt, float* g) {
  Lobe L[LOBES];
  decode(o, L);
  float f[LOBES];
  float q = 0.0f;
#pragma unroll
  for (int k = 0; k < LOBES; ++k) {
    f[k] = vmf_pdf(L[k], wx, wy, wz);
    q += L[k].w * f[k];
  }
  q = fmaxf(q, 1e-30f);
  const float iq = 1.0f / q;
#pragma unroll
  for (int k = 0; k < LOBES; ++k) {
    const float r = L[k].w * f[k] * iq;  // responsibility
    const float kap = L[k].kappa;
    const float c = L[k].mx * wx + L[k].my * wy + L[k].mz * wz;
    // d log f / d kappa = 1/k - 2/(e^{2k} - 1) + (c - 1)
    const float dlk = 1.0f / kap - 2.0f / expm1f(2.0f * kap) + (c - 1.0f);
    const float raw_k = o[5 * k + 3];
    const float dkap = (raw_k > KAPPA_LO && raw_k < KAPPA_HI) ? kap : 0.0f;
    g[5 * k + 3] = -wt * r * dlk * dkap;
    // d log f / d mu = kappa w, through mu = raw / |raw|
    const float gx = -wt * r * kap * wx, gy = -wt * r * kap * wy, gz = -wt * r * kap * wz;
    const float dotm = gx * L[k].mx + gy * L[k].my + gz * L[k].mz;
    const float in = 1.0f / L[k].norm;
    g[5 * k + 0] = (gx - dotm * L[k].mx) * in;
    g[5 * k + 1] = (gy - dotm * L[k].my) * in;
    g[5 * k + 2] = (gz - dotm * L[k].mz) * in;
    // softmax logits
    g[5 * k + 4] = -wt * (r - L[k].w);
  }
  return -wt * __logf(q);
}

}  // namespace guide
}  // namespace lisa

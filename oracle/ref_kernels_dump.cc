// Test infrastructure (oracle), not product code.
//
// Compiles the reference's own device helpers on the host -- the BSDF file
// src/LiSA/src/bsdfs/lambertian.cu (which includes src/LiSA/src/maths.cu,
// src/cuda/random.h, src/sutil/vec_math.h and src/cuda/helpers.h) and the
// camera frame src/sutil/Camera.cpp -- and prints golden vectors of them on
// fixed inputs, one record per line:  <name> <hex words...>.  Floats are
// printed as IEEE-754 bit patterns.  The only addition is a stand-in for the
// OptiX intrinsic optixGetPrimitiveIndex() that get_barycentric_normal()
// calls (src/LiSA/src/maths.cu:58-71).
#include <optix_types.h>

#include <cstdint>
#include <cstdio>
#include <cstring>

static int g_prim_idx = 0;
static inline int optixGetPrimitiveIndex() { return g_prim_idx; }

#include "bsdfs/lambertian.cu"
#include "sutil/Camera.h"

static uint32_t fb(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
static void pf(float f) { std::printf(" %08x", fb(f)); }
static void p3(float3 v) {
  pf(v.x);
  pf(v.y);
  pf(v.z);
}

// deterministic input generator (xorshift32 -> [-1, 1))
static uint32_t g_x = 0x12345678u;
static float u11() {
  g_x ^= g_x << 13;
  g_x ^= g_x >> 17;
  g_x ^= g_x << 5;
  return (float)(g_x >> 8) / 8388608.0f - 1.0f;
}
static float3 r3() { return make_float3(u11(), u11(), u11()); }

int main() {
  // tea<16> (random.h:31-46)
  for (uint32_t a = 0; a < 64; a += 7)
    for (uint32_t b = 0; b < 5; ++b) std::printf("tea16 %08x %08x %08x\n", a * 1000003u, b, tea<16>(a * 1000003u, b));
  // lcg / rnd streams (random.h:49-67)
  for (uint32_t s0 : {0u, 1u, 12345u, 0xdeadbeefu, tea<16>(77u, 0u)}) {
    uint32_t s = s0;
    std::printf("rnd %08x", s0);
    for (int k = 0; k < 8; ++k) pf(rnd(s));
    std::printf(" %08x\n", s);
  }
  // vec_math helpers
  for (int i = 0; i < 16; ++i) {
    float3 a = r3(), b = r3();
    float t = 0.5f * (u11() + 1.0f);
    std::printf("normalize");
    p3(a);
    p3(normalize(a));
    std::printf("\nreflect");
    p3(a);
    p3(b);
    p3(reflect(a, b));
    std::printf("\nfaceforward");
    p3(a);
    p3(b);
    p3(faceforward(a, b, a));
    std::printf("\nlerp");
    p3(a);
    p3(b);
    pf(t);
    p3(lerp(a, b, t));
    std::printf("\n");
  }
  // fresnel / BTDF (maths.cu:17-20, lambertian.cu:24-27)
  for (float eta : {1.0f / 1.5f, 1.5f, 1.0f / 1.33f, 2.4f})
    for (int k = 0; k <= 10; ++k) {
      const float c = 0.1f * (float)k;
      std::printf("fresnel");
      pf(c);
      pf(eta);
      pf(BTDF(c, eta));
      std::printf("\n");
    }
  // refract (maths.cu:22-30), including total internal reflection
  for (int i = 0; i < 16; ++i) {
    float3 d = normalize(r3()), n = normalize(r3());
    float cosI = dot(d, n);
    float eta = (i & 1) ? 1.5f : 1.0f / 1.5f;
    if (cosI < 0) cosI = -cosI; else n = -n;
    std::printf("refract");
    pf(cosI);
    p3(d);
    p3(n);
    pf(eta);
    p3(refract(cosI, d, n, eta));
    std::printf("\n");
  }
  // BRDF (lambertian.cu:15-22)
  Material mat;
  std::memset(&mat, 0, sizeof(mat));
  mat.roughness = 1.0f;
  for (int i = 0; i < 16; ++i) {
    float3 n = normalize(r3()), l = normalize(r3());
    std::printf("brdf");
    p3(n);
    p3(l);
    pf(BRDF(n, l, &mat));
    std::printf("\n");
  }
  // bounce with roughness 0: the reflection (the hemisphere draw is still
  // consumed, three LCG steps)
  mat.roughness = 0.0f;
  for (int i = 0; i < 8; ++i) {
    float3 d = normalize(r3()), n = normalize(r3());
    uint32_t s = 1000u + (uint32_t)i;
    float3 b = bounce(d, n, s, &mat);
    std::printf("bounce0");
    p3(d);
    p3(n);
    p3(b);
    std::printf(" %08x\n", s);
  }
  // barycentric shading normal (maths.cu:33-71)
  for (int i = 0; i < 16; ++i) {
    float3 vs[3] = {r3(), r3(), r3()};
    float3 ns[3] = {normalize(r3()), normalize(r3()), normalize(r3())};
    float w0 = 0.5f * (u11() + 1.0f), w1 = 0.5f * (u11() + 1.0f) * (1.0f - w0);
    float3 p = vs[0] + w0 * (vs[1] - vs[0]) + w1 * (vs[2] - vs[0]);
    HitGroupData hg;
    hg.material = &mat;
    hg.vertices = vs;
    hg.normals = ns;
    g_prim_idx = 0;
    float3 nn = get_barycentric_normal(p, &hg);
    std::printf("barynormal");
    p3(p);
    for (auto& x : ns) p3(x);
    for (auto& x : vs) p3(x);
    p3(nn);
    std::printf("\n");
  }
  // make_color (helpers.h:35-62)
  for (int i = 0; i <= 64; ++i) {
    const float x = (float)i / 48.0f - 0.1f;
    float3 c = make_float3(x, x * 0.5f, x * x);
    uchar4 u = make_color(c);
    std::printf("make_color");
    p3(c);
    std::printf(" %02x %02x %02x %02x\n", u.x, u.y, u.z, u.w);
  }
  // camera UVW frame (Camera.cpp:34-45) with the set-up of init_params
  // (optix_wrapper.cc:434-442)
  const float cams[][9] = {{0, 0, 1.9f, 0, 0, 0, 40, 256, 256},
                           {-0.01f, 0.015f, 0.6f, -0.01f, 0.015f, 0, 40, 2000, 2000},
                           {50, 50, 175, 50, 50, 50, 40, 1920, 1080},
                           {1, 2, 3, -1, 0.5f, -2, 65, 640, 480}};
  for (auto& c : cams) {
    sutil::Camera cam;
    cam.setEye(make_float3(c[0], c[1], c[2]));
    cam.setLookat(make_float3(c[3], c[4], c[5]));
    cam.setUp(make_float3(0.0f, 1.0f, 0.0f));
    cam.setFovY(c[6]);
    cam.setAspectRatio((float)c[7] / (float)c[8]);
    float3 U, V, W;
    cam.UVWFrame(U, V, W);
    std::printf("uvw");
    for (int k = 0; k < 7; ++k) pf(c[k]);
    std::printf(" %u %u", (unsigned)c[7], (unsigned)c[8]);
    p3(U);
    p3(V);
    p3(W);
    std::printf("\n");
  }
  return 0;
}

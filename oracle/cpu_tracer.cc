// ORACLE -- test infrastructure only.  Never linked into or called by the
// product library; tests, __graft_entry__.smoke() and the CPU-baseline leg of
// bench.py load it as the checker.
//
// A scalar CPU restatement of LiSA's Monte Carlo estimator and of the
// closest-hit query it relies on:
//   * RNG: tea<16> seed hash, 24-bit LCG, rnd (src/cuda/random.h:31-67),
//     rng = 2*rnd-1 (src/LiSA/src/maths.cu:6-8)
//   * vector helpers as src/sutil/vec_math.h (:521-564, :494-497)
//   * hemisphere sampling, Schlick, refraction, barycentric shading normal
//     (src/LiSA/src/maths.cu:10-70)
//   * bounce / BRDF / BTDF (src/LiSA/src/bsdfs/lambertian.cu:7-27)
//   * the raygen / path loop / closest-hit / occlusion programs
//     (src/LiSA/src/shader.cu:102-255), with the stale emitter flag
//   * camera UVW frame (src/sutil/Camera.cpp:34-45)
//   * tone map make_color (src/cuda/helpers.h:35-62)
// Closest hits come from a brute-force scan or a CPU BVH, both using the
// watertight triangle test (Woop, Benthin, Wald, JCGT 2013) with the
// lowest-index tie rule.  Every float operation is one IEEE rounding: the
// file is compiled with -ffp-contract=off and no fast-math, and
// pow(x,2)/pow(x,5) are written as products.
//
// It also restates the product's opt-in physically based estimator
// (estimator = 1; no reference counterpart): emitter sampling by area x
// luminance with two-sided emitters, cosine-weighted diffuse sampling,
// power-heuristic MIS between the two, roughness as the weight of the
// diffuse lobe against a mirror, and Schlick's Fresnel term evaluated on the
// less dense side (the transmitted cosine when leaving a medium).  A path
// has at most `bounces` scattering vertices; the ray leaving the last one is
// still traced for the emission it reaches (the BSDF half of that vertex's
// MIS), so every emitter sample keeps its power-heuristic weight.
//
// Deliberate readings of the reference (shared with the product):
//   * a zero direction (total internal reflection) is a miss, not traced;
//   * occlusion queries return the closest hit (OptiX's terminate-on-first-
//     hit may report another one);
//   * make_float3(rng, rng, rng) draws x, then y, then z.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

namespace {

struct V3 {
  float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 normalize(V3 v) {
  const float inv = 1.0f / std::sqrt(dot(v, v));
  return v * inv;
}
inline V3 reflect(V3 i, V3 n) { return i - (2.0f * n) * dot(n, i); }
inline V3 faceforward(V3 n, V3 i, V3 nref) { return n * std::copysign(1.0f, dot(i, nref)); }
inline V3 lerp(V3 a, V3 b, float t) { return a + t * (b - a); }
inline float clampf(float f, float a, float b) { return std::fmax(a, std::fmin(f, b)); }
inline bool is_zero(V3 v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }

// ---- RNG ----
template <unsigned N>
uint32_t tea(uint32_t v0, uint32_t v1) {
  uint32_t s0 = 0;
  for (unsigned n = 0; n < N; n++) {
    s0 += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  return v0;
}
inline uint32_t lcg(uint32_t& prev) {
  prev = 1664525u * prev + 1013904223u;
  return prev & 0x00FFFFFFu;
}
inline float rnd(uint32_t& s) { return (float)lcg(s) / 16777216.0f; }
inline float rng11(uint32_t& s) { return rnd(s) * 2.0f - 1.0f; }

// ---- maths.cu / lambertian.cu ----
V3 hemi(V3 N, uint32_t& seed) {
  const float x = rng11(seed);
  const float y = rng11(seed);
  const float z = rng11(seed);
  const V3 r = normalize(v3(x, y, z));
  return faceforward(r, N, r);
}
float fresnel(float cosT, float eta) {
  const float r = (1.0f - eta) / (1.0f + eta);
  const float R0 = r * r;
  const float x = 1.0f - cosT;
  const float x5 = (((x * x) * x) * x) * x;
  return R0 + (1.0f - R0) * x5;
}
V3 refract(float cosI, V3 d, V3 N, float eta) {
  const float cost2 = 1.0f - (eta * eta) * (1.0f - cosI * cosI);
  const float k = eta * cosI - std::sqrt(std::fabs(cost2));
  const V3 t = eta * d + k * N;
  return t * (cost2 > 0.0f ? 1.0f : 0.0f);
}
V3 barycentric_normal(V3 p, V3 n1, V3 n2, V3 n3, V3 v1, V3 v2, V3 v3_) {
  const V3 e1 = v2 - v1, e2 = v3_ - v1, i = p - v1;
  const float d00 = dot(e1, e1), d01 = dot(e1, e2), d11 = dot(e2, e2);
  const float d20 = dot(i, e1), d21 = dot(i, e2);
  const float denom = d00 * d11 - d01 * d01;
  const float w = (d00 * d21 - d01 * d20) / denom;
  const float v = (d11 * d20 - d01 * d21) / denom;
  const float u = 1.0f - v - w;
  return normalize((u * n1 + v * n2) + w * n3);
}
float BRDF(V3 N, V3 L) {
  const float NdotL = clampf(dot(N, L), 0.0f, 1.0f);
  const float sp = NdotL / 3.14159265358979323846f;
  return NdotL * sp;
}
V3 bounce(V3 D, V3 N, uint32_t& seed, float roughness) {
  const V3 r = reflect(D, N);
  const V3 h = hemi(N, seed);
  return lerp(r, h, roughness);
}

// ---- helpers.h tone map ----
unsigned char quantize8(float x) {
  x = clampf(x, 0.0f, 1.0f);
  return (unsigned char)std::min((unsigned)(x * 256.0f), 255u);
}
float to_srgb(float c) {
  const float inv_gamma = 1.0f / 2.4f;
  return c < 0.0031308f ? 12.92f * c : 1.055f * std::pow(c, inv_gamma) - 0.055f;
}

// ---- Camera.cpp UVW frame ----
void uvw(const float* eye, const float* look, float fov, uint32_t w, uint32_t h, V3& U, V3& V, V3& W) {
  const V3 e = v3(eye[0], eye[1], eye[2]), la = v3(look[0], look[1], look[2]), up = v3(0.0f, 1.0f, 0.0f);
  const float aspect = (float)w / (float)h;
  W = la - e;
  const float wlen = std::sqrt(dot(W, W));
  U = normalize(cross(W, up));
  V = normalize(cross(U, W));
  const float vlen = wlen * std::tan(0.5f * fov * 3.14159265358979323846f / 180.0f);
  V = V * vlen;
  const float ulen = vlen * aspect;
  U = U * ulen;
}

// ---- watertight triangle test (same operation order as the product) ----
struct RayPre {
  float o[3];
  int kx, ky, kz;
  float Sx, Sy, Sz;
};
RayPre prepare(V3 o, V3 d) {
  RayPre r;
  r.o[0] = o.x;
  r.o[1] = o.y;
  r.o[2] = o.z;
  const float dd[3] = {d.x, d.y, d.z};
  const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
  int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  int kx = kz + 1;
  if (kx == 3) kx = 0;
  int ky = kx + 1;
  if (ky == 3) ky = 0;
  if (dd[kz] < 0.0f) std::swap(kx, ky);
  r.kx = kx;
  r.ky = ky;
  r.kz = kz;
  r.Sx = dd[kx] / dd[kz];
  r.Sy = dd[ky] / dd[kz];
  r.Sz = 1.0f / dd[kz];
  return r;
}
const float INF = std::numeric_limits<float>::infinity();
float intersect(const RayPre& r, const float* a, const float* b, const float* c, float tmin) {
  const float A[3] = {a[0] - r.o[0], a[1] - r.o[1], a[2] - r.o[2]};
  const float B[3] = {b[0] - r.o[0], b[1] - r.o[1], b[2] - r.o[2]};
  const float C[3] = {c[0] - r.o[0], c[1] - r.o[1], c[2] - r.o[2]};
  const float Ax = A[r.kx] - r.Sx * A[r.kz], Ay = A[r.ky] - r.Sy * A[r.kz];
  const float Bx = B[r.kx] - r.Sx * B[r.kz], By = B[r.ky] - r.Sy * B[r.kz];
  const float Cx = C[r.kx] - r.Sx * C[r.kz], Cy = C[r.ky] - r.Sy * C[r.kz];
  const float U = Cx * By - Cy * Bx;
  const float V = Ax * Cy - Ay * Cx;
  const float W = Bx * Ay - By * Ax;
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return INF;
  const float det = (U + V) + W;
  if (det == 0.0f) return INF;
  const float Az = r.Sz * A[r.kz], Bz = r.Sz * B[r.kz], Cz = r.Sz * C[r.kz];
  const float T = (U * Az + V * Bz) + W * Cz;
  const float t = T / det;
  if (!(t > tmin)) return INF;
  return t;
}

// ---- scene + closest hit ----
struct Bvh {
  struct Node {
    float lo[3], hi[3];
    uint32_t left, count;  // count>0: leaf with prims[left .. left+count)
  };
  std::vector<Node> nodes;
  std::vector<uint32_t> prims;
};

// Emitters of the physically based estimator: one 16-float record per
// emissive triangle of positive area and luminance --
// (v0.xyz, area pdf) (e1 = v1 - v0, material as int bits) (e2 = v2 - v0, 0)
// (unit normal, 0) -- a CDF over area x luminance, and per material the
// area pdf luminance / total of its triangles.
struct Emitters {
  std::vector<float> rec;
  std::vector<float> cdf;
  std::vector<float> mat_pdf;
  uint32_t count = 0;
};

struct Ctx {
  const float* v = nullptr;   // 9 per triangle
  const float* n = nullptr;   // 9 per triangle
  const int32_t* mi = nullptr;
  uint32_t T = 0;
  std::vector<int> cls;
  std::vector<float> albedo, emission, rough, ior;
  float extent = 1.0f;
  Bvh bvh;
  bool use_bvh = false;
  Emitters em;
  // bounds of the emissive triangles, padded by 1e-4 of the scene diagonal
  // (the same float steps as the product's scene upload)
  bool has_emit_box = false;
  float emit_lo[3] = {0, 0, 0}, emit_hi[3] = {0, 0, 0};
};

void build_bvh(Ctx& c) {
  const uint32_t T = c.T;
  std::vector<float> lo(3ull * T), hi(3ull * T), ce(3ull * T);
  for (uint32_t p = 0; p < T; ++p)
    for (int k = 0; k < 3; ++k) {
      const float* t = c.v + 9ull * p;
      lo[3 * p + k] = std::min(std::min(t[k], t[3 + k]), t[6 + k]);
      hi[3 * p + k] = std::max(std::max(t[k], t[3 + k]), t[6 + k]);
      ce[3 * p + k] = 0.5f * (lo[3 * p + k] + hi[3 * p + k]);
    }
  c.bvh.prims.resize(T);
  std::iota(c.bvh.prims.begin(), c.bvh.prims.end(), 0u);
  c.bvh.nodes.clear();
  c.bvh.nodes.reserve(2ull * T + 1);
  struct Item {
    uint32_t node, b, e;
  };
  std::vector<Item> st;
  c.bvh.nodes.push_back({});
  st.push_back({0, 0, T});
  while (!st.empty()) {
    Item it = st.back();
    st.pop_back();
    Bvh::Node nd;
    for (int k = 0; k < 3; ++k) {
      nd.lo[k] = INF;
      nd.hi[k] = -INF;
    }
    float clo[3] = {INF, INF, INF}, chi[3] = {-INF, -INF, -INF};
    for (uint32_t i = it.b; i < it.e; ++i) {
      const uint32_t p = c.bvh.prims[i];
      for (int k = 0; k < 3; ++k) {
        nd.lo[k] = std::min(nd.lo[k], lo[3 * p + k]);
        nd.hi[k] = std::max(nd.hi[k], hi[3 * p + k]);
        clo[k] = std::min(clo[k], ce[3 * p + k]);
        chi[k] = std::max(chi[k], ce[3 * p + k]);
      }
    }
    if (it.e - it.b <= 4) {
      nd.left = it.b;
      nd.count = it.e - it.b;
      c.bvh.nodes[it.node] = nd;
      continue;
    }
    int ax = 0;
    for (int k = 1; k < 3; ++k)
      if (chi[k] - clo[k] > chi[ax] - clo[ax]) ax = k;
    const uint32_t mid = (it.b + it.e) / 2;
    std::nth_element(c.bvh.prims.begin() + it.b, c.bvh.prims.begin() + mid, c.bvh.prims.begin() + it.e,
                     [&](uint32_t a, uint32_t b) {
                       return ce[3 * a + ax] < ce[3 * b + ax] || (ce[3 * a + ax] == ce[3 * b + ax] && a < b);
                     });
    const uint32_t l = (uint32_t)c.bvh.nodes.size();
    c.bvh.nodes.push_back({});
    c.bvh.nodes.push_back({});
    nd.left = l;
    nd.count = 0;
    c.bvh.nodes[it.node] = nd;
    st.push_back({l, it.b, mid});
    st.push_back({l + 1, mid, it.e});
  }
}

// conservative slab test in double
inline bool box_hit(const Bvh::Node& nd, const double* o, const double* inv, const bool* zero, double tmin, double tmax,
                    double* tnear) {
  double t0 = tmin, t1 = tmax;
  for (int k = 0; k < 3; ++k) {
    if (zero[k]) {
      if (o[k] < nd.lo[k] || o[k] > nd.hi[k]) return false;
      continue;
    }
    double a = ((double)nd.lo[k] - o[k]) * inv[k], b = ((double)nd.hi[k] - o[k]) * inv[k];
    if (a > b) std::swap(a, b);
    t0 = std::max(t0, a);
    t1 = std::min(t1, b);
  }
  *tnear = t0;
  return t0 <= t1;
}

void closest(const Ctx& c, V3 o, V3 d, float tmin, float tmax, int* prim, float* tout) {
  *prim = -1;
  *tout = INF;
  if (is_zero(d)) return;
  const RayPre r = prepare(o, d);
  float best_t = tmax;
  int best = -1;
  auto test = [&](uint32_t p) {
    const float* t = c.v + 9ull * p;
    const float th = intersect(r, t, t + 3, t + 6, tmin);
    if (th < best_t || (th == best_t && best >= 0 && (int)p < best)) {
      best_t = th;
      best = (int)p;
    }
  };
  if (!c.use_bvh) {
    for (uint32_t p = 0; p < c.T; ++p) test(p);
  } else if (c.T) {
    const double od[3] = {o.x, o.y, o.z};
    const double dd[3] = {d.x, d.y, d.z};
    double inv[3];
    bool zero[3];
    for (int k = 0; k < 3; ++k) {
      zero[k] = dd[k] == 0.0;
      inv[k] = zero[k] ? 0.0 : 1.0 / dd[k];
    }
    const double dmax = std::max(std::fabs(dd[0]), std::max(std::fabs(dd[1]), std::fabs(dd[2])));
    const double slack = 1e-5 * c.extent / dmax;
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
      const Bvh::Node& nd = c.bvh.nodes[stack[--sp]];
      double tn;
      const double lim = (double)best_t * (1.0 + 1e-5) + slack;
      if (!box_hit(nd, od, inv, zero, (double)tmin - slack, lim, &tn)) continue;
      if (nd.count) {
        for (uint32_t i = 0; i < nd.count; ++i) test(c.bvh.prims[nd.left + i]);
      } else {
        stack[sp++] = nd.left;
        stack[sp++] = nd.left + 1;
      }
    }
  }
  if (best >= 0) {
    *prim = best;
    *tout = best_t;
  }
}

struct Counters {
  uint64_t primary = 0, bounce = 0, shadow = 0;
};

// One path of the reference estimator (shader.cu:102-124 with the
// closest-hit programs :172-255).
V3 trace_path(const Ctx& c, V3 o, V3 d, int bounces, uint32_t& seed, Counters& cnt) {
  V3 color = v3(0.0f, 0.0f, 0.0f), att = v3(1.0f, 1.0f, 1.0f);
  int stale = -1;
  for (int i = 0; i < bounces; ++i) {
    if (is_zero(d)) break;  // zero direction: a miss
    if (i == 0) ++cnt.primary; else ++cnt.bounce;
    int prim;
    float t;
    closest(c, o, d, 1e-4f, 1e16f, &prim, &t);
    if (prim < 0) break;  // miss: background 0
    const int m = c.mi[prim];
    if (c.cls[m] == 2) {
      color = color + v3(c.emission[3 * m], c.emission[3 * m + 1], c.emission[3 * m + 2]) * att;
      break;
    }
    if (i == bounces) break;
    const V3 p = o + t * d;
    const float* tv = c.v + 9ull * prim;
    const float* tn = c.n + 9ull * prim;
    const V3 N = barycentric_normal(p, v3(tn[0], tn[1], tn[2]), v3(tn[3], tn[4], tn[5]), v3(tn[6], tn[7], tn[8]),
                                    v3(tv[0], tv[1], tv[2]), v3(tv[3], tv[4], tv[5]), v3(tv[6], tv[7], tv[8]));
    const V3 albedo = v3(c.albedo[3 * m], c.albedo[3 * m + 1], c.albedo[3 * m + 2]);
    if (c.cls[m] == 1) {
      float cosI = dot(d, N);
      float eta;
      V3 nrm;
      if (cosI < 0.0f) {
        cosI = -cosI;
        eta = 1.0f / c.ior[m];
        nrm = N;
      } else {
        att = att * albedo;
        eta = c.ior[m];
        nrm = -N;
      }
      V3 nd;
      if (eta == 1.0f) nd = d;
      else if (rnd(seed) <= fresnel(cosI, eta)) nd = reflect(d, nrm);
      else nd = refract(cosI, d, nrm, eta);
      d = nd;
      o = p;
    } else {
      att = att * albedo;
      for (int k = 0; k < 30; ++k) {
        const V3 dir = hemi(N, seed);
        ++cnt.shadow;
        int hp;
        float ht;
        closest(c, p, dir, 1e-4f, 1e16f, &hp, &ht);
        if (hp >= 0) {
          const int hm = c.mi[hp];
          if (c.cls[hm] == 2) stale = hm;
        } else {
          stale = -1;
        }
        if (stale >= 0) {
          const float brdf = BRDF(N, dir);
          color = color + (v3(c.emission[3 * stale], c.emission[3 * stale + 1], c.emission[3 * stale + 2]) * brdf) * att;
          break;
        }
      }
      d = bounce(d, N, seed, c.rough[m]);
      o = p;
    }
  }
  return color;
}

// ---- physically based estimator (the product's opt-in mode) ----
constexpr float PI_F = 3.14159265358979323846f;

inline float luminance(float r, float g, float b) { return (0.2126f * r + 0.7152f * g) + 0.0722f * b; }

// Emitter records, CDF and per-material area pdf, in triangle order.
void build_emitters(Ctx& c) {
  Emitters& e = c.em;
  e.rec.clear();
  e.cdf.clear();
  e.count = 0;
  const size_t M = c.cls.size();
  e.mat_pdf.assign(M, 0.0f);
  std::vector<float> lum(M, 0.0f);
  for (size_t m = 0; m < M; ++m)
    if (c.cls[m] == 2) lum[m] = luminance(c.emission[3 * m], c.emission[3 * m + 1], c.emission[3 * m + 2]);
  std::vector<double> w;
  for (uint32_t p = 0; p < c.T; ++p) {
    const int m = c.mi[p];
    if (c.cls[m] != 2 || !(lum[m] > 0.0f)) continue;
    const float* t = c.v + 9ull * p;
    const V3 v0 = v3(t[0], t[1], t[2]);
    const V3 e1 = v3(t[3], t[4], t[5]) - v0, e2 = v3(t[6], t[7], t[8]) - v0;
    const V3 cr = cross(e1, e2);
    const float len = std::sqrt(dot(cr, cr));
    const float area = 0.5f * len;
    if (!(area > 0.0f)) continue;
    const V3 n = cr * (1.0f / len);
    int mbits;
    std::memcpy(&mbits, &m, 4);
    float mf;
    std::memcpy(&mf, &mbits, 4);
    const float r[16] = {v0.x, v0.y, v0.z, 0.0f, e1.x, e1.y, e1.z, mf, e2.x, e2.y, e2.z, 0.0f, n.x, n.y, n.z, 0.0f};
    e.rec.insert(e.rec.end(), r, r + 16);
    w.push_back((double)area * (double)lum[m]);
  }
  e.count = (uint32_t)w.size();
  if (!e.count) return;
  double total = 0.0;
  for (double x : w) total += x;
  double acc = 0.0;
  e.cdf.resize(e.count);
  for (uint32_t i = 0; i < e.count; ++i) {
    acc += w[i];
    e.cdf[i] = (float)(acc / total);
  }
  e.cdf[e.count - 1] = 1.0f;
  for (size_t m = 0; m < M; ++m) e.mat_pdf[m] = (float)((double)lum[m] / total);
  for (uint32_t i = 0; i < e.count; ++i) {
    int m;
    std::memcpy(&m, &e.rec[16ull * i + 7], 4);
    e.rec[16ull * i + 3] = e.mat_pdf[m];
  }
}

// unit geometric normal of triangle p (cross(v1 - v0, v2 - v0) normalised)
V3 tri_normal(const Ctx& c, int p) {
  const float* t = c.v + 9ull * p;
  const V3 v0 = v3(t[0], t[1], t[2]);
  const V3 cr = cross(v3(t[3], t[4], t[5]) - v0, v3(t[6], t[7], t[8]) - v0);
  return cr * (1.0f / std::sqrt(dot(cr, cr)));
}

// Orthonormal basis around a unit vector (Duff et al., JCGT 2017).
void onb(V3 n, V3& t, V3& b) {
  const float sign = std::copysign(1.0f, n.z);
  const float a = -1.0f / (sign + n.z);
  const float bb = (n.x * n.y) * a;
  t = v3(1.0f + ((sign * n.x) * n.x) * a, sign * bb, -(sign * n.x));
  b = v3(bb, sign + (n.y * n.y) * a, -n.y);
}

// Cosine-weighted direction about n: a uniform point of the unit disk by
// rejection (at most 16 pairs, then the centre), lifted to the hemisphere
// (Malley's method).
V3 cosine_dir(V3 n, uint32_t& seed) {
  float x = 0.0f, y = 0.0f, r2 = 0.0f;
  for (int k = 0; k < 16; ++k) {
    x = rng11(seed);
    y = rng11(seed);
    r2 = x * x + y * y;
    if (r2 < 1.0f) break;
  }
  if (!(r2 < 1.0f)) x = y = r2 = 0.0f;
  const float z = std::sqrt(std::fmax(0.0f, 1.0f - r2));
  V3 t, b;
  onb(n, t, b);
  return normalize((x * t + y * b) + z * n);
}

// A point of an emitter, chosen by area x luminance, uniform on it.
// Returns the record index.
uint32_t sample_emitter(const Emitters& e, uint32_t& seed, V3& y) {
  const float u0 = rnd(seed), u1 = rnd(seed), u2 = rnd(seed);
  uint32_t lo = 0, hi = e.count - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (u0 < e.cdf[mid]) hi = mid;
    else lo = mid + 1;
  }
  const float* r = e.rec.data() + 16ull * lo;
  const float a = std::sqrt(u1);
  const float bu = a * (1.0f - u2), bv = a * u2;
  y = v3(r[0], r[1], r[2]) + (bu * v3(r[4], r[5], r[6]) + bv * v3(r[8], r[9], r[10]));
  return lo;
}

// Whether the ray may meet the padded bounds of the emissive triangles in
// (1e-4, 1e16): slab distances with the correctly rounded 1/d (a huge
// finite value for a zero component), widened by 2^-20 of their magnitude.
// The ray leaving a path's last vertex only gathers emission, so one that
// cannot meet an emitter is not traced (the product takes the same
// decision with the same float steps).
bool final_ray_wanted(const Ctx& c, V3 o, V3 d) {
  if (!c.has_emit_box) return false;
  const float dd[3] = {d.x, d.y, d.z}, oo[3] = {o.x, o.y, o.z};
  float tn = 1e-4f, tf = 1e16f;
  for (int k = 0; k < 3; ++k) {
    const float inv = dd[k] != 0.0f ? 1.0f / dd[k] : std::copysign(1e30f, dd[k]);
    const float a = (c.emit_lo[k] - oo[k]) * inv, b = (c.emit_hi[k] - oo[k]) * inv;
    const float g = 9.5367431640625e-7f * (std::fabs(a) + std::fabs(b));
    tn = std::fmax(tn, std::fmin(a, b) - g);
    tf = std::fmin(tf, std::fmax(a, b) + g);
  }
  return tn <= tf;
}

// One path of the physically based estimator.
V3 trace_path_pb(const Ctx& c, V3 o, V3 d, int bounces, uint32_t& seed, Counters& cnt) {
  V3 color = v3(0.0f, 0.0f, 0.0f), att = v3(1.0f, 1.0f, 1.0f);
  float prev_pdf = 0.0f;  // solid-angle pdf of the last diffuse bounce; 0 after camera / specular
  const Emitters& em = c.em;
  // `bounces` scattering vertices; the ray leaving the last one is traced
  // for the emission it reaches only (its MIS half of that vertex's
  // emitter sample), with no vertex of its own
  for (int i = 0; i <= bounces; ++i) {
    if (is_zero(d)) break;
    if (i == bounces && i > 0 && !final_ray_wanted(c, o, d)) break;
    if (i == 0) ++cnt.primary; else ++cnt.bounce;
    int prim;
    float t;
    closest(c, o, d, 1e-4f, 1e16f, &prim, &t);
    if (prim < 0) break;
    const int m = c.mi[prim];
    const V3 le = v3(c.emission[3 * m], c.emission[3 * m + 1], c.emission[3 * m + 2]);
    if (c.cls[m] == 2) {
      if (prev_pdf > 0.0f) {
        const float cos_y = std::fabs(dot(tri_normal(c, prim), d));
        float w = 0.0f;
        if (cos_y > 0.0f) {
          const float pl = (em.mat_pdf[m] * (t * t)) / cos_y;
          w = (prev_pdf * prev_pdf) / ((prev_pdf * prev_pdf) + (pl * pl));
        }
        color = color + (le * att) * w;
      } else {
        color = color + le * att;
      }
      break;
    }
    if (i == bounces) break;
    const V3 p = o + t * d;
    const float* tv = c.v + 9ull * prim;
    const float* tn = c.n + 9ull * prim;
    const V3 N = barycentric_normal(p, v3(tn[0], tn[1], tn[2]), v3(tn[3], tn[4], tn[5]), v3(tn[6], tn[7], tn[8]),
                                    v3(tv[0], tv[1], tv[2]), v3(tv[3], tv[4], tv[5]), v3(tv[6], tv[7], tv[8]));
    const V3 albedo = v3(c.albedo[3 * m], c.albedo[3 * m + 1], c.albedo[3 * m + 2]);
    if (c.cls[m] == 1) {
      float cosI = dot(d, N);
      float eta;
      V3 nrm;
      if (cosI < 0.0f) {
        cosI = -cosI;
        eta = 1.0f / c.ior[m];
        nrm = N;
      } else {
        att = att * albedo;
        eta = c.ior[m];
        nrm = -N;
      }
      V3 nd;
      if (eta == 1.0f) {
        nd = d;
      } else {
        const float cost2 = 1.0f - (eta * eta) * (1.0f - cosI * cosI);
        if (cost2 <= 0.0f) {
          nd = reflect(d, nrm);  // total internal reflection
        } else {
          const float F = fresnel(eta > 1.0f ? std::sqrt(cost2) : cosI, eta);
          if (rnd(seed) <= F) nd = reflect(d, nrm);
          else nd = refract(cosI, d, nrm, eta);
        }
      }
      prev_pdf = 0.0f;
      d = nd;
      o = p;
      continue;
    }
    att = att * albedo;
    const V3 Ns = dot(N, d) < 0.0f ? N : -N;
    const float r = c.rough[m];
    if (r > 0.0f && em.count > 0) {
      V3 y;
      const uint32_t k = sample_emitter(em, seed, y);
      const float* rec = em.rec.data() + 16ull * k;
      const V3 w = y - p;
      const float d2 = dot(w, w);
      const float dist = std::sqrt(d2);
      const V3 wi = w * (1.0f / dist);
      const float cos_x = dot(Ns, wi);
      const float cos_y = std::fabs(dot(v3(rec[12], rec[13], rec[14]), wi));
      if (cos_x > 0.0f && cos_y > 0.0f && dist > 0.0f) {
        ++cnt.shadow;
        int hp;
        float ht;
        closest(c, p, wi, 1e-4f, dist * (1.0f - 0.0009765625f), &hp, &ht);
        if (hp < 0) {
          int em_m;
          std::memcpy(&em_m, &rec[7], 4);
          const V3 le_y = v3(c.emission[3 * em_m], c.emission[3 * em_m + 1], c.emission[3 * em_m + 2]);
          const float pl = (rec[3] * d2) / cos_y;
          const float fcos = r * (cos_x / PI_F);
          const float wl = (pl * pl) / ((pl * pl) + (fcos * fcos));
          color = color + ((att * le_y) * (fcos / pl)) * wl;
        }
      }
    }
    const bool diffuse = r >= 1.0f || (r > 0.0f && rnd(seed) < r);
    if (diffuse) {
      d = cosine_dir(Ns, seed);
      prev_pdf = r * (dot(Ns, d) / PI_F);
    } else {
      d = reflect(d, Ns);
      prev_pdf = 0.0f;
    }
    o = p;
  }
  return color;
}

}  // namespace

// ===========================================================================
extern "C" {

// Material rows in the reference layout (structs.hh:16-23, 40 bytes).
struct oracle_material {
  float roughness, alpha, n;
  float diffuse[3];
  uint8_t emit;
  uint8_t pad[3];
  float emission[3];
};

struct oracle_scene {
  const float* vertices;  // 9 floats per triangle
  const float* normals;
  const int32_t* mat_indices;
  uint32_t num_triangles;
  const oracle_material* materials;
  uint32_t num_materials;
  uint32_t width, height, spp, bounces;
  float eye[3], look_at[3], fov;
  uint32_t rng_mode;  // 0 = per (seed, pixel, sample), 1 = one stream per pixel
  uint32_t seed;
  uint64_t sample_base;
  uint32_t subframe;
  uint32_t estimator;  // 0 = the reference estimator, 1 = physically based
  float lens_radius;     // thin lens (the product's option; 0 = pinhole, as the reference)
  float focal_distance;  // 0 = |W|
};

static void make_ctx(const oracle_scene* s, int use_bvh, Ctx& c) {
  c.v = s->vertices;
  c.n = s->normals;
  c.mi = s->mat_indices;
  c.T = s->num_triangles;
  const uint32_t M = s->num_materials;
  c.cls.resize(M);
  c.albedo.resize(3 * M);
  c.emission.resize(3 * M);
  c.rough.resize(M);
  c.ior.resize(M);
  for (uint32_t i = 0; i < M; ++i) {
    const oracle_material& m = s->materials[i];
    c.cls[i] = m.emit ? 2 : (m.alpha < 1.0f ? 1 : 0);
    for (int k = 0; k < 3; ++k) {
      c.albedo[3 * i + k] = m.diffuse[k];
      c.emission[3 * i + k] = m.emission[k];
    }
    c.rough[i] = m.roughness;
    c.ior[i] = m.n;
  }
  float lo[3] = {INF, INF, INF}, hi[3] = {-INF, -INF, -INF};
  for (uint64_t i = 0; i < 3ull * c.T; ++i)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], c.v[3 * i + k]);
      hi[k] = std::max(hi[k], c.v[3 * i + k]);
    }
  double e2 = 0;
  for (int k = 0; k < 3; ++k) e2 += c.T ? (double)(hi[k] - lo[k]) * (hi[k] - lo[k]) : 0.0;
  c.extent = e2 > 0 ? (float)std::sqrt(e2) : 1.0f;
  c.use_bvh = use_bvh != 0;
  if (c.use_bvh) build_bvh(c);
  if (c.mi) build_emitters(c);
  if (c.mi && c.T) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    float ext = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (!(ext > 0.0f) || !std::isfinite(ext)) ext = 1.0f;
    float elo[3] = {INF, INF, INF}, ehi[3] = {-INF, -INF, -INF};
    for (uint32_t t = 0; t < c.T; ++t) {
      const int32_t m = c.mi[t];
      if (m < 0 || m >= (int32_t)c.cls.size() || c.cls[m] != 2) continue;
      c.has_emit_box = true;
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          elo[k] = std::min(elo[k], c.v[9ull * t + 3 * j + k]);
          ehi[k] = std::max(ehi[k], c.v[9ull * t + 3 * j + k]);
        }
    }
    const float pad = 1e-4f * ext;
    for (int k = 0; k < 3; ++k) {
      c.emit_lo[k] = c.has_emit_box ? elo[k] - pad : 0.0f;
      c.emit_hi[k] = c.has_emit_box ? ehi[k] + pad : 0.0f;
    }
  }
}

// Closest hit of n rays (8 floats each: ox oy oz tmin dx dy dz tmax).
int oracle_closest(const float* verts, uint32_t T, const float* rays, uint32_t n, int use_bvh, int threads,
                   int32_t* prim, float* tout) {
  oracle_scene s;
  std::memset(&s, 0, sizeof(s));
  s.vertices = verts;
  s.num_triangles = T;
  Ctx c;
  make_ctx(&s, use_bvh, c);
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const float* r = rays + 8 * i;
    int p;
    float t;
    closest(c, v3(r[0], r[1], r[2]), v3(r[4], r[5], r[6]), r[3], r[7], &p, &t);
    prim[i] = p;
    tout[i] = t;
  }
  return 0;
}

// A scene context (material table, CPU BVH) reusable across render calls.
void* oracle_ctx_create(const oracle_scene* s, int use_bvh) {
  Ctx* c = new Ctx();
  make_ctx(s, use_bvh, *c);
  return c;
}
void oracle_ctx_destroy(void* c) { delete (Ctx*)c; }

// Closest hit of one ray (origin o, direction d) on [tmin, tmax] against a
// scene context.  The host build of the reference's shader programs
// (oracle/ref_shader_run.cc) calls it as its optixTrace.
void oracle_ctx_closest(const void* ctx, const float* o, const float* d, float tmin, float tmax, int32_t* prim,
                        float* t) {
  int p;
  float th;
  closest(*(const Ctx*)ctx, v3(o[0], o[1], o[2]), v3(d[0], d[1], d[2]), tmin, tmax, &p, &th);
  *prim = p;
  *t = th;
}

int oracle_ctx_render(void* ctx, const oracle_scene* s, int threads, uint32_t px0, uint32_t px1, double* sum,
                      double* sumsq, uint64_t* rays);

// Render pixels [px0, px1) of the scene: per pixel the FP64 sum and sum of
// squares of the spp sample radiances (3 doubles each).  rays[3] receives
// primary, bounce and shadow ray counts.
int oracle_render(const oracle_scene* s, int use_bvh, int threads, uint32_t px0, uint32_t px1, double* sum,
                  double* sumsq, uint64_t* rays) {
  Ctx c;
  make_ctx(s, use_bvh, c);
  return oracle_ctx_render(&c, s, threads, px0, px1, sum, sumsq, rays);
}

int oracle_ctx_render(void* ctx, const oracle_scene* s, int threads, uint32_t px0, uint32_t px1, double* sum,
                      double* sumsq, uint64_t* rays) {
  const Ctx& c = *(const Ctx*)ctx;
  V3 U, V, W;
  uvw(s->eye, s->look_at, s->fov, s->width, s->height, U, V, W);
  const V3 eye = v3(s->eye[0], s->eye[1], s->eye[2]);
  const float fw = (float)s->width, fh = (float)s->height;
  // unit camera axes and focal distance of the thin lens (the same float
  // steps as the product's scene upload)
  const float ul = std::sqrt(U.x * U.x + U.y * U.y + U.z * U.z);
  const float vl = std::sqrt(V.x * V.x + V.y * V.y + V.z * V.z);
  const float wl = std::sqrt(W.x * W.x + W.y * W.y + W.z * W.z);
  const V3 uU = ul > 0 ? v3(U.x / ul, U.y / ul, U.z / ul) : v3(0, 0, 0);
  const V3 uV = vl > 0 ? v3(V.x / vl, V.y / vl, V.z / vl) : v3(0, 0, 0);
  const V3 uW = wl > 0 ? v3(W.x / wl, W.y / wl, W.z / wl) : v3(0, 0, 0);
  const float fl_dist = s->focal_distance > 0.0f ? s->focal_distance : wl;
  uint64_t tp = 0, tb = 0, ts = 0;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : tp, tb, ts)
  for (int64_t pi = (int64_t)px0; pi < (int64_t)px1; ++pi) {
    const uint32_t pix = (uint32_t)pi;
    const uint32_t x = pix % s->width, y = pix / s->width;
    Counters cnt;
    double a[3] = {0, 0, 0}, q[3] = {0, 0, 0};
    uint32_t seed = s->rng_mode == 1 ? tea<16>(pix, s->subframe) : 0u;
    for (uint32_t j = 0; j < s->spp; ++j) {
      if (s->rng_mode != 1) seed = tea<16>(pix, tea<4>((uint32_t)(s->sample_base + j), s->seed));
      const float jx = rng11(seed);
      const float jy = rng11(seed);
      const float dx = (2.0f * (float)x + jx) / fw - 1.0f;
      const float dy = (2.0f * (float)y + jy) / fh - 1.0f;
      V3 dir = normalize((dx * U + dy * V) + W);
      V3 org = eye;
      if (s->lens_radius > 0.0f) {
        // thin lens: the pinhole ray's point on the focal plane, seen from a
        // uniform point of the lens disk drawn by rejection from the square
        const float tf = fl_dist / dot(dir, uW);
        const V3 focus = org + tf * dir;
        float lu, lv;
        do {
          lu = rng11(seed);
          lv = rng11(seed);
        } while (lu * lu + lv * lv > 1.0f);
        org = org + (s->lens_radius * lu) * uU + (s->lens_radius * lv) * uV;
        dir = normalize(focus - org);
      }
      const V3 col = s->estimator == 1 ? trace_path_pb(c, org, dir, (int)s->bounces, seed, cnt)
                                       : trace_path(c, org, dir, (int)s->bounces, seed, cnt);
      const float cc[3] = {col.x, col.y, col.z};
      for (int k = 0; k < 3; ++k) {
        a[k] += cc[k];
        q[k] += (double)cc[k] * cc[k];
      }
    }
    const uint64_t o = 3ull * (pix - px0);
    for (int k = 0; k < 3; ++k) {
      sum[o + k] = a[k];
      sumsq[o + k] = q[k];
    }
    tp += cnt.primary;
    tb += cnt.bounce;
    ts += cnt.shadow;
  }
  rays[0] = tp;
  rays[1] = tb;
  rays[2] = ts;
  return 0;
}

// make_color of n RGB pixels -> n RGBA bytes (helpers.h:57-62)
void oracle_make_color(const float* rgb, uint64_t n, uint8_t* rgba) {
  for (uint64_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) rgba[4 * i + k] = quantize8(to_srgb(clampf(rgb[3 * i + k], 0.0f, 1.0f)));
    rgba[4 * i + 3] = 255;
  }
}

// Building blocks, exported so tests can pin them against golden vectors of
// the reference's own code.
uint32_t oracle_tea16(uint32_t a, uint32_t b) { return tea<16>(a, b); }
uint32_t oracle_tea4(uint32_t a, uint32_t b) { return tea<4>(a, b); }
float oracle_rnd(uint32_t* s) { return rnd(*s); }
void oracle_normalize(const float* v, float* o) {
  const V3 r = normalize(v3(v[0], v[1], v[2]));
  o[0] = r.x; o[1] = r.y; o[2] = r.z;
}
void oracle_reflect(const float* i, const float* n, float* o) {
  const V3 r = reflect(v3(i[0], i[1], i[2]), v3(n[0], n[1], n[2]));
  o[0] = r.x; o[1] = r.y; o[2] = r.z;
}
void oracle_faceforward(const float* n, const float* i, const float* nref, float* o) {
  const V3 r = faceforward(v3(n[0], n[1], n[2]), v3(i[0], i[1], i[2]), v3(nref[0], nref[1], nref[2]));
  o[0] = r.x; o[1] = r.y; o[2] = r.z;
}
void oracle_lerp(const float* a, const float* b, float t, float* o) {
  const V3 r = lerp(v3(a[0], a[1], a[2]), v3(b[0], b[1], b[2]), t);
  o[0] = r.x; o[1] = r.y; o[2] = r.z;
}
float oracle_fresnel(float cosT, float eta) { return fresnel(cosT, eta); }
void oracle_refract(float cosI, const float* d, const float* N, float eta, float* o) {
  const V3 r = refract(cosI, v3(d[0], d[1], d[2]), v3(N[0], N[1], N[2]), eta);
  o[0] = r.x; o[1] = r.y; o[2] = r.z;
}
float oracle_brdf(const float* N, const float* L) { return BRDF(v3(N[0], N[1], N[2]), v3(L[0], L[1], L[2])); }
void oracle_barycentric_normal(const float* p, const float* n9, const float* v9, float* o) {
  const V3 r = barycentric_normal(v3(p[0], p[1], p[2]), v3(n9[0], n9[1], n9[2]), v3(n9[3], n9[4], n9[5]),
                                  v3(n9[6], n9[7], n9[8]), v3(v9[0], v9[1], v9[2]), v3(v9[3], v9[4], v9[5]),
                                  v3(v9[6], v9[7], v9[8]));
  o[0] = r.x; o[1] = r.y; o[2] = r.z;
}
void oracle_hemi(const float* N, uint32_t* seed, float* o) {
  const V3 r = hemi(v3(N[0], N[1], N[2]), *seed);
  o[0] = r.x; o[1] = r.y; o[2] = r.z;
}
void oracle_uvw(const float* eye, const float* look, float fov, uint32_t w, uint32_t h, float* U9) {
  V3 U, V, W;
  uvw(eye, look, fov, w, h, U, V, W);
  const float out[9] = {U.x, U.y, U.z, V.x, V.y, V.z, W.x, W.y, W.z};
  std::memcpy(U9, out, sizeof(out));
}

}  // extern "C"

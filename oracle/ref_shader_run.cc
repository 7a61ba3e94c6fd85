// Test infrastructure (oracle), not product code.
//
// Runs the reference's own estimator on the host: src/LiSA/src/shader.cu
// (with the files it includes: bsdfs/lambertian.cu, maths.cu, random.h,
// vec_math.h, helpers.h) is compiled by g++ from the reference sources where
// they lie -- never copied -- behind host stand-ins for the OptiX device
// functions it calls.  The scene goes through the reference's own front end
// (SceneParser, src/LiSA/src/scene_parser.cc:35-261) and the set-up of
// OptixWrapper is mirrored on the host:
//   * one hit-group record per material and ray type, radiance records
//     carrying the vertex and normal arrays (optix_wrapper.cc:381-402);
//   * miss records with bg_color = 0 (optix_wrapper.cc:352-356);
//   * the SBT index of a triangle = its material index
//     (optix_wrapper.cc:99-102), primitive index = triangle index;
//   * params: width, height, num_bounces, eye and the sutil::Camera UVW frame
//     (optix_wrapper.cc:419-442); render() sets samples_per_launch to
//     num_samples and launches subframe 0 (render.cc:133-148).
// The stand-ins:
//   * optixTrace: closest hit of [tmin, tmax] from the oracle's scene
//     context (oracle_ctx_closest: watertight test, lowest index on ties),
//     then the closest-hit or miss program of the SBT entry, exactly as
//     OptiX dispatches them.  A zero direction finds no hit (a miss).
//     Occlusion rays use the closest hit too: OptiX's
//     TERMINATE_ON_FIRST_HIT (shader.cu:69) may accept another hit, which is
//     implementation-defined.
//   * optixGetPayload_0/1, optixGetSbtDataPointer, optixGetWorldRayOrigin /
//     Direction, optixGetRayTmax, optixGetPrimitiveIndex: the state of the
//     innermost trace of the calling thread.
//   * optixGetLaunchIndex: the pixel the calling thread runs.
// Argument order: shader.cu:149 and maths.cu:11 build vectors from
// successive RNG draws, make_float2(rng(seed), rng(seed)) and
// make_float3(rng(seed), rng(seed), rng(seed)), whose evaluation order C++
// leaves unspecified.  g++ evaluates these arguments right to left; the
// reference runs them as device code, where the draws go to x, then y, then
// z.  So make_float2/make_float3 are routed through braced
// initialisation, which C++ evaluates left to right, for the shader only.
// Pixels run in parallel (OpenMP); every trace keeps its state on the
// thread's own stack of frames, so nested traces (an occlusion trace from
// inside a closest-hit program) see their own values.
//
// Usage: ref_shader_run scene.rto > out.txt
// Output: a header line, then per pixel the accumulation buffer value the
// raygen program wrote (float bits), the frame buffer bytes, and the number
// of radiance traces, occlusion traces and radiance traces with a zero
// direction that the pixel made.
// With --soup (a raw soup, no text parsing) it times the raygen over a
// sample of pixels on all host threads instead: the reference's own
// estimator as a CPU baseline (closest hits from the oracle's CPU BVH).
#include <omp.h>

#include <cstdint>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "scene_parser.hh"
#include "sutil/Camera.h"

// ---- OptiX device functions: declarations before the shader ------------------
static unsigned int optixGetPayload_0();
static unsigned int optixGetPayload_1();
static CUdeviceptr optixGetSbtDataPointer();
static float3 optixGetWorldRayOrigin();
static float3 optixGetWorldRayDirection();
static float optixGetRayTmax();
static unsigned int optixGetPrimitiveIndex();
static uint3 optixGetLaunchIndex();
static void optixTrace(OptixTraversableHandle handle, float3 origin, float3 direction, float tmin, float tmax,
                       float ray_time, OptixVisibilityMask mask, unsigned int flags, unsigned int sbt_offset,
                       unsigned int sbt_stride, unsigned int miss_index, unsigned int& p0, unsigned int& p1);

#include <sutil/vec_math.h>

#include <utility>

struct LtrFloat2 {
  float2 v;
  template <class... A>
  LtrFloat2(A&&... a) : v(make_float2(std::forward<A>(a)...)) {}
};
struct LtrFloat3 {
  float3 v;
  template <class... A>
  LtrFloat3(A&&... a) : v(make_float3(std::forward<A>(a)...)) {}
};
#define make_float2(...) (LtrFloat2{__VA_ARGS__}.v)
#define make_float3(...) (LtrFloat3{__VA_ARGS__}.v)
#include "shader.cu"
#undef make_float2
#undef make_float3

extern "C" void oracle_ctx_closest(const void* ctx, const float* o, const float* d, float tmin, float tmax,
                                   int32_t* prim, float* t);
extern "C" void* oracle_ctx_create(const void* scene, int use_bvh);

namespace {

// The scene description the oracle library takes (oracle/cpu_tracer.cc,
// struct oracle_scene); only the geometry fields matter for closest hits.
struct OracleScene {
  const float* vertices;
  const float* normals;
  const int32_t* mat_indices;
  uint32_t num_triangles;
  const void* materials;
  uint32_t num_materials;
  uint32_t width, height, spp, bounces;
  float eye[3], look_at[3], fov;
  uint32_t rng_mode, seed;
  uint64_t sample_base;
  uint32_t subframe, estimator;
  float lens_radius, focal_distance;
};

struct Frame {
  float3 origin, direction;
  float tmax;
  unsigned int prim;
  CUdeviceptr sbt;
  unsigned int p0, p1;
};

struct Counts {
  uint64_t radiance = 0, occlusion = 0, zero_dir = 0;
};

void* g_ctx = nullptr;
const int* g_mat_indices = nullptr;
std::vector<HitGroupData> g_hit_records;  // material-major, RAY_TYPE_COUNT per material
MissData g_miss_records[RAY_TYPE_COUNT];

thread_local std::vector<Frame> t_frames;
thread_local uint3 t_launch;
thread_local Counts t_counts;

}  // namespace

// ---- OptiX device functions: definitions -------------------------------------
static unsigned int optixGetPayload_0() { return t_frames.back().p0; }
static unsigned int optixGetPayload_1() { return t_frames.back().p1; }
static CUdeviceptr optixGetSbtDataPointer() { return t_frames.back().sbt; }
static float3 optixGetWorldRayOrigin() { return t_frames.back().origin; }
static float3 optixGetWorldRayDirection() { return t_frames.back().direction; }
static float optixGetRayTmax() { return t_frames.back().tmax; }
static unsigned int optixGetPrimitiveIndex() { return t_frames.back().prim; }
static uint3 optixGetLaunchIndex() { return t_launch; }

static void optixTrace(OptixTraversableHandle, float3 origin, float3 direction, float tmin, float tmax, float,
                       OptixVisibilityMask, unsigned int, unsigned int sbt_offset, unsigned int sbt_stride,
                       unsigned int miss_index, unsigned int& p0, unsigned int& p1) {
  const bool zero = direction.x == 0.0f && direction.y == 0.0f && direction.z == 0.0f;
  if (sbt_offset == RAY_TYPE_RADIANCE) {
    ++t_counts.radiance;
    if (zero) ++t_counts.zero_dir;
  } else {
    ++t_counts.occlusion;
  }
  const float o[3] = {origin.x, origin.y, origin.z};
  const float d[3] = {direction.x, direction.y, direction.z};
  int32_t prim = -1;
  float t = 0.0f;
  oracle_ctx_closest(g_ctx, o, d, tmin, tmax, &prim, &t);
  Frame f;
  f.origin = origin;
  f.direction = direction;
  f.p0 = p0;
  f.p1 = p1;
  if (prim >= 0) {
    f.tmax = t;
    f.prim = (unsigned int)prim;
    const size_t rec = (size_t)g_mat_indices[prim] * sbt_stride + sbt_offset;
    f.sbt = reinterpret_cast<CUdeviceptr>(&g_hit_records[rec]);
  } else {
    f.tmax = tmax;
    f.prim = 0;
    f.sbt = reinterpret_cast<CUdeviceptr>(&g_miss_records[miss_index]);
  }
  t_frames.push_back(f);
  if (prim >= 0) {
    if (sbt_offset == RAY_TYPE_RADIANCE) __closesthit__radiance();
    else __closesthit__occlusion();
  } else {
    if (miss_index == RAY_TYPE_RADIANCE) __miss__radiance();
    else __miss__occlusion();
  }
  p0 = t_frames.back().p0;
  p1 = t_frames.back().p1;
  t_frames.pop_back();
}

static uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 0x100000001b3ull;
  }
  return h;
}

static uint32_t bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

// A raw soup (the arrays SceneParser produces, without text parsing), in the
// format baseline/optix_harness.cc reads: magic "LSOUP1\0\0", u32 T, M,
// width, height, spp, bounces; f32 eye[3], look_at[3], fov; f32
// vertices[9T], normals[9T]; i32 mat_indices[T]; Material[M] (40 bytes).
struct Soup {
  std::vector<float3> vertices, normals;
  std::vector<int> mat_indices;
  std::vector<Material> materials;
};

static bool load_soup(const char* path, Soup& s, RendererParams& p) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char magic[8];
  uint32_t h[6];
  float cam[7];
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "LSOUP1", 6) == 0 &&
            std::fread(h, 4, 6, f) == 6 && std::fread(cam, 4, 7, f) == 7;
  if (ok) {
    const size_t T = h[0], M = h[1];
    s.vertices.resize(3 * T);
    s.normals.resize(3 * T);
    s.mat_indices.resize(T);
    s.materials.resize(M);
    ok = std::fread(s.vertices.data(), sizeof(float3), 3 * T, f) == 3 * T &&
         std::fread(s.normals.data(), sizeof(float3), 3 * T, f) == 3 * T &&
         std::fread(s.mat_indices.data(), sizeof(int), T, f) == T &&
         std::fread(s.materials.data(), sizeof(Material), M, f) == M;
    p.vertices = s.vertices.data();
    p.normals = s.normals.data();
    p.materials = s.materials.data();
    p.mat_indices = s.mat_indices.data();
    p.num_vertices = (int)(3 * T);
    p.num_materials = (int)M;
    p.width = h[2];
    p.height = h[3];
    p.num_samples = h[4];
    p.num_bounces = h[5];
    p.camera.eye = make_float3(cam[0], cam[1], cam[2]);
    p.camera.look_at = make_float3(cam[3], cam[4], cam[5]);
    p.camera.fov = cam[6];
    p.output_image = "";
  }
  std::fclose(f);
  return ok;
}

int main(int argc, char** argv) {
  // ref_shader_run scene.rto                  per-pixel dump of the whole frame
  // ref_shader_run --soup scene.soup --spp N --rows R --band K [--threads T]
  //     times the reference's raygen over a sample of the frame: R rows
  //     spread evenly over the image, K pixels of each (starting at
  //     (row index * 97) mod (width - K)), N samples per pixel; prints one
  //     JSON line with the traces made and the seconds taken.
  const char* rto = nullptr;
  const char* soup_path = nullptr;
  int spp = -1, rows = 0, band = 0, threads = 0;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--soup" && i + 1 < argc) soup_path = argv[++i];
    else if (a == "--spp" && i + 1 < argc) spp = std::atoi(argv[++i]);
    else if (a == "--rows" && i + 1 < argc) rows = std::atoi(argv[++i]);
    else if (a == "--band" && i + 1 < argc) band = std::atoi(argv[++i]);
    else if (a == "--threads" && i + 1 < argc) threads = std::atoi(argv[++i]);
    else if (a[0] != '-' && !rto) rto = argv[i];
    else {
      std::fprintf(stderr, "usage: %s scene.rto | --soup f --spp N --rows R --band K [--threads T]\n", argv[0]);
      return 2;
    }
  }
  if (!rto == !soup_path) {
    std::fprintf(stderr, "usage: %s scene.rto | --soup f --spp N --rows R --band K [--threads T]\n", argv[0]);
    return 2;
  }
  Soup soup;
  SceneParser* parser = nullptr;
  RendererParams rp{};
  if (rto) {
    parser = new SceneParser(const_cast<char*>(rto));
    rp = parser->get_params();
  } else if (!load_soup(soup_path, soup, rp)) {
    std::fprintf(stderr, "cannot read soup %s\n", soup_path);
    return 1;
  }
  if (spp > 0) rp.num_samples = (unsigned)spp;
  if (threads > 0) omp_set_num_threads(threads);
  const uint32_t T = (uint32_t)rp.num_vertices / 3u;

  OracleScene os;
  std::memset(&os, 0, sizeof(os));
  os.vertices = reinterpret_cast<const float*>(rp.vertices);
  os.normals = reinterpret_cast<const float*>(rp.normals);
  os.num_triangles = T;
  g_ctx = oracle_ctx_create(&os, 1);
  g_mat_indices = rp.mat_indices;

  std::vector<Material> materials(rp.materials, rp.materials + rp.num_materials);
  g_hit_records.assign((size_t)RAY_TYPE_COUNT * rp.num_materials, HitGroupData{});
  for (int i = 0; i < rp.num_materials; ++i) {
    HitGroupData& r = g_hit_records[(size_t)i * RAY_TYPE_COUNT + RAY_TYPE_RADIANCE];
    r.vertices = const_cast<float3*>(rp.vertices);
    r.normals = const_cast<float3*>(rp.normals);
    r.material = &materials[i];
    g_hit_records[(size_t)i * RAY_TYPE_COUNT + RAY_TYPE_OCCLUSION].material = &materials[i];
  }
  g_miss_records[0].bg_color = make_float4(0.0f);
  g_miss_records[1].bg_color = make_float4(0.0f);

  std::vector<float4> accum((size_t)rp.width * rp.height);
  std::vector<uchar4> frame((size_t)rp.width * rp.height);
  std::memset(&params, 0, sizeof(params));
  params.width = rp.width;
  params.height = rp.height;
  params.num_bounces = rp.num_bounces;
  params.samples_per_launch = rp.num_samples;
  params.subframe_index = 0u;
  params.accum_buffer = accum.data();
  params.frame_buffer = frame.data();
  sutil::Camera cam;
  cam.setEye(rp.camera.eye);
  cam.setLookat(rp.camera.look_at);
  cam.setUp(make_float3(0.0f, 1.0f, 0.0f));
  cam.setFovY(rp.camera.fov);
  cam.setAspectRatio(static_cast<float>(rp.width) / static_cast<float>(rp.height));
  params.eye = cam.eye();
  cam.UVWFrame(params.U, params.V, params.W);

  if (soup_path) {
    // timed sample: the pixels of R rows x K columns
    std::vector<int64_t> pix;
    const int w = (int)rp.width, h = (int)rp.height;
    const int R = rows > 0 ? rows : 64, K = band > 0 ? std::min(band, w) : std::min(64, w);
    for (int b = 0; b < R; ++b) {
      const int y = R > 1 ? (int)((double)b * (h - 1) / (R - 1)) : 0;
      const int x0 = w > K ? (b * 97) % (w - K) : 0;
      for (int k = 0; k < K; ++k) pix.push_back((int64_t)y * w + x0 + k);
    }
    uint64_t rad = 0, occ = 0, zero = 0;
    const double t0 = omp_get_wtime();
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : rad, occ, zero)
    for (int64_t i = 0; i < (int64_t)pix.size(); ++i) {
      const int64_t p = pix[i];
      t_launch = make_uint3((unsigned)(p % rp.width), (unsigned)(p / rp.width), 0u);
      t_counts = Counts{};
      __raygen__rg();
      rad += t_counts.radiance;
      occ += t_counts.occlusion;
      zero += t_counts.zero_dir;
    }
    const double sec = omp_get_wtime() - t0;
    std::printf("{\"pixels\": %zu, \"spp\": %u, \"seconds\": %.6f, \"rays_radiance\": %llu, \"rays_occlusion\": "
                "%llu, \"rays_zero_direction\": %llu, \"threads\": %d}\n",
                pix.size(), rp.num_samples, sec, (unsigned long long)rad, (unsigned long long)occ,
                (unsigned long long)zero, omp_get_max_threads());
    return 0;
  }

  const int64_t npix = (int64_t)rp.width * rp.height;
  std::vector<Counts> counts(npix);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t p = 0; p < npix; ++p) {
    t_launch = make_uint3((unsigned)(p % rp.width), (unsigned)(p / rp.width), 0u);
    t_counts = Counts{};
    __raygen__rg();
    counts[p] = t_counts;
  }

  uint64_t h = 0xcbf29ce484222325ull;
  h = fnv1a(h, rp.vertices, sizeof(float3) * 3ull * T);
  h = fnv1a(h, rp.normals, sizeof(float3) * 3ull * T);
  h = fnv1a(h, rp.mat_indices, sizeof(int) * (size_t)T);
  std::printf("scene %u %d %u %u %u %u soup %016llx\n", T, rp.num_materials, rp.width, rp.height, rp.num_samples,
              rp.num_bounces, (unsigned long long)h);
  for (int64_t p = 0; p < npix; ++p) {
    const float4 a = accum[p];
    const uchar4 c = frame[p];
    std::printf("px %lld %08x %08x %08x %02x%02x%02x%02x %llu %llu %llu\n", (long long)p, bits(a.x), bits(a.y),
                bits(a.z), c.x, c.y, c.z, c.w, (unsigned long long)counts[p].radiance,
                (unsigned long long)counts[p].occlusion, (unsigned long long)counts[p].zero_dir);
  }
  delete parser;
  return 0;
}

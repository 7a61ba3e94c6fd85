// C ABI (include/lisa_gb.h) and renderer construction.
//
// Renderer construction replaces OptixWrapper (src/LiSA/src/optix_wrapper.cc):
// the soup is uploaded once (create_mesh_handler :54-82), the BVH is built on
// the GPU instead of optixAccelBuild (:92-145), the camera frame is the SDK
// camera's UVW frame (src/sutil/Camera.cpp:34-45, set up in init_params
// :434-442), and the launch state becomes the wavefront buffers.
#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "guide.cuh"
#include "lisa_device.cuh"
#include "lisa_internal.h"
#include "wavefront.cuh"

namespace lisa {

Status configure_launch(Renderer& r);

// ---- errors ---------------------------------------------------------------
static thread_local std::string g_last_error;
void set_last_error(const Status& s) { g_last_error = s.ok() ? std::string() : s.msg; }

static int ret(const Status& s) {
  set_last_error(s);
  return s.code;
}

#define API_GUARD(...)                                     \
  try {                                                     \
    __VA_ARGS__                                             \
  } catch (const std::bad_alloc&) {                         \
    return ret(Status(LISA_ERR_OOM, "host allocation failed")); \
  } catch (const std::exception& e) {                       \
    return ret(Status(LISA_ERR_INVALID, e.what()));         \
  } catch (...) {                                           \
    return ret(Status(LISA_ERR_INVALID, "unknown error"));  \
  }

// ---- CUDA context identity -------------------------------------------------
using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);

// Unique ID of the current CUDA context (the driver API through the
// runtime's entry-point query, so the library needs no libcuda link).
// *none is set when no context is current yet.
Status current_context_id(unsigned long long* id, bool* none) {
  static PfnCtxGetCurrent get_current = nullptr;
  static PfnCtxGetId get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    LISA_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1));
    LISA_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2));
    if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return Status(LISA_ERR_CUDA, "driver entry points cuCtxGetCurrent/cuCtxGetId unavailable");
    get_current = (PfnCtxGetCurrent)f1;
    get_id = (PfnCtxGetId)f2;
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS) return Status(LISA_ERR_CUDA, "cuCtxGetCurrent failed");
  *none = ctx == nullptr;
  if (*none) return Status();
  if (get_id(ctx, id) != CUDA_SUCCESS) return Status(LISA_ERR_CUDA, "cuCtxGetId failed");
  return Status();
}

// ---- device memory cache -----------------------------------------------------
// Blocks are rounded up to 64 KiB (2 MiB above 32 MiB); a request takes the
// smallest cached block of the current CUDA context that is at least as
// large and at most 1/8 + 2 MiB larger.  Blocks are keyed by context ID, not
// device ordinal: a context the application creates, or the primary context
// after a device reset, never receives another context's addresses.  The cache holds at most LISA_DEVICE_CACHE_MB (default
// 8192; 0 turns it off) of free blocks per process.  The state is never
// destroyed (no CUDA call from a static destructor at process exit).
namespace {
struct DevCache {
  std::mutex mu;
  std::unordered_map<void*, std::pair<size_t, unsigned long long>> live;  // block -> (rounded size, context)
  std::multimap<std::pair<unsigned long long, size_t>, void*> free_blocks;
  size_t free_bytes = 0;
  size_t cap = 0;
  DevCache() {
    const char* v = std::getenv("LISA_DEVICE_CACHE_MB");
    cap = (size_t)(v ? std::strtoull(v, nullptr, 10) : 8192ull) << 20;
  }
  void release_locked() {
    // (blocks of a context that is not current, or no longer exists, fail
    // to free; their records are dropped all the same)
    for (auto& kv : free_blocks)
      if (cudaFree(kv.second) != cudaSuccess) cudaGetLastError();
    free_blocks.clear();
    free_bytes = 0;
  }
};
constexpr unsigned long long NO_CTX = ~0ull;  // a block's context was not known

DevCache& dev_cache() {
  static DevCache* c = new DevCache();
  return *c;
}
size_t dev_round(size_t bytes) {
  bytes = std::max<size_t>(bytes, 16);
  const size_t g = bytes > (32ull << 20) ? (2ull << 20) : (64ull << 10);
  return (bytes + g - 1) / g * g;
}
}  // namespace

cudaError_t dev_alloc(void** p, size_t bytes) {
  DevCache& c = dev_cache();
  unsigned long long ctx = 0;
  bool none = true;
  if (!current_context_id(&ctx, &none).ok()) none = true;  // then nothing is reused
  const size_t need = dev_round(bytes);
  std::lock_guard<std::mutex> lock(c.mu);
  if (!none) {
    auto it = c.free_blocks.lower_bound({ctx, need});
    if (it != c.free_blocks.end() && it->first.first == ctx && it->first.second <= need + need / 8 + (2ull << 20)) {
      *p = it->second;
      c.live[it->second] = {it->first.second, ctx};
      c.free_bytes -= it->first.second;
      c.free_blocks.erase(it);
      return cudaSuccess;
    }
  }
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, need);
  if (e == cudaErrorMemoryAllocation && !c.free_blocks.empty()) {
    cudaGetLastError();
    c.release_locked();
    e = cudaMalloc(&q, need);
  }
  if (e != cudaSuccess) return e;
  if (none && !current_context_id(&ctx, &none).ok()) none = true;  // cudaMalloc made one current
  // a block whose context is unknown is freed, not cached
  c.live[q] = {need, none ? NO_CTX : ctx};
  *p = q;
  return cudaSuccess;
}

void dev_free(void* p) {
  if (!p) return;
  DevCache& c = dev_cache();
  std::lock_guard<std::mutex> lock(c.mu);
  auto it = c.live.find(p);
  if (it == c.live.end()) {  // not ours
    cudaFree(p);
    return;
  }
  const size_t bytes = it->second.first;
  const unsigned long long ctx = it->second.second;
  c.live.erase(it);
  if (ctx != NO_CTX && c.free_bytes + bytes <= c.cap) {
    c.free_blocks.insert({{ctx, bytes}, p});
    c.free_bytes += bytes;
  } else {
    cudaFree(p);
  }
}

size_t dev_cache_release() {
  DevCache& c = dev_cache();
  std::lock_guard<std::mutex> lock(c.mu);
  const size_t n = c.free_bytes;
  c.release_locked();
  return n;
}

// ---- arena -----------------------------------------------------------------
Status DeviceArena::alloc(void** p, size_t bytes, const char* what) {
  bytes = std::max<size_t>(bytes, 16);
  if (cap && used + bytes > cap)
    return Status(LISA_ERR_OOM, std::string("allocation cap exceeded by ") + what);
  void* q = nullptr;
  cudaError_t e = dev_alloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return Status(LISA_ERR_OOM, std::string("cudaMalloc failed for ") + what + ": " + cudaGetErrorString(e));
  }
  blocks.push_back(q);
  used += bytes;
  *p = q;
  return Status();
}

void DeviceArena::release_all() {
  for (void* p : blocks) dev_free(p);
  blocks.clear();
  used = 0;
}

Status TempDeviceBufs::get(void** p, size_t bytes, const char* what) {
  void* q = nullptr;
  cudaError_t e = dev_alloc(&q, std::max<size_t>(bytes, 16));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return Status(LISA_ERR_OOM, std::string("cudaMalloc failed for ") + what + ": " + cudaGetErrorString(e));
  }
  ptrs.push_back(q);
  *p = q;
  return Status();
}

TempDeviceBufs::~TempDeviceBufs() {
  // the blocks go back to the cache, so the work that used them must be
  // done (cudaFree used to wait for the device implicitly)
  if (!ptrs.empty()) {
    if (stream) cudaStreamSynchronize(stream);
    else cudaDeviceSynchronize();
  }
  for (void* p : ptrs) dev_free(p);
}

Status BumpScratch::get(void** p, size_t bytes, const char* what) {
  const size_t need = (std::max<size_t>(bytes, 16) + 255) & ~(size_t)255;
  if (used + need > size) return Status(LISA_ERR_OOM, std::string("scratch region too small for ") + what);
  *p = base + used;
  used += need;
  return Status();
}

Renderer::~Renderer() {
  if (stream) cudaStreamSynchronize(stream);
  for (auto e : ev_pool) cudaEventDestroy(e);
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (d_waves) cudaFree(d_waves);
  guides.clear();
  arena.release_all();
  if (stream) cudaStreamDestroy(stream);
}

// ---- host vector math for the camera frame (Camera.cpp:34-45) ---------------
namespace {
struct H3 {
  float x, y, z;
};
H3 hsub(H3 a, H3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
H3 hmul(H3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float hdot(H3 a, H3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
H3 hcross(H3 a, H3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
H3 hnormalize(H3 v) { return hmul(v, 1.0f / std::sqrt(hdot(v, v))); }

void camera_frame(const lisa_camera& c, uint32_t w, uint32_t h, float* eye, float* U, float* V, float* W) {
  const H3 e{c.eye.x, c.eye.y, c.eye.z}, la{c.look_at.x, c.look_at.y, c.look_at.z}, up{0.0f, 1.0f, 0.0f};
  const float aspect = (float)w / (float)h;
  H3 Wv = hsub(la, e);  // not normalised: its length is the focal length
  const float wlen = std::sqrt(hdot(Wv, Wv));
  H3 Uv = hnormalize(hcross(Wv, up));
  H3 Vv = hnormalize(hcross(Uv, Wv));
  const float vlen = wlen * std::tan(0.5f * c.fov * 3.14159265358979323846f / 180.0f);
  Vv = hmul(Vv, vlen);
  const float ulen = vlen * aspect;
  Uv = hmul(Uv, ulen);
  eye[0] = e.x; eye[1] = e.y; eye[2] = e.z;
  U[0] = Uv.x; U[1] = Uv.y; U[2] = Uv.z;
  V[0] = Vv.x; V[1] = Vv.y; V[2] = Vv.z;
  W[0] = Wv.x; W[1] = Wv.y; W[2] = Wv.z;
}

__global__ void k_pack_prims(const float* __restrict__ v, const float* __restrict__ nrm, const int32_t* __restrict__ mi,
                             uint32_t n, float4* __restrict__ out) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const float* a = v + 9ull * p;
    const float* b = nrm + 9ull * p;
    float4* o = out + 5ull * p;
    o[0] = make_float4(a[0], a[1], a[2], b[0]);
    o[1] = make_float4(a[3], a[4], a[5], b[1]);
    o[2] = make_float4(a[6], a[7], a[8], b[2]);
    o[3] = make_float4(b[3], b[4], b[5], b[6]);
    o[4] = make_float4(b[7], b[8], __int_as_float(mi[p]), 0.0f);
  }
}

DevMaterial to_dev(const lisa_material& m) {
  DevMaterial d;
  std::memset(&d, 0, sizeof(d));
  d.albedo[0] = m.diffuse_color.x;
  d.albedo[1] = m.diffuse_color.y;
  d.albedo[2] = m.diffuse_color.z;
  d.roughness = m.roughness;
  d.emission[0] = m.emission_color.x;
  d.emission[1] = m.emission_color.y;
  d.emission[2] = m.emission_color.z;
  d.ior = m.n;
  d.alpha = m.alpha;
  // shader.cu:216 tests emit first, then alpha < 1 (:226)
  d.cls = m.emit ? MAT_EMIT : (m.alpha < 1.0f ? MAT_DIELECTRIC : MAT_OPAQUE);
  return d;
}

Status validate(const lisa_renderer_params& p) {
  if (p.num_vertices < 0 || p.num_vertices % 3 != 0)
    return Status::invalid("num_vertices must be a non-negative multiple of 3");
  if (p.num_vertices > 0 && (!p.vertices || !p.normals || !p.mat_indices))
    return Status::invalid("null soup pointer");
  if (p.num_materials < 0 || (p.num_materials > 0 && !p.materials)) return Status::invalid("bad material table");
  if (p.width == 0 || p.height == 0) return Status::invalid("width and height must be positive");
  if ((uint64_t)p.width * p.height >= (1ull << 24)) return Status::invalid("at most 2^24 - 1 pixels per scene");
  const uint32_t T = (uint32_t)(p.num_vertices / 3);
  for (uint32_t i = 0; i < T; ++i)
    if (p.mat_indices[i] < 0 || p.mat_indices[i] >= p.num_materials)
      return Status::invalid("material index out of range at triangle " + std::to_string(i));
  return Status();
}
}  // namespace

// Emitters of the physically based estimator, in triangle order: every
// emissive triangle of positive area and luminance gets a record
// (v0, area pdf) (e1 = v1 - v0, material) (e2 = v2 - v0) (unit normal) and a
// CDF entry over area x luminance; each material gets its area pdf
// luminance / total.  Float steps as written (no contraction), sums in double.
Status build_emitters(Renderer& r, const lisa_renderer_params& p, SceneGpu& s, std::vector<DevMaterial>& dm) {
  const int M = p.num_materials;
  const uint32_t T = (uint32_t)(p.num_vertices / 3);
  std::vector<float> lum(std::max(M, 1), 0.0f);
  for (int m = 0; m < M; ++m)
    if (dm[m].cls == MAT_EMIT)
      lum[m] = (0.2126f * dm[m].emission[0] + 0.7152f * dm[m].emission[1]) + 0.0722f * dm[m].emission[2];
  std::vector<float4> rec;
  std::vector<double> w;
  for (uint32_t t = 0; t < T; ++t) {
    const int m = p.mat_indices[t];
    if (dm[m].cls != MAT_EMIT || !(lum[m] > 0.0f)) continue;
    const lisa_float3* v = p.vertices + 3ull * t;
    const float e1x = v[1].x - v[0].x, e1y = v[1].y - v[0].y, e1z = v[1].z - v[0].z;
    const float e2x = v[2].x - v[0].x, e2y = v[2].y - v[0].y, e2z = v[2].z - v[0].z;
    const float cx = e1y * e2z - e1z * e2y, cy = e1z * e2x - e1x * e2z, cz = e1x * e2y - e1y * e2x;
    const float len = std::sqrt(cx * cx + cy * cy + cz * cz);
    const float area = 0.5f * len;
    if (!(area > 0.0f)) continue;
    const float inv = 1.0f / len;
    int32_t mb = m;
    float mf;
    std::memcpy(&mf, &mb, 4);
    rec.push_back(make_float4(v[0].x, v[0].y, v[0].z, 0.0f));
    rec.push_back(make_float4(e1x, e1y, e1z, mf));
    rec.push_back(make_float4(e2x, e2y, e2z, 0.0f));
    rec.push_back(make_float4(cx * inv, cy * inv, cz * inv, 0.0f));
    w.push_back((double)area * (double)lum[m]);
  }
  s.num_emit = (uint32_t)w.size();
  if (!s.num_emit) return Status();
  double total = 0.0;
  for (double x : w) total += x;
  std::vector<float> cdf(s.num_emit);
  double acc = 0.0;
  for (uint32_t i = 0; i < s.num_emit; ++i) {
    acc += w[i];
    cdf[i] = (float)(acc / total);
  }
  cdf[s.num_emit - 1] = 1.0f;
  for (int m = 0; m < M; ++m) dm[m].light_pdf = (float)((double)lum[m] / total);
  for (uint32_t i = 0; i < s.num_emit; ++i) {
    int32_t m;
    std::memcpy(&m, &rec[4ull * i + 1].w, 4);
    rec[4ull * i].w = dm[m].light_pdf;
  }
  LISA_TRY(r.arena.alloc((void**)&s.emit, sizeof(float4) * rec.size(), "emitters"));
  LISA_TRY(r.arena.alloc((void**)&s.emit_cdf, sizeof(float) * cdf.size(), "emitter CDF"));
  LISA_CUDA(cudaMemcpy(s.emit, rec.data(), sizeof(float4) * rec.size(), cudaMemcpyHostToDevice));
  LISA_CUDA(cudaMemcpy(s.emit_cdf, cdf.data(), sizeof(float) * cdf.size(), cudaMemcpyHostToDevice));
  return Status();
}

// Per triangle: its material if that is an emitter, else -1 (what the BVH
// leaves carry, so the emitter search reads the class of a hit without a
// material look-up).
__global__ void k_emit_of_prim(int32_t* m, uint32_t n, const int32_t* em, uint32_t nm) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t k = (uint32_t)m[i];
    m[i] = k < nm ? em[k] : -1;
  }
}

// Leaf triangles of the emitters' own BVH carry their index among the
// emitters; make it the scene-wide triangle index (the tie rule compares
// scene-wide indices).
__global__ void k_emit_global_ids(float4* tris, uint32_t n, const int32_t* __restrict__ global) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int local = __float_as_int(tris[3ull * k].w);
    tris[3ull * k].w = __int_as_float(global[local]);
  }
}

// BVH over the scene's emissive triangles, built like the scene's (same
// builder, so the same exact traversal); leaves carry scene-wide triangle
// indices and emitter materials.
Status build_emitter_bvh(Renderer& r, const lisa_renderer_params& p, SceneGpu& s) {
  std::vector<float> ev;
  std::vector<int32_t> gid, emat;
  const uint32_t T = (uint32_t)(p.num_vertices / 3);
  for (uint32_t t = 0; t < T; ++t) {
    const int32_t m = p.mat_indices[t];
    if (m < 0 || m >= p.num_materials || !p.materials[m].emit) continue;
    for (int j = 0; j < 3; ++j) {
      const lisa_float3& v = p.vertices[3ull * t + j];
      ev.push_back(v.x);
      ev.push_back(v.y);
      ev.push_back(v.z);
    }
    gid.push_back((int32_t)t);
    emat.push_back(m);
  }
  const uint32_t ne = (uint32_t)gid.size();
  if (ne < EMIT_BVH_MIN_TRIS) return Status();  // the emitter search would not use it
  float* d_ev = nullptr;
  int32_t *d_gid = nullptr, *d_emat = nullptr;
  cudaError_t e = dev_alloc((void**)&d_ev, sizeof(float) * ev.size());
  if (e == cudaSuccess) e = dev_alloc((void**)&d_gid, sizeof(int32_t) * ne);
  if (e == cudaSuccess) e = dev_alloc((void**)&d_emat, sizeof(int32_t) * ne);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_ev, ev.data(), sizeof(float) * ev.size(), cudaMemcpyHostToDevice, r.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_gid, gid.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice, r.stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_emat, emat.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice, r.stream);
  Status st = e == cudaSuccess ? Status() : Status::cuda(e, "emitter BVH upload");
  if (st.ok()) {
    TempDeviceBufs tmp;
    tmp.stream = r.stream;
    st = build_bvh(d_ev, ne, r.stream, tmp, r.arena, &s.enodes, &s.etris, &s.ebvh, d_emat, r.opts.bvh_lbvh_only == 0);
    if (st.ok()) {
      k_emit_global_ids<<<r.sm_count * 4, 256, 0, r.stream>>>(s.etris, ne, d_gid);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaStreamSynchronize(r.stream);
      if (e != cudaSuccess) st = Status::cuda(e, "emitter BVH indices");
    }
  }
  cudaStreamSynchronize(r.stream);  // before the blocks are reused
  dev_free(d_ev);
  dev_free(d_gid);
  dev_free(d_emat);
  return st;
}

Status create_scene(Renderer& r, const lisa_renderer_params& p, SceneGpu& s) {
  LISA_TRY(validate(p));
  s.params = p;
  s.output_image = p.output_image ? p.output_image : "";
  s.params.output_image = nullptr;
  s.params.vertices = nullptr;
  s.params.normals = nullptr;
  s.params.materials = nullptr;
  s.params.mat_indices = nullptr;
  s.num_prims = (uint32_t)(p.num_vertices / 3);
  s.npix = p.width * p.height;
  const uint32_t T = s.num_prims;
  // upload the soup (72 B + 4 B per triangle) and pack the shading records
  float *d_v = nullptr, *d_n = nullptr;
  int32_t* d_m = nullptr;
  if (T) {
    LISA_CUDA(dev_alloc((void**)&d_v, sizeof(float) * 9ull * T));
    LISA_CUDA(dev_alloc((void**)&d_n, sizeof(float) * 9ull * T));
    LISA_CUDA(dev_alloc((void**)&d_m, sizeof(int32_t) * T));
    LISA_CUDA(cudaMemcpyAsync(d_v, p.vertices, sizeof(float) * 9ull * T, cudaMemcpyHostToDevice, r.stream));
    LISA_CUDA(cudaMemcpyAsync(d_n, p.normals, sizeof(float) * 9ull * T, cudaMemcpyHostToDevice, r.stream));
    LISA_CUDA(cudaMemcpyAsync(d_m, p.mat_indices, sizeof(int32_t) * T, cudaMemcpyHostToDevice, r.stream));
    LISA_TRY(r.arena.alloc((void**)&s.prims, sizeof(float4) * 5ull * T, "triangle records"));
    k_pack_prims<<<r.sm_count * 8, 256, 0, r.stream>>>(d_v, d_n, d_m, T, s.prims);
    cudaError_t e = cudaGetLastError();
    // then d_m becomes what the BVH leaves carry: the emitter material or -1
    std::vector<int32_t> em(std::max(p.num_materials, 1), -1);
    for (int i = 0; i < p.num_materials; ++i) em[i] = p.materials[i].emit ? i : -1;
    int32_t* d_em = nullptr;
    if (e == cudaSuccess) e = dev_alloc((void**)&d_em, sizeof(int32_t) * em.size());
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_em, em.data(), sizeof(int32_t) * em.size(), cudaMemcpyHostToDevice, r.stream);
    if (e == cudaSuccess) {
      k_emit_of_prim<<<r.sm_count * 8, 256, 0, r.stream>>>(d_m, T, d_em, (uint32_t)em.size());
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(r.stream);
    if (e != cudaSuccess) {
      cudaDeviceSynchronize();  // before the blocks are reused
      dev_free(d_em);
      dev_free(d_v);
      dev_free(d_n);
      dev_free(d_m);
      return Status::cuda(e, "pack triangles");
    }
    dev_free(d_em);
  }
  Status st;
  {
    TempDeviceBufs tmp;
    tmp.stream = r.stream;
    st = build_bvh(d_v, T, r.stream, tmp, r.arena, &s.nodes, &s.tris, &s.bvh, d_m, r.opts.bvh_lbvh_only == 0);
    cudaStreamSynchronize(r.stream);
  }
  dev_free(d_v);
  dev_free(d_n);
  dev_free(d_m);
  LISA_TRY(st);
  const float dx = s.bvh.bmax[0] - s.bvh.bmin[0], dy = s.bvh.bmax[1] - s.bvh.bmin[1],
              dz = s.bvh.bmax[2] - s.bvh.bmin[2];
  s.extent = std::sqrt(dx * dx + dy * dy + dz * dz);
  if (!(s.extent > 0.0f) || !std::isfinite(s.extent)) s.extent = 1.0f;
  // bounds of the emissive triangles, padded by 1e-4 of the scene diagonal
  // (far more than the triangle test's rounding outside an edge): an
  // emitter-search ray that misses them cannot end on an emitter
  {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    bool any = false;
    for (uint32_t t = 0; t < T; ++t) {
      const int32_t m = p.mat_indices[t];
      if (m < 0 || m >= p.num_materials || !p.materials[m].emit) continue;
      any = true;
      for (int j = 0; j < 3; ++j) {
        const lisa_float3& v = p.vertices[3ull * t + j];
        const float c[3] = {v.x, v.y, v.z};
        for (int k = 0; k < 3; ++k) {
          lo[k] = std::min(lo[k], c[k]);
          hi[k] = std::max(hi[k], c[k]);
        }
      }
    }
    s.has_emit_box = any;
    const float pad = 1e-4f * s.extent;
    for (int k = 0; k < 3; ++k) {
      s.emit_lo[k] = any ? lo[k] - pad : 0.0f;
      s.emit_hi[k] = any ? hi[k] + pad : 0.0f;
    }
  }
  // the emitters' own BVH (reference estimator's emitter search)
  if (r.opts.estimator != LISA_ESTIMATOR_PHYSICAL && s.has_emit_box) LISA_TRY(build_emitter_bvh(r, p, s));
  // materials
  std::vector<DevMaterial> dm(std::max(p.num_materials, 1));
  for (int i = 0; i < p.num_materials; ++i) dm[i] = to_dev(p.materials[i]);
  if (r.opts.estimator == LISA_ESTIMATOR_PHYSICAL) LISA_TRY(build_emitters(r, p, s, dm));
  LISA_TRY(r.arena.alloc((void**)&s.mats, sizeof(DevMaterial) * dm.size(), "materials"));
  LISA_CUDA(cudaMemcpyAsync(s.mats, dm.data(), sizeof(DevMaterial) * dm.size(), cudaMemcpyHostToDevice, r.stream));
  // accumulation
  LISA_TRY(r.arena.alloc((void**)&s.acc_sum, sizeof(float4) * s.npix, "accumulation"));
  LISA_TRY(r.arena.alloc((void**)&s.acc_comp, sizeof(float4) * s.npix, "accumulation"));
  LISA_TRY(r.arena.alloc((void**)&s.acc_sq, sizeof(double) * 3ull * s.npix, "variance"));
  if (r.opts.accum_fp64) LISA_TRY(r.arena.alloc((void**)&s.acc_sum64, sizeof(double) * 3ull * s.npix, "fp64 mean"));
  if (r.opts.rng == LISA_RNG_PER_PIXEL)
    LISA_TRY(r.arena.alloc((void**)&s.pix_rng, sizeof(uint32_t) * s.npix, "pixel rng"));
  LISA_CUDA(cudaMemsetAsync(s.acc_sum, 0, sizeof(float4) * s.npix, r.stream));
  LISA_CUDA(cudaMemsetAsync(s.acc_comp, 0, sizeof(float4) * s.npix, r.stream));
  LISA_CUDA(cudaMemsetAsync(s.acc_sq, 0, sizeof(double) * 3ull * s.npix, r.stream));
  if (s.acc_sum64) LISA_CUDA(cudaMemsetAsync(s.acc_sum64, 0, sizeof(double) * 3ull * s.npix, r.stream));
  camera_frame(p.camera, p.width, p.height, s.eye, s.U, s.V, s.W);
  return Status();
}

SceneDev scene_dev(const Renderer& r, const SceneGpu& s) {
  SceneDev d;
  std::memset(&d, 0, sizeof(d));
  d.nodes = s.nodes;
  d.tris = s.tris;
  d.prims = s.prims;
  d.mats = s.mats;
  d.num_prims = s.num_prims;
  d.num_nodes = s.bvh.num_nodes;
  d.enodes = s.enodes;
  d.etris = s.etris;
  d.num_enodes = s.enodes ? s.ebvh.num_nodes : 0u;
  d.num_etris = s.enodes ? s.ebvh.num_tri_slots : 0u;
  d.num_mats = (uint32_t)std::max(s.params.num_materials, 0);
  d.extent = s.extent;
  d.width = s.params.width;
  d.height = s.params.height;
  d.num_bounces = s.params.num_bounces;
  d.has_emit_box = s.has_emit_box ? 1u : 0u;
  for (int k = 0; k < 3; ++k) {
    d.emit_lo[k] = s.emit_lo[k];
    d.emit_hi[k] = s.emit_hi[k];
  }
  for (int k = 0; k < 3; ++k) {
    d.eye[k] = s.eye[k];
    d.U[k] = s.U[k];
    d.V[k] = s.V[k];
    d.W[k] = s.W[k];
    d.bmin[k] = s.bvh.bmin[k];
    d.bmax[k] = s.bvh.bmax[k];
  }
  d.lens_radius = r.opts.aperture;
  const float ul = std::sqrt(s.U[0] * s.U[0] + s.U[1] * s.U[1] + s.U[2] * s.U[2]);
  const float vl = std::sqrt(s.V[0] * s.V[0] + s.V[1] * s.V[1] + s.V[2] * s.V[2]);
  const float wl = std::sqrt(s.W[0] * s.W[0] + s.W[1] * s.W[1] + s.W[2] * s.W[2]);
  for (int k = 0; k < 3; ++k) {
    d.unitU[k] = ul > 0 ? s.U[k] / ul : 0.0f;
    d.unitV[k] = vl > 0 ? s.V[k] / vl : 0.0f;
    d.unitW[k] = wl > 0 ? s.W[k] / wl : 0.0f;
  }
  d.focal_distance = r.opts.focal_distance > 0.0f ? r.opts.focal_distance : wl;
  d.acc_sum = s.acc_sum;
  d.acc_comp = s.acc_comp;
  d.acc_sq = s.acc_sq;
  d.acc_sum64 = s.acc_sum64;
  d.pix_rng = s.pix_rng;
  d.guide = s.guide;
  d.emit = s.emit;
  d.emit_cdf = s.emit_cdf;
  d.num_emit = s.num_emit;
  return d;
}

Status renderer_create(const lisa_renderer_params* scenes, int n, const lisa_options* opts, Renderer** out) {
  if (!scenes || n <= 0 || !out) return Status::invalid("no scenes");
  if (n > 255) return Status::invalid("at most 255 scenes per renderer");
  std::unique_ptr<Renderer> r(new Renderer());
  lisa_options_default(&r->opts);
  if (opts) {
    if (opts->struct_size != sizeof(lisa_options)) return Status::invalid("lisa_options.struct_size mismatch");
    r->opts = *opts;
  }
  if (r->opts.mode > LISA_MODE_GUIDED) return Status::invalid("unknown mode");
  if (r->opts.rng > LISA_RNG_PER_PIXEL) return Status::invalid("unknown rng mode");
  if (r->opts.estimator > LISA_ESTIMATOR_PHYSICAL) return Status::invalid("unknown estimator");
  // the persistent traversal kernels work on whole warps, at most 4 per block
  if (r->opts.threads_per_block % 32u || r->opts.threads_per_block > 128u)
    return Status::invalid("threads_per_block: 0 (auto) or a multiple of 32 up to 128");
  if (r->opts.refill_idle > 32u) return Status::invalid("refill_idle: 0 (default) or 1..32");
  r->arena.cap = r->opts.alloc_cap_bytes;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return Status(LISA_ERR_UNSUPPORTED, "no CUDA device");
  }
  LISA_CUDA(cudaGetDevice(&r->device));
  cudaDeviceProp prop;
  LISA_CUDA(cudaGetDeviceProperties(&prop, r->device));
  if (prop.major < 10) return Status(LISA_ERR_UNSUPPORTED, "needs a Blackwell (sm_10x) GPU");
  r->sm_count = prop.multiProcessorCount;
  LISA_CUDA(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking));
  r->scenes.resize(n);
  uint64_t total_paths = 0;
  for (int i = 0; i < n; ++i) {
    LISA_TRY(create_scene(*r, scenes[i], r->scenes[i]));
    total_paths += (uint64_t)r->scenes[i].npix * std::max<uint32_t>(scenes[i].num_samples, 1);
  }
  // wavefront capacity
  // default: 16 Mi paths (2.6 GB of queues; larger waves mean fewer launches
  // and shorter tails: the 1024x1024 16-spp icosphere frame takes 45.4 ms in
  // 4 Mi waves, 38.5 ms in one 16 Mi wave); guided mode keeps 4 Mi, the
  // wave its training schedule is set for
  uint64_t W = r->opts.paths_in_flight ? r->opts.paths_in_flight
                                       : (r->opts.mode == LISA_MODE_GUIDED ? (1ull << 22) : (1ull << 24));
  W = std::min<uint64_t>(W, std::max<uint64_t>(total_paths, 1));
  W = std::max<uint64_t>(W, 32);
  if (W > (1ull << 30)) return Status::invalid("paths_in_flight too large");
  r->capacity = (uint32_t)W;
  for (int k = 0; k < 2; ++k) {
    LISA_TRY(r->arena.alloc((void**)&r->ro[k], sizeof(float4) * W, "ray queue"));
    LISA_TRY(r->arena.alloc((void**)&r->rd[k], sizeof(float4) * W, "ray queue"));
  }
  LISA_TRY(r->arena.alloc((void**)&r->hit, sizeof(int2) * W, "hit queue"));
  LISA_TRY(r->arena.alloc((void**)&r->ps_att, sizeof(float4) * W, "path state"));
  LISA_TRY(r->arena.alloc((void**)&r->ps_col, sizeof(float4) * W, "path state"));
  LISA_TRY(r->arena.alloc((void**)&r->ps_rng, sizeof(uint32_t) * W, "path state"));
  LISA_TRY(r->arena.alloc((void**)&r->nee_a, sizeof(float4) * W, "emitter queue"));
  LISA_TRY(r->arena.alloc((void**)&r->nee_b, sizeof(float4) * W, "emitter queue"));
  LISA_TRY(r->arena.alloc((void**)&r->nee_c, sizeof(float4) * W, "emitter queue"));
  LISA_TRY(r->arena.alloc((void**)&r->ctrl, sizeof(WaveCtrl), "control block"));
  LISA_CUDA(cudaMemsetAsync(r->ctrl, 0, sizeof(WaveCtrl), r->stream));
  if (r->opts.mode == LISA_MODE_GUIDED) LISA_TRY(guide_renderer_init(*r));
  std::vector<SceneDev> sd(n);
  for (int i = 0; i < n; ++i) sd[i] = scene_dev(*r, r->scenes[i]);
  LISA_TRY(r->arena.alloc((void**)&r->d_scenes, sizeof(SceneDev) * n, "scene table"));
  LISA_CUDA(cudaMemcpyAsync(r->d_scenes, sd.data(), sizeof(SceneDev) * n, cudaMemcpyHostToDevice, r->stream));
  LISA_TRY(configure_launch(*r));
  LISA_CUDA(cudaStreamSynchronize(r->stream));
  *out = r.release();
  return Status();
}

// ---- PPM (sutil.cpp:97-117, 523-553) ------------------------------------------
Status write_ppm_rgb8_flipped(const char* path, const uint8_t* rgb8, uint32_t w, uint32_t h) {
  if (!path || !rgb8 || w < 1 || h < 1) return Status::invalid("savePPM: Image is ill-formed. Not saving");
  const std::string fn(path);
  if (fn.size() < 5) return Status::invalid("saveImage(): Failed to determine filename extension");
  const std::string ext = fn.substr(fn.size() - 3);
  if (ext != "ppm" && ext != "PPM") return Status::invalid("saveImage(): only .ppm output is supported");
  FILE* f = std::fopen(path, "wb");
  if (!f) return Status::io("savePPM: Could not open file for writing: " + fn);
  std::fprintf(f, "P6\n%u %u\n255\n", w, h);
  const size_t n = 3ull * w * h;
  const size_t wrote = std::fwrite(rgb8, 1, n, f);
  std::fclose(f);
  if (wrote != n) return Status::io("savePPM: short write");
  return Status();
}

Status write_ppm_rgba8(const char* path, const uint8_t* rgba8, uint32_t w, uint32_t h) {
  if (!rgba8 || w < 1 || h < 1) return Status::invalid("savePPM: Image is ill-formed. Not saving");
  std::vector<uint8_t> pix(3ull * w * h);
  for (int64_t j = (int64_t)h - 1; j >= 0; --j)
    for (uint32_t i = 0; i < w; ++i) {
      const size_t dst = 3ull * w * (h - j - 1) + 3ull * i;
      const size_t src = 4ull * w * j + 4ull * i;
      pix[dst] = rgba8[src];
      pix[dst + 1] = rgba8[src + 1];
      pix[dst + 2] = rgba8[src + 2];
    }
  return write_ppm_rgb8_flipped(path, pix.data(), w, h);
}

}  // namespace lisa

// ===========================================================================
// extern "C"
using namespace lisa;

struct lisa_scene {
  Scene s;
};
struct lisa_renderer {
  Renderer* r;
};

extern "C" {

const char* lisa_last_error(void) { return g_last_error.c_str(); }

const char* lisa_version(void) { return "lisa_gb300 1.0 (sm_103a)"; }

int lisa_device_cache_release(uint64_t* bytes) {
  API_GUARD({
    const size_t n = dev_cache_release();
    if (bytes) *bytes = n;
    return ret(Status());
  });
}

int lisa_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  API_GUARD({
    int dev = 0, n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
      cudaGetLastError();
      return ret(Status(LISA_ERR_UNSUPPORTED, "no CUDA device"));
    }
    cudaDeviceProp p;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess || (e = cudaGetDeviceProperties(&p, dev)) != cudaSuccess)
      return ret(Status::cuda(e, "device query"));
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
    return ret(Status());
  })
}

int lisa_scene_parse(const char* rto_path, lisa_scene** out) {
  API_GUARD({
    if (!rto_path || !out) return ret(Status::invalid("null argument"));
    std::unique_ptr<lisa_scene> sc(new lisa_scene());
    Status s = parse_scene_file(rto_path, sc->s);
    if (!s.ok()) return ret(s);
    *out = sc.release();
    return ret(Status());
  })
}

int lisa_scene_parse_string(const char* text, size_t len, const char* base_dir, lisa_scene** out) {
  API_GUARD({
    if (!text || !out) return ret(Status::invalid("null argument"));
    std::unique_ptr<lisa_scene> sc(new lisa_scene());
    Status s = parse_scene_text(std::string(text, len), base_dir ? base_dir : "", sc->s);
    if (!s.ok()) return ret(s);
    *out = sc.release();
    return ret(Status());
  })
}

int lisa_scene_params(const lisa_scene* scene, lisa_renderer_params* out) {
  API_GUARD({
    if (!scene || !out) return ret(Status::invalid("null argument"));
    scene_fill_params(scene->s, out);
    return ret(Status());
  })
}

void lisa_scene_destroy(lisa_scene* scene) { delete scene; }

int lisa_scene_create_empty(lisa_scene** out) {
  API_GUARD({
    if (!out) return ret(Status::invalid("null argument"));
    *out = new lisa_scene();
    return ret(Status());
  })
}

int lisa_scene_append_obj(lisa_scene* scene, const char* obj_path, int32_t mat_idx) {
  API_GUARD({
    if (!scene || !obj_path) return ret(Status::invalid("null argument"));
    return ret(obj_append(scene->s, obj_path, mat_idx));
  })
}

void lisa_options_default(lisa_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->struct_size = sizeof(lisa_options);
  o->mode = LISA_MODE_COMPAT;
  o->rng = LISA_RNG_PER_SAMPLE;
  o->use_graph = 1;
  o->guide_bsdf_fraction = 0.5f;
  // 128 Adam steps of one 128-sample tile per SM (19,456 samples on 152
  // SMs) per 4 Mi paths at lr 1e-3, up to 2048 steps per scene, after 2
  // warm-up waves, with at most 16 spp per wave
  o->guide_lr = 1e-3f;
  o->guide_train_batch = 0;
  o->guide_warmup_waves = 2;
  o->guide_steps_per_wave = 128;
  o->guide_spp_per_wave = 16;
  o->guide_min_spp = 256;  // below that, warm-up waves would take most of the render
  o->guide_train_steps = 2048;
}

int lisa_renderer_create(const lisa_renderer_params* params, const lisa_options* opts, lisa_renderer** out) {
  return lisa_renderer_create_batch(params, 1, opts, out);
}

int lisa_renderer_create_batch(const lisa_renderer_params* scenes, int32_t n, const lisa_options* opts,
                               lisa_renderer** out) {
  API_GUARD({
    if (!out) return ret(Status::invalid("null argument"));
    Renderer* r = nullptr;
    Status s = renderer_create(scenes, n, opts, &r);
    if (!s.ok()) return ret(s);
    *out = new lisa_renderer{r};
    return ret(Status());
  })
}

void lisa_renderer_destroy(lisa_renderer* r) {
  if (!r) return;
  delete r->r;
  delete r;
}

int lisa_render(lisa_renderer* r, lisa_render_stats* stats) {
  API_GUARD({
    if (!r) return ret(Status::invalid("null renderer"));
    return ret(renderer_render(*r->r, 0, false, stats));
  })
}

int lisa_batch_render(const lisa_renderer_params* scenes, int32_t n, const lisa_options* opts,
                      lisa_render_stats* stats) {
  API_GUARD({
    Renderer* raw = nullptr;
    Status s = renderer_create(scenes, n, opts, &raw);
    if (!s.ok()) return ret(s);
    std::unique_ptr<Renderer> r(raw);
    s = renderer_render(*r, 0, false, stats);
    for (int i = 0; s.ok() && i < n; ++i) {
      SceneGpu& sg = r->scenes[i];
      if (sg.output_image.empty()) continue;
      std::vector<uint8_t> rgb(3ull * sg.npix);
      s = renderer_get_ppm(*r, i, rgb.data());
      if (s.ok()) s = write_ppm_rgb8_flipped(sg.output_image.c_str(), rgb.data(), sg.params.width, sg.params.height);
    }
    return ret(s);
  })
}

int lisa_render_progressive(lisa_renderer* r, uint32_t spp, lisa_render_stats* stats) {
  API_GUARD({
    if (!r) return ret(Status::invalid("null renderer"));
    if (spp == 0) return ret(Status::invalid("spp must be positive"));
    return ret(renderer_render(*r->r, spp, true, stats));
  })
}

int lisa_reset_accumulation(lisa_renderer* r) {
  API_GUARD({
    if (!r) return ret(Status::invalid("null renderer"));
    return ret(renderer_reset(*r->r));
  })
}

int lisa_set_sample_offset(lisa_renderer* r, int32_t scene, uint64_t first_sample) {
  API_GUARD({
    if (!r) return ret(Status::invalid("null renderer"));
    Renderer& R = *r->r;
    if (scene < 0 || scene >= (int)R.scenes.size()) return ret(Status::invalid("scene index out of range"));
    if (first_sample > 0xffffffffull) return ret(Status::invalid("sample index beyond 2^32"));
    R.scenes[scene].sample_offset = first_sample;
    R.scenes[scene].next_sample = first_sample;
    return ret(Status());
  })
}

int lisa_get_image(lisa_renderer* r, int32_t scene, float* rgb32, uint8_t* rgba8, double* var, double* mean64) {
  API_GUARD({
    if (!r) return ret(Status::invalid("null renderer"));
    return ret(renderer_get_image(*r->r, scene, rgb32, rgba8, var, mean64));
  })
}

int lisa_get_ppm_rgb8(lisa_renderer* r, int32_t scene, uint8_t* rgb8) {
  API_GUARD({
    if (!r || !rgb8) return ret(Status::invalid("null argument"));
    return ret(renderer_get_ppm(*r->r, scene, rgb8));
  })
}

int lisa_save_image(lisa_renderer* r, int32_t scene, const char* path) {
  API_GUARD({
    if (!r) return ret(Status::invalid("null renderer"));
    Renderer& R = *r->r;
    if (scene < 0 || scene >= (int)R.scenes.size()) return ret(Status::invalid("scene index out of range"));
    SceneGpu& s = R.scenes[scene];
    std::vector<uint8_t> rgb(3ull * s.npix);
    Status st = renderer_get_ppm(R, scene, rgb.data());
    if (!st.ok()) return ret(st);
    const std::string p = path ? std::string(path) : s.output_image;
    return ret(write_ppm_rgb8_flipped(p.c_str(), rgb.data(), s.params.width, s.params.height));
  })
}

int lisa_write_ppm(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height) {
  API_GUARD({ return ret(write_ppm_rgba8(path, rgba8, width, height)); })
}

int lisa_trace_closest(lisa_renderer* r, const float* rays, uint32_t n, int32_t* prim, float* t) {
  API_GUARD({
    if (!r || (n && (!rays || !prim || !t))) return ret(Status::invalid("null argument"));
    if (n == 0) return ret(Status());
    Renderer& R = *r->r;
    float* d_r = nullptr;
    int32_t* d_p = nullptr;
    float* d_t = nullptr;
    Status s;
    auto run = [&]() -> Status {
      LISA_CUDA(cudaMalloc(&d_r, sizeof(float) * 8ull * n));
      LISA_CUDA(cudaMalloc(&d_p, sizeof(int32_t) * n));
      LISA_CUDA(cudaMalloc(&d_t, sizeof(float) * n));
      LISA_CUDA(cudaMemcpyAsync(d_r, rays, sizeof(float) * 8ull * n, cudaMemcpyHostToDevice, R.stream));
      LISA_TRY(trace_rays(R, d_r, n, d_p, d_t, R.stream, false));
      LISA_CUDA(cudaMemcpyAsync(prim, d_p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, R.stream));
      LISA_CUDA(cudaMemcpyAsync(t, d_t, sizeof(float) * n, cudaMemcpyDeviceToHost, R.stream));
      LISA_CUDA(cudaStreamSynchronize(R.stream));
      return Status();
    };
    s = run();
    if (d_r) cudaFree(d_r);
    if (d_p) cudaFree(d_p);
    if (d_t) cudaFree(d_t);
    return ret(s);
  })
}

int lisa_trace_closest_device(lisa_renderer* r, const float* d_rays, uint32_t n, int32_t* d_prim, float* d_t,
                              void* stream) {
  API_GUARD({
    if (!r || (n && (!d_rays || !d_prim || !d_t))) return ret(Status::invalid("null argument"));
    Renderer& R = *r->r;
    return ret(trace_rays(R, d_rays, n, d_prim, d_t, stream ? (cudaStream_t)stream : R.stream, false));
  })
}

int lisa_trace_brute_device(lisa_renderer* r, const float* d_rays, uint32_t n, int32_t* d_prim, float* d_t,
                            void* stream) {
  API_GUARD({
    if (!r || (n && (!d_rays || !d_prim || !d_t))) return ret(Status::invalid("null argument"));
    Renderer& R = *r->r;
    return ret(trace_rays(R, d_rays, n, d_prim, d_t, stream ? (cudaStream_t)stream : R.stream, true));
  })
}

int lisa_trace_count(lisa_renderer* r, const float* rays, uint32_t n, uint64_t* node_visits, uint64_t* tri_tests) {
  API_GUARD({
    if (!r || !node_visits || !tri_tests || (n && !rays)) return ret(Status::invalid("null argument"));
    Renderer& R = *r->r;
    float* d_r = nullptr;
    auto run = [&]() -> Status {
      LISA_CUDA(cudaMalloc(&d_r, sizeof(float) * 8ull * std::max<uint32_t>(n, 1)));
      if (n) LISA_CUDA(cudaMemcpyAsync(d_r, rays, sizeof(float) * 8ull * n, cudaMemcpyHostToDevice, R.stream));
      return trace_count(R, d_r, n, node_visits, tri_tests);
    };
    Status s = run();
    if (d_r) cudaFree(d_r);
    return ret(s);
  })
}

int lisa_renderer_guide(lisa_renderer* r, int32_t scene, lisa_guide** out) {
  API_GUARD({
    if (!r || !out) return ret(Status::invalid("null argument"));
    Renderer& R = *r->r;
    if (scene < 0 || scene >= (int)R.scenes.size()) return ret(Status::invalid("scene index out of range"));
    if (R.scenes[scene].guide < 0) return ret(Status::invalid("renderer is not in guided mode"));
    lisa_guide* g = new lisa_guide();
    g->borrowed = R.guides[R.scenes[scene].guide].get();
    g->stream = R.stream;
    g->owns_stream = false;
    *out = g;
    return ret(Status());
  })
}

int lisa_bvh_info(lisa_renderer* r, int32_t scene, uint32_t* nodes, uint32_t* tri_slots, uint32_t* depth,
                  double* build_ms) {
  API_GUARD({
    if (!r) return ret(Status::invalid("null renderer"));
    Renderer& R = *r->r;
    if (scene < 0 || scene >= (int)R.scenes.size()) return ret(Status::invalid("scene index out of range"));
    const BvhBuildResult& b = R.scenes[scene].bvh;
    if (nodes) *nodes = b.num_nodes;
    if (tri_slots) *tri_slots = b.num_tri_slots;
    if (depth) *depth = b.depth;
    if (build_ms) *build_ms = b.build_ms;
    return ret(Status());
  })
}

}  // extern "C"

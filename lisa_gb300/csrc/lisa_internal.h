// Host-side internals shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/lisa_gb.h"

namespace lisa {

// ---- status ---------------------------------------------------------------
struct Status {
  int code = LISA_OK;
  std::string msg;
  Status() = default;
  Status(int c, std::string m) : code(c), msg(std::move(m)) {}
  bool ok() const { return code == LISA_OK; }
  static Status invalid(const std::string& m) { return Status(LISA_ERR_INVALID, m); }
  static Status parse(const std::string& m) { return Status(LISA_ERR_PARSE, m); }
  static Status io(const std::string& m) { return Status(LISA_ERR_IO, m); }
  static Status cuda(cudaError_t e, const char* what) {
    return Status(e == cudaErrorMemoryAllocation ? LISA_ERR_OOM : LISA_ERR_CUDA,
                  std::string(what) + ": " + cudaGetErrorString(e));
  }
};

#define LISA_CUDA(call)                                       \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::lisa::Status::cuda(e_, #call); \
  } while (0)

#define LISA_TRY(expr)              \
  do {                              \
    ::lisa::Status s_ = (expr);     \
    if (!s_.ok()) return s_;        \
  } while (0)

// ---- parsed scene (host) ---------------------------------------------------
struct Scene {
  std::vector<lisa_float3> vertices;
  std::vector<lisa_float3> normals;
  std::vector<lisa_material> materials;
  std::vector<int32_t> mat_indices;
  uint32_t width = 0, height = 0, num_samples = 0, num_bounces = 0;
  lisa_camera camera{};
  std::string output_image;
  std::map<std::string, int> mat_name_idx;
};

Status parse_scene_file(const std::string& path, Scene& sc);
Status parse_scene_text(const std::string& raw, const std::string& base_dir, Scene& sc);
Status obj_append(Scene& sc, const std::string& path, int32_t mat_idx);
void scene_fill_params(const Scene& sc, lisa_renderer_params* p);
Status write_ppm_rgba8(const char* path, const uint8_t* rgba8, uint32_t w, uint32_t h);
Status write_ppm_rgb8_flipped(const char* path, const uint8_t* rgb8, uint32_t w, uint32_t h);

// ---- device memory sources ---------------------------------------------------
// Device memory for the library's buffers.  Freed blocks are kept for
// reuse (per device, up to a cap) instead of being returned with cudaFree:
// cudaMalloc and cudaFree are synchronous and take milliseconds at the
// renderer's sizes, which a create-render-destroy cycle pays every time.
// A block may be freed only once the work that used it has finished (the
// callers synchronise their stream first).  dev_alloc returns
// cudaErrorMemoryAllocation after dropping the cache and retrying once.
// Unique ID of the current CUDA context (*none when no context is current).
Status current_context_id(unsigned long long* id, bool* none);
cudaError_t dev_alloc(void** p, size_t bytes);
void dev_free(void* p);
size_t dev_cache_release();  // cudaFree every cached block; the bytes freed

// Where a builder takes its device buffers from: cudaMalloc (DeviceArena,
// TempDeviceBufs) or a caller-provided region (BumpScratch).
struct ScratchSource {
  virtual Status get(void** p, size_t bytes, const char* what) = 0;
  virtual ~ScratchSource() = default;
};

// cudaMalloc with an optional cap; blocks live until release_all().
struct DeviceArena : ScratchSource {
  uint64_t cap = 0;
  uint64_t used = 0;
  std::vector<void*> blocks;
  Status alloc(void** p, size_t bytes, const char* what);
  Status get(void** p, size_t bytes, const char* what) override { return alloc(p, bytes, what); }
  void release_all();
  ~DeviceArena() override { release_all(); }
};

// cudaMalloc'd temporaries freed when the object goes out of scope.
struct TempDeviceBufs : ScratchSource {
  std::vector<void*> ptrs;
  cudaStream_t stream = nullptr;  // the work using the buffers (null: the whole device)
  Status get(void** p, size_t bytes, const char* what) override;
  ~TempDeviceBufs() override;
};

// Carves 256-byte aligned pieces out of one existing device region.
struct BumpScratch : ScratchSource {
  char* base = nullptr;
  size_t size = 0, used = 0;
  BumpScratch(void* b, size_t s) : base((char*)b), size(s) {}
  Status get(void** p, size_t bytes, const char* what) override;
};

// ---- BVH ------------------------------------------------------------------
struct BvhBuildResult {
  uint32_t num_nodes = 0;
  uint32_t num_tri_slots = 0;
  uint32_t depth = 0;
  double build_ms = 0.0;
  float bmin[3], bmax[3];
};

// Builds the 8-wide compressed BVH of `num_prims` triangles whose vertices
// are d_verts (3 float3 per triangle, device).  Temporaries come from `tmp`,
// the node and leaf-triangle arrays from `out`.  With d_mat (one material
// index per triangle, device) each leaf triangle also carries its material.
// With refine, the binary LBVH is restructured by SAH (treelets) before the
// 8-wide collapse.
Status build_bvh(const float* d_verts, uint32_t num_prims, cudaStream_t stream, ScratchSource& tmp,
                 ScratchSource& out, uint4** d_nodes, float4** d_tris, BvhBuildResult* info,
                 const int32_t* d_mat = nullptr, bool refine = true);
// Device bytes build_bvh takes from `tmp` and from `out` for n triangles.
size_t bvh_temp_bytes(uint32_t n);
size_t bvh_output_bytes(uint32_t n);

// ---- renderer ---------------------------------------------------------------
struct SceneDev;
struct WaveDesc;
struct WaveCtrl;
struct DevMaterial;

struct GuideNet;  // MLP path guide (guide.cu)

struct SceneGpu {
  lisa_renderer_params params{};  // copied (pointers not kept)
  std::string output_image;
  uint32_t num_prims = 0;
  uint32_t npix = 0;
  uint64_t samples_done = 0;  // samples per pixel accumulated
  uint64_t sample_offset = 0; // first sample index of this renderer's range
  uint64_t next_sample = 0;   // index of the next sample to render
  uint32_t subframe = 0;      // progressive launches done
  BvhBuildResult bvh;
  // device
  uint4* nodes = nullptr;
  float4* tris = nullptr;
  // BVH over the emissive triangles alone (reference estimator): leaves
  // carry the triangles' scene-wide indices and their emitter materials
  BvhBuildResult ebvh{};
  uint4* enodes = nullptr;
  float4* etris = nullptr;
  float4* prims = nullptr;
  DevMaterial* mats = nullptr;
  float4* acc_sum = nullptr;
  float4* acc_comp = nullptr;
  double* acc_sq = nullptr;
  double* acc_sum64 = nullptr;
  uint32_t* pix_rng = nullptr;
  float4* emit = nullptr;       // physically based estimator: emitter records
  float* emit_cdf = nullptr;
  uint32_t num_emit = 0;
  bool has_emit_box = false;  // bounds of the emissive triangles (padded), for the emitter search
  float emit_lo[3] = {0, 0, 0}, emit_hi[3] = {0, 0, 0};
  float extent = 0.0f;
  float eye[3], U[3], V[3], W[3];
  int guide = -1;
  uint64_t guide_waves_done = 0;  // guided waves of this scene so far
  uint64_t guide_steps_done = 0;  // Adam steps of its guide so far
};

struct Renderer {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  lisa_options opts{};
  DeviceArena arena;
  std::vector<SceneGpu> scenes;
  SceneDev* d_scenes = nullptr;
  // wavefront buffers
  uint32_t capacity = 0;
  float4* ro[2] = {nullptr, nullptr};
  float4* rd[2] = {nullptr, nullptr};
  int2* hit = nullptr;
  float4* ps_att = nullptr;
  float4* ps_col = nullptr;
  uint32_t* ps_rng = nullptr;
  float4* nee_a = nullptr;
  float4* nee_b = nullptr;
  float4* nee_c = nullptr;
  WaveCtrl* ctrl = nullptr;
  WaveDesc* d_waves = nullptr;  // device wave table
  uint32_t wave_capacity = 0;   // entries in d_waves
  // launch shapes
  int trace_blocks = 0, trace_threads = 128;
  int nee_blocks = 0, nee_threads = 128;
  int nee_pb_blocks = 0;  // physically based emitter kernel
  int shade_blocks = 0, shade_threads = 256;
  // events for stage timing
  std::vector<cudaEvent_t> ev_pool;
  // CUDA graph of the last launch sequence, reused while its shape (waves
  // and their depths, flags, wave-table address) stays the same
  cudaGraphExec_t graph_exec = nullptr;
  std::vector<uint64_t> graph_key;
  std::vector<std::pair<int, std::pair<size_t, size_t>>> graph_marks;
  uint32_t graph_launches[5] = {0, 0, 0, 0, 0};  // trace, shade, nee, total, guide
  // guided mode
  std::vector<std::unique_ptr<GuideNet>> guides;
  float4* rec_list = nullptr;    // rec_cap kept training records (4 float4 each, then rec_cap float4: rec_col)
  uint32_t rec_cap = 0;
  float4* nee_light = nullptr;   // guided physically based mode: capacity x 2 emitter samples
  float4* guide_batch = nullptr; // guide_batch_cap x 4 training samples
  uint32_t guide_batch_cap = 0;  // samples collected per wave
  uint32_t guide_chunk = 0;      // samples per Adam step
  uint32_t guide_max_steps = 0;  // Adam steps after the largest wave
  float* guide_grad_part = nullptr;  // partial-gradient slots shared by the scenes' guides
  float* guide_loss_part = nullptr;
  uint32_t* guide_grid_bar = nullptr;  // the training rounds' grid-barrier counter
  uint64_t guide_waves_done = 0; // waves rendered in guided mode so far
  ~Renderer();
};

Status renderer_create(const lisa_renderer_params* scenes, int n, const lisa_options* opts, Renderer** out);
Status renderer_render(Renderer& r, uint32_t spp, bool progressive, lisa_render_stats* stats);
Status renderer_reset(Renderer& r);
Status renderer_get_image(Renderer& r, int scene, float* rgb32, uint8_t* rgba8, double* var, double* mean64);
Status renderer_get_ppm(Renderer& r, int scene, uint8_t* rgb8);
Status trace_rays(Renderer& r, const float* d_rays, uint32_t n, int32_t* d_prim, float* d_t, cudaStream_t s,
                  bool brute);
Status trace_count(Renderer& r, const float* d_rays, uint32_t n, uint64_t* visits, uint64_t* tests);
// Closest hit (or brute force) of n device rays against the scene d_scene;
// d_ctrl receives the device status word.  Synchronises `s`.
Status launch_trace_closest(const SceneDev* d_scene, WaveCtrl* d_ctrl, const float* d_rays, uint32_t n,
                            int32_t* d_prim, float* d_t, cudaStream_t s, int sm_count, bool brute);

// error string per thread (api.cu)
void set_last_error(const Status& s);

}  // namespace lisa

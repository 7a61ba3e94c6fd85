// Closest-hit queries over a caller's triangle soup without any device
// allocation.
//
// Who needs this: code that may not call cudaMalloc / cudaFree at query
// time -- for example a plugin living inside a host application whose own
// caching allocator has already reserved the device memory, or a per-frame
// loop that cannot afford the implicit device-wide synchronisation cudaFree
// performs.  lisa_trace_closest_device needs a renderer, and creating one
// allocates; this entry point instead builds its BVH in a fixed scratch
// array that is part of the library image and traces the caller's rays
// into the caller's output buffers.
//
// The scratch is the file-scope array below.  Every GPU that loads the
// library holds it (NOALLOC_SCRATCH_BYTES = 22,020,096 bytes, 21 MiB) until
// the process exits.  Its host-side name is only a stand-in for the device
// array, so host code obtains the device address with cudaGetSymbolAddress,
// once per CUDA context, the first time the entry point runs in that
// context (with it current); that first call should therefore come before
// any stream capture.  The address belongs to the context the module was
// loaded into, so it is cached by the context's unique ID (cuCtxGetId): a
// caller that makes its own context current, or a cudaDeviceReset that
// replaces the primary context, gets a fresh look-up.  All calls share the
// one array and it keeps the previous call's contents: every counter the
// build needs zeroed is cleared at the start of each call, and calls that
// overlap on the GPU (two host threads, or two streams) race on the array,
// so callers must serialise them.
#include <cuda.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "lisa_device.cuh"
#include "lisa_internal.h"

namespace lisa {
namespace {

constexpr uint32_t NOALLOC_MAX_TRIANGLES = 65536;
// BVH build temporaries (~172 B per triangle) + 8-wide nodes and leaf
// triangles (~128 B per triangle) + the scene record and status word, with
// room for alignment.
constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)NOALLOC_MAX_TRIANGLES * 320 + (1u << 20);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Scratch addresses already looked up, by CUDA context ID.  Contexts are
// few (one primary context per device, plus any a host application creates);
// the table is a small ring, a full one re-uses its oldest slot.
constexpr int MAX_CONTEXTS = 64;
struct ScratchEntry {
  unsigned long long ctx_id;
  void* ptr;
};
std::mutex g_mu;
ScratchEntry g_scratch[MAX_CONTEXTS] = {};
int g_scratch_used = 0, g_scratch_next = 0;

// Device address of the scratch array in the current context (looked up
// once per context).
Status scratch_address(void** out) {
  unsigned long long id = 0;
  bool none = false;
  LISA_TRY(current_context_id(&id, &none));
  std::lock_guard<std::mutex> lock(g_mu);
  if (!none)
    for (int i = 0; i < g_scratch_used; ++i)
      if (g_scratch[i].ctx_id == id) {
        *out = g_scratch[i].ptr;
        return Status();
      }
  // with no context current, this binds the device's primary context
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return Status::cuda(e, "cudaGetSymbolAddress(no-allocation scratch)");
  }
  if (none) {
    LISA_TRY(current_context_id(&id, &none));
    if (none) return Status(LISA_ERR_CUDA, "no CUDA context after the scratch look-up");
  }
  const int slot = g_scratch_used < MAX_CONTEXTS ? g_scratch_used++ : (g_scratch_next++ % MAX_CONTEXTS);
  g_scratch[slot] = ScratchEntry{id, p};
  *out = p;
  return Status();
}

Status trace_soup_noalloc(const float* d_vertices, uint32_t num_triangles, const float* d_rays, uint32_t num_rays,
                          int32_t* d_prim, float* d_t, cudaStream_t stream) {
  if (num_triangles > NOALLOC_MAX_TRIANGLES)
    return Status::invalid("num_triangles " + std::to_string(num_triangles) +
                           " exceeds the no-allocation limit of " + std::to_string(NOALLOC_MAX_TRIANGLES));
  if ((num_triangles && !d_vertices) || (num_rays && (!d_rays || !d_prim || !d_t)))
    return Status::invalid("null buffer");
  // nothing to trace: touch neither the scratch nor the stream
  if (num_rays == 0) return Status();
  int dev = 0;
  LISA_CUDA(cudaGetDevice(&dev));
  int sm = 0;
  LISA_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
  void* base = nullptr;
  LISA_TRY(scratch_address(&base));
  BumpScratch region(base, NOALLOC_SCRATCH_BYTES);
  SceneDev* d_scene = nullptr;
  WaveCtrl* d_ctrl = nullptr;
  LISA_TRY(region.get((void**)&d_scene, sizeof(SceneDev), "scene record"));
  LISA_TRY(region.get((void**)&d_ctrl, sizeof(WaveCtrl), "status word"));
  uint4* nodes = nullptr;
  float4* tris = nullptr;
  BvhBuildResult info;
  LISA_TRY(build_bvh(d_vertices, num_triangles, stream, region, region, &nodes, &tris, &info));
  SceneDev h;
  std::memset(&h, 0, sizeof(h));
  h.nodes = nodes;
  h.tris = tris;
  h.num_prims = num_triangles;
  h.num_nodes = info.num_nodes;
  double e2 = 0.0;
  for (int k = 0; k < 3; ++k) e2 += (double)(info.bmax[k] - info.bmin[k]) * (info.bmax[k] - info.bmin[k]);
  h.extent = (e2 > 0.0 && e2 < 1e76) ? (float)std::sqrt(e2) : 1.0f;
  LISA_CUDA(cudaMemcpyAsync(d_scene, &h, sizeof(h), cudaMemcpyHostToDevice, stream));
  // launch_trace_closest clears the status word before tracing
  return launch_trace_closest(d_scene, d_ctrl, d_rays, num_rays, d_prim, d_t, stream, sm, false);
}

}  // namespace
}  // namespace lisa

extern "C" int lisa_trace_soup_noalloc(const float* d_vertices, uint32_t num_triangles, const float* d_rays,
                                       uint32_t num_rays, int32_t* d_prim, float* d_t, void* stream) {
  lisa::Status s;
  try {
    s = lisa::trace_soup_noalloc(d_vertices, num_triangles, d_rays, num_rays, d_prim, d_t, (cudaStream_t)stream);
  } catch (const std::exception& e) {
    s = lisa::Status(LISA_ERR_INVALID, e.what());
  }
  lisa::set_last_error(s);
  return s.code;
}

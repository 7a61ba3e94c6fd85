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
// library holds it (NOALLOC_SCRATCH_BYTES, about 17 MB) until the process
// exits.  Its host-side name is only a stand-in for the device array, so
// host code obtains the device address with cudaGetSymbolAddress, once per
// device, the first time the entry point runs on that device (with that
// device current); that first call should therefore come before any stream
// capture.  All calls share the one array and it keeps the previous call's
// contents: every counter the build needs zeroed is cleared at the start of
// each call, and calls that overlap on the GPU (two host threads, or two
// streams) race on the array, so callers must serialise them.
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

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void* g_scratch_ptr[MAX_DEVICES] = {};

// Device address of the scratch array on the current device (set up once
// per device).
Status scratch_address(int dev, void** out) {
  if (dev < 0 || dev >= MAX_DEVICES) return Status::invalid("device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return Status::cuda(e, "cudaGetSymbolAddress(no-allocation scratch)");
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return Status();
}

Status trace_soup_noalloc(const float* d_vertices, uint32_t num_triangles, const float* d_rays, uint32_t num_rays,
                          int32_t* d_prim, float* d_t, cudaStream_t stream) {
  if (num_triangles > NOALLOC_MAX_TRIANGLES)
    return Status::invalid("num_triangles " + std::to_string(num_triangles) +
                           " exceeds the no-allocation limit of " + std::to_string(NOALLOC_MAX_TRIANGLES));
  if ((num_triangles && !d_vertices) || (num_rays && (!d_rays || !d_prim || !d_t)))
    return Status::invalid("null buffer");
  int dev = 0;
  LISA_CUDA(cudaGetDevice(&dev));
  int sm = 0;
  LISA_CUDA(cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev));
  void* base = nullptr;
  LISA_TRY(scratch_address(dev, &base));
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

// The reference's own OptiX render, run headless: a baseline, not product code.
//
// Drives the reference's OptixWrapper (src/LiSA/src/optix_wrapper.cc:24-465:
// OptiX context, GAS build over the soup, module from shader.cu's PTX,
// program groups, pipeline, SBT, launch parameters) exactly as the
// reference's main does, then launches the pipeline the way
// launchSubframe / render do (src/LiSA/src/render.cc:35-58,133-148):
// copy the parameters, optixLaunch(width, height, 1), synchronise.  The
// only differences are headless ones: the frame buffer is plain device
// memory instead of a mapped display buffer, and the launch is timed with
// CUDA events on the wrapper's stream.  shader.cu is compiled to PTX by nvcc
// ahead of time (baseline/stage_optix.py, the reference's own nvcc flags);
// getInputData hands that PTX to the unchanged set-up code.
//
// Ray counts come from a second pipeline built from a copy of shader.cu
// with one atomicAdd before each optixTrace (radiance, occlusion) and the
// launch parameters extended by a counter pointer; it runs once, untimed,
// on the same scene and seeds.
//
// Usage:
//   lisa_optix_harness (--rto scene.rto | --soup scene.soup) [--spp N]
//       [--warmup W] [--reps R] [--count-ptx counted.ptx] [--accum out.f32]
// The PTX of the stock shader comes from $LISA_OPTIX_PTX.  Prints one JSON
// line: launch time, rays per launch, GAS build + pipeline set-up time.
#include <optix_function_table_definition.h>
#include <optix_stubs.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "optix_wrapper.hh"
#include "scene_parser.hh"
#include "sutil/Exception.h"
#include "sutil/sutil.h"

namespace sutil {
const char* getInputData(const char*, const char*, const char*, size_t& size) {
  static std::string buf;
  const char* path = std::getenv("LISA_OPTIX_PTX");
  if (!path) throw std::runtime_error("LISA_OPTIX_PTX is not set");
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error(std::string("cannot open ") + path);
  std::stringstream ss;
  ss << f.rdbuf();
  buf = ss.str();
  size = buf.size();
  return buf.c_str();
}
}  // namespace sutil

namespace {

// Launch parameters of the counting module: the reference's, then the
// address of two counters (radiance, occlusion traces).
struct OptixParamsCounted : OptixParams {
  unsigned long long* ray_counts;
};

// A raw soup: the arrays SceneParser would produce, without the text
// parsing (used for multi-million-triangle scenes).  Layout, little endian:
// magic "LSOUP1\0\0", u32 T, M, width, height, spp, bounces; f32 eye[3],
// look_at[3], fov; f32 vertices[9T], normals[9T]; i32 mat_indices[T];
// Material[M] (40 bytes each, the layout of structs.hh:16-23).
struct Soup {
  std::vector<float3> vertices, normals;
  std::vector<int> mat_indices;
  std::vector<Material> materials;
  RendererParams params{};
};

template <class T>
void read_into(std::ifstream& f, T* dst, size_t n) {
  f.read(reinterpret_cast<char*>(dst), sizeof(T) * n);
  if (!f) throw std::runtime_error("truncated soup file");
}

void load_soup(const char* path, Soup& s) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error(std::string("cannot open ") + path);
  char magic[8];
  read_into(f, magic, 8);
  if (std::memcmp(magic, "LSOUP1", 6) != 0) throw std::runtime_error("not a soup file");
  uint32_t h[6];
  read_into(f, h, 6);
  float cam[7];
  read_into(f, cam, 7);
  const size_t T = h[0], M = h[1];
  s.vertices.resize(3 * T);
  s.normals.resize(3 * T);
  s.mat_indices.resize(T);
  s.materials.resize(M);
  read_into(f, s.vertices.data(), 3 * T);
  read_into(f, s.normals.data(), 3 * T);
  read_into(f, s.mat_indices.data(), T);
  read_into(f, s.materials.data(), M);
  RendererParams& p = s.params;
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

void launch(RendererState& st, CUdeviceptr d_params, size_t params_size, const void* host_params) {
  CUDA_CHECK(cudaMemcpyAsync(reinterpret_cast<void*>(d_params), host_params, params_size, cudaMemcpyHostToDevice,
                             st.stream));
  OPTIX_CHECK(optixLaunch(st.pipeline, st.stream, d_params, params_size, &st.sbt, st.params.width,
                          st.params.height, 1));
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

int main(int argc, char** argv) {
  const char* rto = nullptr;
  const char* soup_path = nullptr;
  const char* count_ptx = nullptr;
  const char* accum_out = nullptr;
  int spp = -1, warmup = 2, reps = 5;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "missing value after %s\n", a.c_str());
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "--rto") rto = next();
    else if (a == "--soup") soup_path = next();
    else if (a == "--spp") spp = std::atoi(next());
    else if (a == "--warmup") warmup = std::atoi(next());
    else if (a == "--reps") reps = std::atoi(next());
    else if (a == "--count-ptx") count_ptx = next();
    else if (a == "--accum") accum_out = next();
    else {
      std::fprintf(stderr, "unknown argument %s\n", a.c_str());
      return 2;
    }
  }
  if (!rto == !soup_path) {
    std::fprintf(stderr, "give exactly one of --rto or --soup\n");
    return 2;
  }
  try {
    Soup soup;
    SceneParser* parser = nullptr;
    RendererParams params;
    if (rto) {
      parser = new SceneParser(const_cast<char*>(rto));
      params = parser->get_params();
    } else {
      load_soup(soup_path, soup);
      params = soup.params;
    }
    if (spp > 0) params.num_samples = (unsigned)spp;
    const std::string stock_ptx = std::getenv("LISA_OPTIX_PTX") ? std::getenv("LISA_OPTIX_PTX") : "";

    auto t0 = std::chrono::steady_clock::now();
    OptixWrapper wrapper(params);
    CUDA_SYNC_CHECK();
    const double setup_s = seconds_since(t0);
    RendererState& st = *wrapper.get_pstate();
    const size_t npix = (size_t)params.width * params.height;
    uchar4* d_frame = nullptr;
    CUDA_CHECK(cudaMalloc(reinterpret_cast<void**>(&d_frame), npix * sizeof(uchar4)));
    st.params.frame_buffer = d_frame;
    st.params.samples_per_launch = params.num_samples;  // render.cc:141
    st.params.subframe_index = 0u;

    for (int i = 0; i < warmup; ++i) launch(st, reinterpret_cast<CUdeviceptr>(st.d_params), sizeof(OptixParams),
                                            &st.params);
    CUDA_CHECK(cudaStreamSynchronize(st.stream));
    cudaEvent_t e0, e1;
    CUDA_CHECK(cudaEventCreate(&e0));
    CUDA_CHECK(cudaEventCreate(&e1));
    std::vector<float> launch_ms;
    for (int i = 0; i < reps; ++i) {
      CUDA_CHECK(cudaEventRecord(e0, st.stream));
      launch(st, reinterpret_cast<CUdeviceptr>(st.d_params), sizeof(OptixParams), &st.params);
      CUDA_CHECK(cudaEventRecord(e1, st.stream));
      CUDA_CHECK(cudaEventSynchronize(e1));
      float ms = 0.0f;
      CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
      launch_ms.push_back(ms);
    }
    CUDA_SYNC_CHECK();
    if (accum_out) {
      std::vector<float4> acc(npix);
      CUDA_CHECK(cudaMemcpy(acc.data(), st.params.accum_buffer, npix * sizeof(float4), cudaMemcpyDeviceToHost));
      std::ofstream f(accum_out, std::ios::binary);
      f.write(reinterpret_cast<const char*>(acc.data()), npix * sizeof(float4));
    }

    unsigned long long counts[2] = {0, 0};
    if (count_ptx) {
      setenv("LISA_OPTIX_PTX", count_ptx, 1);
      OptixWrapper counted(params);
      setenv("LISA_OPTIX_PTX", stock_ptx.c_str(), 1);
      RendererState& cs = *counted.get_pstate();
      unsigned long long* d_counts = nullptr;
      CUDA_CHECK(cudaMalloc(reinterpret_cast<void**>(&d_counts), sizeof(counts)));
      CUDA_CHECK(cudaMemset(d_counts, 0, sizeof(counts)));
      OptixParamsCounted pc;
      std::memset(&pc, 0, sizeof(pc));
      static_cast<OptixParams&>(pc) = cs.params;
      pc.frame_buffer = d_frame;
      pc.samples_per_launch = params.num_samples;
      pc.subframe_index = 0u;
      pc.ray_counts = d_counts;
      CUdeviceptr d_pc = 0;
      CUDA_CHECK(cudaMalloc(reinterpret_cast<void**>(&d_pc), sizeof(pc)));
      launch(cs, d_pc, sizeof(pc), &pc);
      CUDA_SYNC_CHECK();
      CUDA_CHECK(cudaMemcpy(counts, d_counts, sizeof(counts), cudaMemcpyDeviceToHost));
      CUDA_CHECK(cudaFree(d_counts));
      CUDA_CHECK(cudaFree(reinterpret_cast<void*>(d_pc)));
    }
    std::vector<float> sorted = launch_ms;
    std::sort(sorted.begin(), sorted.end());
    double sum = 0;
    for (float m : launch_ms) sum += m;
    std::printf("{\"ms_per_launch\": %.6f, \"ms_median\": %.6f, \"reps\": %d, \"spp\": %u, \"width\": %u, "
                "\"height\": %u, \"bounces\": %u, \"triangles\": %d, \"materials\": %d, "
                "\"rays_radiance\": %llu, \"rays_occlusion\": %llu, \"setup_s\": %.4f}\n",
                reps ? sum / reps : 0.0, reps ? sorted[sorted.size() / 2] : 0.0f, reps, params.num_samples,
                params.width, params.height, params.num_bounces, params.num_vertices / 3, params.num_materials,
                counts[0], counts[1], setup_s);
    CUDA_CHECK(cudaFree(d_frame));
    delete parser;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}

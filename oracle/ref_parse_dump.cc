// Test infrastructure (oracle), not product code.
//
// Drives the reference's own scene front end -- SceneParser
// (src/LiSA/src/scene_parser.cc:35-261) and parse_obj
// (src/LiSA/src/parse_obj.cc:24-69), compiled from the reference sources by
// oracle/Makefile -- and prints the RendererParams it produces
// (src/LiSA/include/structs.hh:90-103) as one "key value..." line per field,
// so that tests can compare the product parser against the reference field by
// field.  Floats are printed as their IEEE-754 bit patterns (hex) so the
// comparison is bit exact.  Material fields the reference leaves
// uninitialised (structs.hh:25-52) are not printed.
// With --time as the first argument it parses the scene and prints only
// the wall time of SceneParser + get_params in seconds (the reference's
// front end, timed for oracle/parse_bench.py).
#include "scene_parser.hh"

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>

static uint32_t bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s [--time] scene.rto\n", argv[0]);
    return 2;
  }
  if (argc >= 3 && std::strcmp(argv[1], "--time") == 0) {
    const auto t0 = std::chrono::steady_clock::now();
    SceneParser timed(argv[2]);
    RendererParams q = timed.get_params();
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("%.6f %d\n", s, q.num_vertices);
    return 0;
  }
  SceneParser parser(argv[1]);
  RendererParams p = parser.get_params();
  std::printf("width %u\nheight %u\nnum_samples %u\nnum_bounces %u\n", p.width, p.height,
              p.num_samples, p.num_bounces);
  std::printf("output_image %zu ", std::strlen(p.output_image));
  for (const char* c = p.output_image; *c; ++c) std::printf("%02x", (unsigned char)*c);
  std::printf("\n");
  std::printf("camera %08x %08x %08x %08x %08x %08x %08x\n", bits(p.camera.eye.x), bits(p.camera.eye.y),
              bits(p.camera.eye.z), bits(p.camera.look_at.x), bits(p.camera.look_at.y),
              bits(p.camera.look_at.z), bits(p.camera.fov));
  std::printf("num_materials %d\n", p.num_materials);
  for (int i = 0; i < p.num_materials; ++i) {
    const Material& m = p.materials[i];
    if (m.emit) {
      std::printf("material %d emit %08x %08x %08x alpha %08x\n", i, bits(m.emission_color.x),
                  bits(m.emission_color.y), bits(m.emission_color.z), bits(m.alpha));
    } else if (m.alpha < 1.0f) {
      std::printf("material %d dielectric %08x %08x %08x alpha %08x n %08x\n", i,
                  bits(m.diffuse_color.x), bits(m.diffuse_color.y), bits(m.diffuse_color.z),
                  bits(m.alpha), bits(m.n));
    } else {
      std::printf("material %d diffuse %08x %08x %08x alpha %08x roughness %08x\n", i,
                  bits(m.diffuse_color.x), bits(m.diffuse_color.y), bits(m.diffuse_color.z),
                  bits(m.alpha), bits(m.roughness));
    }
  }
  std::printf("num_vertices %d\n", p.num_vertices);
  // FNV-1a over the raw soup bytes: vertices, normals, then one material
  // index per triangle.
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](const void* data, size_t n) {
    const unsigned char* b = (const unsigned char*)data;
    for (size_t i = 0; i < n; ++i) {
      h ^= b[i];
      h *= 1099511628211ull;
    }
  };
  mix(p.vertices, sizeof(float) * 3 * (size_t)p.num_vertices);
  mix(p.normals, sizeof(float) * 3 * (size_t)p.num_vertices);
  mix(p.mat_indices, sizeof(int) * (size_t)(p.num_vertices / 3));
  std::printf("soup_fnv1a %016llx\n", (unsigned long long)h);
  return 0;
}

// lisa: command-line renderer with the reference's interface
// (src/LiSA/src/main.cc:6-27, src/LiSA/include/parse_args.hh:3-16):
//
//   lisa -s scene.rto [-d] [--guided] [--physical] [--seed N] [--reference-rng]
//        [--autotune cache.json]
//
// -s   scene file (required)
// -d   the reference's interactive display mode, headless: progressive
//      launches of 16 spp until num_samples (render.cc:75-131), then the PPM
// --autotune  queue and block sizes from the autotuner, kept in the given
//      JSON cache (short probe renders the first time for a workload)
// The image goes to the scene's output_image, as in render.cc:9-17.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "lisa_gb.h"

static const char* get_option(int argc, char** argv, const char* opt) {
  for (int i = 1; i + 1 < argc; ++i)
    if (std::strcmp(argv[i], opt) == 0) return argv[i + 1];
  return nullptr;
}
static bool has_option(int argc, char** argv, const char* opt) {
  for (int i = 1; i < argc; ++i)
    if (std::strcmp(argv[i], opt) == 0) return true;
  return false;
}
static int fail(const char* what) {
  std::fprintf(stderr, "%s: %s\n", what, lisa_last_error());
  return 1;
}

int main(int argc, char** argv) {
  const char* scene_path = get_option(argc, argv, "-s");
  if (!scene_path) {
    std::fprintf(stderr, "Missing scene path.\nUsage: %s -s scene_path\n", argv[0]);
    return 1;
  }
  lisa_scene* scene = nullptr;
  if (lisa_scene_parse(scene_path, &scene) != LISA_OK) return fail("scene");
  lisa_renderer_params params;
  lisa_scene_params(scene, &params);
  lisa_options opts;
  lisa_options_default(&opts);
  if (has_option(argc, argv, "--guided")) opts.mode = LISA_MODE_GUIDED;
  if (has_option(argc, argv, "--physical")) opts.estimator = LISA_ESTIMATOR_PHYSICAL;
  if (has_option(argc, argv, "--reference-rng")) opts.rng = LISA_RNG_PER_PIXEL;
  if (const char* s = get_option(argc, argv, "--seed")) opts.seed = (uint32_t)std::strtoul(s, nullptr, 10);
  if (const char* cache = get_option(argc, argv, "--autotune")) {
    lisa_tuning t;
    std::memset(&t, 0, sizeof(t));
    t.struct_size = sizeof(t);
    if (lisa_autotune(&params, 1, &opts, cache, &t) != LISA_OK) return fail("autotune");
    lisa_tuning_apply(&t, &opts);
  }
  lisa_renderer* r = nullptr;
  if (lisa_renderer_create(&params, &opts, &r) != LISA_OK) return fail("renderer");
  std::printf("Starting rendering...\n");
  const auto t0 = std::chrono::system_clock::now();
  lisa_render_stats st;
  uint64_t rays = 0;
  if (has_option(argc, argv, "-d")) {
    const uint32_t per_launch = params.num_samples > 16 ? 16 : params.num_samples;
    for (uint32_t done = 0; done < params.num_samples; done += per_launch) {
      if (lisa_render_progressive(r, per_launch, &st) != LISA_OK) return fail("render");
      rays += st.rays_primary + st.rays_bounce + st.rays_shadow;
      std::printf("nb sample   : %8u\r", done + per_launch);
      std::fflush(stdout);
    }
    std::printf("\n");
  } else {
    if (lisa_render(r, &st) != LISA_OK) return fail("render");
    rays = st.rays_primary + st.rays_bounce + st.rays_shadow;
  }
  if (lisa_save_image(r, 0, nullptr) != LISA_OK) return fail("save");
  const std::chrono::duration<float> dt = std::chrono::system_clock::now() - t0;
  std::printf("Rendering finished in %.2f mn (%.1f Mrays/s).\n", dt.count() / 60.0f, rays / dt.count() / 1e6);
  lisa_renderer_destroy(r);
  lisa_scene_destroy(scene);
  return 0;
}

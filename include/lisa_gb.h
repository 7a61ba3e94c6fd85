/*
 * lisa_gb.h -- C ABI of the GB300 path tracer.
 *
 * This is the drop-in boundary for LiSA's host surface.  Each entry point
 * names the reference interface it replaces (paths are relative to the LiSA
 * source tree).  Conventions:
 *   - every function returns LISA_OK (0) or an error code; the message of the
 *     last error on the calling thread is available from lisa_last_error();
 *     no C++ exception crosses this boundary (the reference throws
 *     sutil::Exception or calls exit(1), src/sutil/Exception.h:167-200,
 *     src/LiSA/src/scene_parser.cc:15-16,100-101,107-111);
 *   - the caller owns every input array; the library copies what it keeps;
 *   - plain pointers and sizes only: no CUDA or C++ types in signatures
 *     (streams are passed as void* = cudaStream_t);
 *   - one renderer must not be used from two threads at once; different
 *     renderers are independent.  Each renderer owns one CUDA stream.
 */
#ifndef LISA_GB_H
#define LISA_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LISA_OK 0
#define LISA_ERR_INVALID 1     /* bad argument or size                          */
#define LISA_ERR_PARSE 2       /* .rto / OBJ grammar error (reference: exit(1)) */
#define LISA_ERR_IO 3          /* file missing or unreadable                    */
#define LISA_ERR_CUDA 4        /* CUDA runtime error                            */
#define LISA_ERR_OOM 5         /* allocation failed or over the allocation cap  */
#define LISA_ERR_DEVICE 6      /* a device-side check failed (status word set)  */
#define LISA_ERR_UNSUPPORTED 7 /* no usable sm_103a device / feature missing    */

/* ---- reference-layout types ------------------------------------------- */

typedef struct lisa_float3 {
  float x, y, z;
} lisa_float3;

/* Material, field for field (src/LiSA/include/structs.hh:16-23): 40 bytes,
 * offsets 0/4/8/12/24/28.  emit is a C++ bool there (one byte). */
typedef struct lisa_material {
  float roughness;
  float alpha;     /* < 1: dielectric, n is the refractive index */
  float n;
  lisa_float3 diffuse_color;
  uint8_t emit;
  uint8_t _pad[3];
  lisa_float3 emission_color;
} lisa_material;

/* Camera (structs.hh:54-58). fov is the vertical field of view in degrees. */
typedef struct lisa_camera {
  lisa_float3 eye;
  lisa_float3 look_at;
  float fov;
} lisa_camera;

/* RendererParams (structs.hh:90-103): a flat triangle soup with three
 * vertices and three normals per triangle and one material index per
 * triangle.  Pointers are borrowed (the reference points into the parser's
 * vectors, scene_parser.cc:247-260). */
typedef struct lisa_renderer_params {
  const lisa_float3* vertices;
  const lisa_float3* normals;
  const lisa_material* materials;
  const int32_t* mat_indices;
  int32_t num_vertices;
  int32_t num_materials;
  uint32_t width, height;
  lisa_camera camera;
  uint32_t num_samples;
  uint32_t num_bounces;
  const char* output_image;
} lisa_renderer_params;

/* ---- options (no reference counterpart; defaults reproduce the reference) */

#define LISA_MODE_COMPAT 0 /* the reference estimator, quirks included       */
#define LISA_MODE_GUIDED 1 /* same estimator, bounce drawn from MLP guide+BSDF
                              by one-sample MIS                               */

#define LISA_ESTIMATOR_COMPAT 0   /* the reference estimator (default)      */
#define LISA_ESTIMATOR_PHYSICAL 1 /* opt-in physically based estimator: emitter
                                     sampling by area x luminance, cosine-
                                     weighted diffuse sampling, power-heuristic
                                     MIS, roughness = weight of the diffuse
                                     lobe against a mirror, Schlick on the
                                     less dense side; combines with
                                     LISA_MODE_GUIDED                         */

#define LISA_RNG_PER_SAMPLE 0 /* one LCG stream per (seed, pixel, sample)    */
#define LISA_RNG_PER_PIXEL 1  /* the reference stream: tea<16>(pixel,
                                 subframe) shared by all samples of a pixel
                                 (src/LiSA/src/shader.cu:141)               */

typedef struct lisa_options {
  uint32_t struct_size;      /* sizeof(lisa_options)                           */
  uint32_t mode;             /* LISA_MODE_*                                    */
  uint32_t rng;              /* LISA_RNG_*                                     */
  uint32_t seed;
  uint32_t paths_in_flight;  /* wavefront size (0 = 16 Mi; 4 Mi guided)       */
  uint32_t blocks_per_sm;    /* persistent-kernel residency (0 = auto)         */
  uint32_t threads_per_block;/* persistent-kernel block size (0 = auto)        */
  uint32_t use_graph;        /* capture each launch sequence in a CUDA graph   */
  uint32_t stage_timing;     /* record CUDA events around every stage launch   */
  uint32_t accum_fp64;       /* also accumulate the pixel mean in FP64         */
  float aperture;            /* thin-lens aperture radius; 0 = pinhole (ref.)  */
  float focal_distance;      /* 0 = |look_at - eye|                            */
  /* path guide (LISA_MODE_GUIDED) */
  float guide_bsdf_fraction; /* probability c of sampling the BSDF strategy    */
  float guide_lr;            /* Adam learning rate                             */
  uint32_t guide_train_batch;/* samples per Adam step (multiple of 128; 0 = one
                                128-sample tile per SM)                        */
  uint32_t guide_train_waves;/* waves that train (0 = every wave)              */
  uint64_t alloc_cap_bytes;  /* refuse device allocations beyond this (0=none) */
  uint32_t count_traversal;  /* run the counting variants of the traversal
                                kernels (node visits / triangle tests)        */
  uint32_t guide_warmup_waves;/* first waves train the guide but sample the
                                BSDF only                                      */
  uint32_t guide_steps_per_wave;/* Adam steps after a guided wave per 4 Mi of
                                its paths (at least one), each on its own slice
                                of guide_train_batch samples                  */
  uint32_t guide_spp_per_wave;/* guided mode: at most this many samples per
                                pixel per wave (more for images under 1 Mi
                                pixels), so every scene trains over several
                                waves (0 = fill the wavefront)                */
  uint32_t refill_idle;      /* persistent traversal kernels take new work once
                                this many of a warp's 32 lanes are idle
                                (1..32; 0 = 12)                               */
  uint32_t estimator;        /* LISA_ESTIMATOR_*                               */
  uint32_t bvh_lbvh_only;    /* 1 = keep the plain LBVH: skip its SAH treelet
                                restructuring before the 8-wide collapse      */
  uint32_t guide_min_spp;    /* guided mode guides the scenes with at least
                                this many samples per pixel (num_samples);
                                the others render plain, packed together     */
  uint32_t guide_max_depth;  /* the guide draws the bounces of the first this
                                many vertices of a path; deeper ones sample
                                the BSDF (0 = every vertex)                  */
  uint32_t guide_train_steps;/* Adam steps per scene, after which its guide
                                stays fixed (0 = no limit)                   */
} lisa_options;

/* Per-call statistics.  Ray counts are rays actually traced: primary +
 * bounce (radiance) + shadow (emitter queries). */
typedef struct lisa_render_stats {
  uint64_t rays_primary;
  uint64_t rays_bounce;
  uint64_t rays_shadow;
  uint64_t paths;
  uint64_t samples_total;      /* samples per pixel accumulated so far        */
  double ms_device;            /* CUDA-event time of the whole call            */
  double ms_trace;             /* stage sums (only with stage_timing)          */
  double ms_shade;
  double ms_nee;
  double ms_guide;
  double ms_other;
  uint32_t launches_trace;     /* stage launch counts                          */
  uint32_t launches_shade;
  uint32_t launches_nee;
  uint32_t launches_guide;
  uint32_t launches_total;     /* all kernels this call launched               */
  uint32_t device_status;      /* device status word (0 = clean)               */
  double guide_loss;           /* last training loss (guided mode)             */
  uint64_t nee_vertices;       /* opaque vertices that ran the emitter search  */
  uint64_t node_visits_trace;  /* counting pass only (count_traversal)         */
  uint64_t tri_tests_trace;
  uint64_t node_visits_nee;
  uint64_t tri_tests_nee;
  uint64_t shadow_traversals;  /* emitter-search rays that walked the BVH; the
                                * rest of rays_shadow could neither light their
                                * vertex nor change its emitter flag (they
                                * cannot reach an emitter and the flag was
                                * unset), so only their count was kept      */
  double ms_guide_infer;       /* guide stage split (stage_timing): inference */
  double ms_guide_train;       /* and training (collection, steps, Adam)      */
  uint64_t guide_infer_rows;   /* emitter-queue entries the inference ran on  */
  uint64_t guide_train_samples;/* samples of the training steps               */
} lisa_render_stats;

typedef struct lisa_scene lisa_scene;
typedef struct lisa_renderer lisa_renderer;
typedef struct lisa_guide lisa_guide;

/* ---- errors and device ------------------------------------------------- */

/* Message of the last failed call on this thread ("" if none). */
const char* lisa_last_error(void);
/* Library version string. */
const char* lisa_version(void);
/* SM count and compute capability of the current CUDA device.  Replaces the
 * device bring-up of OptixWrapper::init_optix (optix_wrapper.cc:39-52). */
int lisa_device_info(int* sm_count, int* cc_major, int* cc_minor);
/* Device memory that destroyed renderers left for reuse: renderers and BVH
 * builds take their buffers from a per-process cache (at most
 * LISA_DEVICE_CACHE_MB MiB of free blocks, default 8192; 0 turns it off),
 * so a create-render-destroy cycle does not pay cudaMalloc/cudaFree each
 * time.  This returns every cached block to the device and the number of
 * bytes freed in *bytes (may be NULL). */
int lisa_device_cache_release(uint64_t* bytes);

/* ---- scene front end (host) ------------------------------------------- */

/* Parse a .rto scene and every OBJ it names.  Replaces
 * SceneParser::SceneParser (src/LiSA/src/scene_parser.cc:35-57) and
 * parse_obj (src/LiSA/src/parse_obj.cc:24-69).  Grammar errors return
 * LISA_ERR_PARSE, missing files LISA_ERR_IO (the reference exits). */
int lisa_scene_parse(const char* rto_path, lisa_scene** out);
/* Parse .rto text held in memory; OBJ paths resolve against base_dir
 * (NULL = working directory, as the reference). */
int lisa_scene_parse_string(const char* rto_text, size_t len, const char* base_dir,
                            lisa_scene** out);
/* Borrowed view of the parsed scene, valid until lisa_scene_destroy.
 * Replaces SceneParser::get_params (scene_parser.hh:13). */
int lisa_scene_params(const lisa_scene* scene, lisa_renderer_params* out);
void lisa_scene_destroy(lisa_scene* scene);

/* Load one OBJ and append its de-indexed soup (3 vertices + 3 normals per
 * triangle, material index mat_idx per triangle) to scene.  Replaces
 * parse_obj (parse_obj.cc:24-69).  scene may be an empty scene from
 * lisa_scene_create_empty. */
int lisa_scene_create_empty(lisa_scene** out);
int lisa_scene_append_obj(lisa_scene* scene, const char* obj_path, int32_t mat_idx);

/* ---- renderer ----------------------------------------------------------- */

void lisa_options_default(lisa_options* opts);

/* Upload one scene, build its BVH on the GPU, allocate the wavefront.
 * Replaces OptixWrapper::OptixWrapper (optix_wrapper.cc:24-33: GAS build
 * optix_wrapper.cc:54-149, launch state optix_wrapper.cc:419-446). */
int lisa_renderer_create(const lisa_renderer_params* params, const lisa_options* opts,
                         lisa_renderer** out);
/* Several scenes (uneven sizes, resolutions, spp, bounces) served by one
 * renderer: their paths share every wavefront launch. */
int lisa_renderer_create_batch(const lisa_renderer_params* scenes, int32_t num_scenes,
                               const lisa_options* opts, lisa_renderer** out);
void lisa_renderer_destroy(lisa_renderer* r);

/* Batch render: num_samples samples per pixel for every scene.  Replaces
 * render() (src/LiSA/src/render.cc:133-148) minus the PPM write. */
int lisa_render(lisa_renderer* r, lisa_render_stats* stats);
/* Headless progressive launch: adds spp samples per pixel to the running
 * mean.  Replaces the display loop's launchSubframe + lerp
 * (render.cc:35-58,75-131; shader.cu:160-164) without the GL window. */
int lisa_render_progressive(lisa_renderer* r, uint32_t spp, lisa_render_stats* stats);
/* One call for a batch of scenes: creates a renderer over all of them
 * (lisa_renderer_create_batch), renders num_samples per pixel for each
 * (lisa_render), writes every scene with an output_image path to it as a
 * PPM, and destroys the renderer.  stats (may be NULL) covers the render.
 * What render() (render.cc:133-148) does for one scene, for many. */
int lisa_batch_render(const lisa_renderer_params* scenes, int32_t num_scenes, const lisa_options* opts,
                      lisa_render_stats* stats);
/* Forget the accumulated samples (and, in guided mode, keep the guide). */
int lisa_reset_accumulation(lisa_renderer* r);
/* Index of the next sample of scene `scene` (LISA_RNG_PER_SAMPLE streams are
 * keyed by it).  Renderers given disjoint sample ranges of one frame -- the
 * shards of a multi-GPU render -- produce means that merge exactly into the
 * single-GPU result.  No reference counterpart (the reference runs on one
 * GPU).  Also the index lisa_reset_accumulation returns to. */
int lisa_set_sample_offset(lisa_renderer* r, int32_t scene, uint64_t first_sample);

/* Image of scene `scene` (0 for a single-scene renderer).  Any output may be
 * NULL.  rgb32: w*h*3 mean radiance, row 0 = bottom (the accum_buffer
 * layout, shader.cu:165); rgba8: w*h*4 tone-mapped bytes as make_color
 * (src/cuda/helpers.h:57-62); var: w*h*3 per-pixel sample variance (FP64);
 * mean64: w*h*3 FP64 mean (only if accum_fp64). */
int lisa_get_image(lisa_renderer* r, int32_t scene, float* rgb32, uint8_t* rgba8, double* var,
                   double* mean64);
/* PPM payload computed on the device: w*h*3 bytes, rows flipped, exactly the
 * bytes sutil::saveImage writes after the header (sutil.cpp:523-553). */
int lisa_get_ppm_rgb8(lisa_renderer* r, int32_t scene, uint8_t* rgb8);
/* Write scene's image to its output_image path (or `path` if not NULL).
 * Replaces save_image (render.cc:9-17). */
int lisa_save_image(lisa_renderer* r, int32_t scene, const char* path);

/* ---- output (host) ------------------------------------------------------ */

/* Binary P6 PPM from RGBA8 pixels (row 0 = bottom): header "P6\nW H\n255\n",
 * rows flipped, alpha dropped.  Replaces sutil::saveImage for
 * UNSIGNED_BYTE4 (src/sutil/sutil.cpp:523-553,97-117). */
int lisa_write_ppm(const char* path, const uint8_t* rgba8, uint32_t width, uint32_t height);

/* ---- traversal hooks (closest hit) ------------------------------------ */

/* Closest hit of n rays against scene 0 of r.  rays: n x 8 floats
 * (ox oy oz tmin dx dy dz tmax).  prim: original triangle index or -1;
 * t: hit distance (+inf on a miss).  Ties go to the lowest triangle index.
 * Replaces optixTrace with OPTIX_RAY_FLAG_NONE (shader.cu:77-98).
 * Host buffers. */
int lisa_trace_closest(lisa_renderer* r, const float* rays, uint32_t n, int32_t* prim, float* t);
/* Same with device buffers on `stream` (cudaStream_t, NULL = renderer's). */
int lisa_trace_closest_device(lisa_renderer* r, const float* d_rays, uint32_t n, int32_t* d_prim,
                              float* d_t, void* stream);
/* Brute-force scan over every triangle on the GPU (same intersection
 * routine, same tie rule); for checking the BVH at sizes the CPU cannot. */
int lisa_trace_brute_device(lisa_renderer* r, const float* d_rays, uint32_t n, int32_t* d_prim,
                            float* d_t, void* stream);
/* Closest hit of num_rays device rays (same layout and tie rule as
 * lisa_trace_closest) against a soup of num_triangles triangles given as
 * device vertices (9 floats per triangle), with no device allocation: the
 * BVH is built in a scratch array compiled into the library (21 MiB =
 * 22,020,096 bytes, held on every GPU that loads it).  No counterpart in the reference; it
 * serves callers that cannot call cudaMalloc/cudaFree at query time (a
 * plugin inside an application whose allocator owns the device memory, or
 * a per-frame loop that cannot take cudaFree's device-wide sync).  Limits
 * and contract: at most 65536 triangles (larger soups return
 * LISA_ERR_INVALID); the first call in a CUDA context looks up the
 * scratch address (cached per context) and should come before any stream
 * capture; calls share the scratch, so calls that overlap on the GPU race
 * and must be serialised by the caller.  num_rays == 0 returns at once
 * without touching the scratch or the stream; otherwise the call
 * synchronises `stream` (cudaStream_t, NULL = default). */
int lisa_trace_soup_noalloc(const float* d_vertices, uint32_t num_triangles, const float* d_rays,
                            uint32_t num_rays, int32_t* d_prim, float* d_t, void* stream);
/* Node visits and triangle tests of the last counted traversal pass:
 * runs the closest-hit kernel on the rays with counters enabled. */
int lisa_trace_count(lisa_renderer* r, const float* rays, uint32_t n, uint64_t* node_visits,
                     uint64_t* tri_tests);
/* BVH statistics: 8-wide node count, leaf triangle slots, depth. */
int lisa_bvh_info(lisa_renderer* r, int32_t scene, uint32_t* nodes, uint32_t* tri_slots,
                  uint32_t* depth, double* build_ms);

/* ---- autotuner (no reference counterpart; the reference launches one fixed
 * optixLaunch(w, h, 1), render.cc:46-55) ---------------------------------- */

/* Queue and tile sizes for a workload: the wavefront size (paths in flight,
 * which sizes every ray/hit/path-state queue), the block size of the
 * persistent traversal kernels and their refill threshold. */
typedef struct lisa_tuning {
  uint32_t struct_size;        /* sizeof(lisa_tuning)                          */
  uint32_t paths_in_flight;
  uint32_t threads_per_block;
  uint32_t blocks_per_sm;      /* 0 = as many as fit                           */
  uint32_t refill_idle;
  uint32_t candidates;         /* configurations timed (0 = from the cache)    */
  uint32_t probe_spp;          /* spp of every scene per timed probe render    */
  uint32_t reserved;
  double mrays_per_s;          /* probe throughput of the chosen configuration */
  char key[160];               /* device + bucketed workload signature         */
} lisa_tuning;

/* Times short progressive renders of the workload (`n` scenes, options
 * `base`, NULL = defaults) under candidate queue and block sizes and
 * returns the fastest.  With a non-NULL `cache_path` (a JSON file) a workload
 * of the same signature on the same device is answered from the file, and a
 * new choice is added to it. */
int lisa_autotune(const lisa_renderer_params* scenes, int32_t n, const lisa_options* base,
                  const char* cache_path, lisa_tuning* out);
/* Copies the tuned sizes into options. */
void lisa_tuning_apply(const lisa_tuning* t, lisa_options* o);
/* Host-only access to a tuning cache file: look a key up (*found = 0 or 1),
 * or add / replace the entry `t->key`. */
int lisa_tuning_cache_lookup(const char* cache_path, const char* key, lisa_tuning* out, int32_t* found);
int lisa_tuning_cache_store(const char* cache_path, const lisa_tuning* t);

/* ---- path guide (no reference counterpart) ------------------------------ */

/* Guide network: 64 input features -> 4 hidden layers of 64 (ReLU) -> 40
 * outputs (8 von Mises-Fisher lobes x {mu xyz, kappa, weight}).  FP32 master
 * weights, BF16 tensor-core copies. */
#define LISA_GUIDE_IN 64
#define LISA_GUIDE_HIDDEN 64
#define LISA_GUIDE_OUT 40
#define LISA_GUIDE_NUM_PARAMS (4 * 64 * 64 + 64 * 40 + 4 * 64 + 40)

int lisa_guide_create(uint32_t seed, lisa_guide** out);
void lisa_guide_destroy(lisa_guide* g);
/* FP32 master parameters, LISA_GUIDE_NUM_PARAMS floats: W1..W4 (64x64,
 * row = output), W5 (40x64), b1..b4 (64), b5 (40). */
int lisa_guide_get_params(lisa_guide* g, float* params);
int lisa_guide_set_params(lisa_guide* g, const float* params);
/* Forward pass of n rows (host buffers).  features: n x 64 FP32 (rounded to
 * BF16 on upload); out: n x 40 raw network outputs (FP32). */
int lisa_guide_forward(lisa_guide* g, const float* features, uint32_t n, float* out);
/* One training step on n samples (n multiple of 128): loss =
 * -mean_i(weight_i * log q(dir_i | features_i)).  Writes the loss and,
 * if grads != NULL, the FP32 gradient of that loss (before Adam); then
 * applies one Adam step with learning rate lr when lr > 0. */
int lisa_guide_train_step(lisa_guide* g, const float* features, const float* dirs,
                          const float* weights, uint32_t n, float lr, float* loss,
                          float* grads);
/* Up to `steps` training steps with Adam (learning rate lr > 0), step k on
 * samples [k * chunk, (k + 1) * chunk) of the n given (chunk a multiple of
 * 128; the steps end with the samples), all in one launch: the same
 * updates, bit for bit, as lisa_guide_train_step on each slice in turn.
 * Writes the last step's loss. */
int lisa_guide_train_steps(lisa_guide* g, const float* features, const float* dirs,
                           const float* weights, uint32_t n, uint32_t chunk, uint32_t steps,
                           float lr, float* loss);
/* The guide a renderer trains in guided mode (borrowed). */
int lisa_renderer_guide(lisa_renderer* r, int32_t scene, lisa_guide** out);

/* ---- diagnostics ---------------------------------------------------------- */

/* Runs a kernel that waits, with `limit` polls, on an mbarrier that nothing
 * completes -- the bounded-wait time-out path of the tensor-core kernels,
 * taken on purpose -- and returns the device status word it left in
 * *status_word (LISA_STATUS_WAIT_TIMEOUT set when the wait ran out).  The
 * context stays usable afterwards. */
#define LISA_STATUS_WAIT_TIMEOUT 16u
int lisa_selftest_wait_timeout(uint32_t limit, uint32_t* status_word);

#ifdef __cplusplus
}
#endif

#endif /* LISA_GB_H */

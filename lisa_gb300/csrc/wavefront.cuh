// Kernel interfaces of the wavefront estimator (wavefront.cu) shared with
// the guide (guide.cu) and the API layer (api.cu).
#pragma once

#include "lisa_device.cuh"

namespace lisa {

// Structure-of-arrays wavefront state.  A "slot" is one path in flight.
struct WaveBufs {
  float4* ro[2];    // ray queues (ping-pong): origin xyz, w = slot
  float4* rd[2];    //                          direction xyz, w = scene index (bits; every
                    //                          queued ray runs to RAY_TMAX)
  int2* hit;        // closest hit per queued ray: (triangle, t bits)
  float4* ps_att;   // per slot: throughput xyz, w = stale emitter material (int, -1 none)
  float4* ps_col;   // per slot: radiance xyz,  w = scene<<24 | pixel
  uint32_t* ps_rng; // per slot: LCG state
  float4* nee_a;    // emitter-search queue: hit point xyz, w = slot
  float4* nee_b;    //                       shading normal xyz, w = material
  float4* nee_c;    //                       incoming direction xyz, w = scene index (bits)
  WaveCtrl* ctrl;
  const SceneDev* scenes;
  uint32_t capacity;
  uint32_t refill_busy_max;  // persistent kernels refill a warp once at most this many lanes are busy
  uint32_t physical;         // physically based estimator: ps_att.w = pdf of the last diffuse bounce
  // guided mode (null otherwise)
  float4* rec_list;   // kept training records, 4 float4 each (see below)
  float4* rec_col;    // and their fifth float4, in an array of its own
  uint32_t rec_cap;   // records rec_list holds
  uint32_t rec_salt;  // per-wave salt of the keep decision
  float4* nee_light;  // guided physically based mode: per entry, the emitter sample (2 float4)
  float bsdf_fraction;  // one-sample MIS: probability of the BSDF strategy
};

// Training record of one kept guided vertex, appended to rec_list:
//   (p.xyz, weight = p_bsdf/q)  (N.xyz, w.x)  (view.xyz, w.y)
//   (throughput after the bounce .xyz, w.z)
// and, at the same index of rec_col,
//   (radiance so far .xyz, bits: slot << 1 | emitter flag)
// -- what the collection reads first to learn whether the path gathered
// radiance after the vertex (most do not, and their other 64 B are never
// read).

struct GuideSampling {
  float bsdf_fraction;  // c in q = c p_bsdf + (1-c) p_guide
  int enabled;
};

}  // namespace lisa

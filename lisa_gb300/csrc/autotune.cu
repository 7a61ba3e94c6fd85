// Autotuner for the wavefront's queue and tile sizes.
//
// The reference renders with one fixed launch (render.cc:46-55); here the
// wavefront's size (paths in flight, which sets every SoA queue), the block
// size of the persistent traversal kernels and their refill threshold are
// picked per workload by timing short progressive renders of the workload
// itself (coordinate descent: queue size first, then block size, then the
// refill threshold).  Choices are keyed by device and by a bucketed
// signature of the workload (pixels, triangles, depth, scene count, mode) and
// persisted in a small JSON file, so a batch of the same shape is tuned once.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "lisa_internal.h"

namespace lisa {

Status configure_launch(Renderer& r);

namespace {

struct Entry {
  double paths_in_flight = 0, threads_per_block = 0, blocks_per_sm = 0, refill_idle = 0, mrays_per_s = 0,
         probe_spp = 0;
};

uint32_t log2_bucket(uint64_t v) {
  uint32_t b = 0;
  while (v > 1) {
    v >>= 1;
    ++b;
  }
  return b;
}

// ---- the cache file: {"key": {"field": number, ...}, ...} -------------------

struct Reader {
  const std::string& s;
  size_t i = 0;
  explicit Reader(const std::string& str) : s(str) {}
  void ws() {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
  }
  bool eat(char c) {
    ws();
    if (i < s.size() && s[i] == c) {
      ++i;
      return true;
    }
    return false;
  }
  bool str(std::string& out) {
    ws();
    if (i >= s.size() || s[i] != '"') return false;
    ++i;
    out.clear();
    while (i < s.size() && s[i] != '"') {
      if (s[i] == '\\') return false;  // keys and fields written here need no escapes
      out += s[i++];
    }
    if (i >= s.size()) return false;
    ++i;
    return true;
  }
  bool num(double& v) {
    ws();
    const char* b = s.c_str() + i;
    char* e = nullptr;
    v = std::strtod(b, &e);
    if (e == b) return false;
    i += (size_t)(e - b);
    return true;
  }
};

// Parses the whole file; false if it is not in the format written below.
bool parse_cache(const std::string& text, std::map<std::string, Entry>& out) {
  Reader rd(text);
  if (!rd.eat('{')) return false;
  if (rd.eat('}')) return true;
  do {
    std::string key;
    if (!rd.str(key) || !rd.eat(':') || !rd.eat('{')) return false;
    Entry e;
    if (!rd.eat('}')) {
      do {
        std::string f;
        double v = 0;
        if (!rd.str(f) || !rd.eat(':') || !rd.num(v)) return false;
        if (f == "paths_in_flight") e.paths_in_flight = v;
        else if (f == "threads_per_block") e.threads_per_block = v;
        else if (f == "blocks_per_sm") e.blocks_per_sm = v;
        else if (f == "refill_idle") e.refill_idle = v;
        else if (f == "mrays_per_s") e.mrays_per_s = v;
        else if (f == "probe_spp") e.probe_spp = v;
      } while (rd.eat(','));
      if (!rd.eat('}')) return false;
    }
    out[key] = e;
  } while (rd.eat(','));
  if (!rd.eat('}')) return false;
  rd.ws();
  return rd.i == text.size();
}

Status read_file(const char* path, std::string& text, bool& exists) {
  exists = false;
  text.clear();
  FILE* f = std::fopen(path, "rb");
  if (!f) return Status();
  exists = true;
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
  std::fclose(f);
  return Status();
}

Status load_cache(const char* path, std::map<std::string, Entry>& m) {
  m.clear();
  std::string text;
  bool exists = false;
  LISA_TRY(read_file(path, text, exists));
  if (!exists) return Status();
  if (!parse_cache(text, m)) return Status::invalid(std::string("tuning cache is not in the expected format: ") + path);
  return Status();
}

Status store_cache(const char* path, const std::map<std::string, Entry>& m) {
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return Status::io(std::string("cannot write tuning cache: ") + tmp);
  std::fprintf(f, "{\n");
  size_t k = 0;
  for (const auto& kv : m) {
    const Entry& e = kv.second;
    std::fprintf(f,
                 "  \"%s\": {\"paths_in_flight\": %.0f, \"threads_per_block\": %.0f, \"blocks_per_sm\": %.0f, "
                 "\"refill_idle\": %.0f, \"probe_spp\": %.0f, \"mrays_per_s\": %.3f}%s\n",
                 kv.first.c_str(), e.paths_in_flight, e.threads_per_block, e.blocks_per_sm, e.refill_idle,
                 e.probe_spp, e.mrays_per_s, ++k < m.size() ? "," : "");
  }
  std::fprintf(f, "}\n");
  const bool ok = std::fflush(f) == 0;
  std::fclose(f);
  if (!ok || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return Status::io(std::string("cannot write tuning cache: ") + path);
  }
  return Status();
}

bool key_ok(const char* key) {
  if (!key || !*key || std::strlen(key) >= sizeof(((lisa_tuning*)nullptr)->key)) return false;
  for (const char* p = key; *p; ++p)
    if (*p == '"' || *p == '\\' || (unsigned char)*p < 0x20) return false;
  return true;
}

void to_tuning(const std::string& key, const Entry& e, lisa_tuning* t) {
  std::memset(t, 0, sizeof(*t));
  t->struct_size = sizeof(lisa_tuning);
  t->paths_in_flight = (uint32_t)e.paths_in_flight;
  t->threads_per_block = (uint32_t)e.threads_per_block;
  t->blocks_per_sm = (uint32_t)e.blocks_per_sm;
  t->refill_idle = (uint32_t)e.refill_idle;
  t->probe_spp = (uint32_t)e.probe_spp;
  t->mrays_per_s = e.mrays_per_s;
  std::snprintf(t->key, sizeof(t->key), "%s", key.c_str());
}

Entry from_tuning(const lisa_tuning* t) {
  Entry e;
  e.paths_in_flight = t->paths_in_flight;
  e.threads_per_block = t->threads_per_block;
  e.blocks_per_sm = t->blocks_per_sm;
  e.refill_idle = t->refill_idle;
  e.probe_spp = t->probe_spp;
  e.mrays_per_s = t->mrays_per_s;
  return e;
}

// ---- timing ----------------------------------------------------------------

// Best-of-two probe throughput (Mrays/s) of progressive renders of `spp`
// samples per pixel of every scene, after one untimed render that captures
// the launch sequence's graph.
Status probe(Renderer& r, uint32_t spp, double* mrays) {
  lisa_render_stats st;
  std::memset(&st, 0, sizeof(st));
  LISA_TRY(renderer_render(r, spp, true, &st));
  double best = 0.0;
  for (int k = 0; k < 2; ++k) {
    std::memset(&st, 0, sizeof(st));
    LISA_TRY(renderer_render(r, spp, true, &st));
    const double rays = (double)st.rays_primary + (double)st.rays_bounce + (double)st.rays_shadow;
    if (st.ms_device > 0.0) best = std::max(best, rays / (st.ms_device * 1e3));
  }
  *mrays = best;
  return Status();
}

Status apply_launch(Renderer& r, uint32_t threads, uint32_t refill) {
  r.opts.threads_per_block = threads;
  r.opts.refill_idle = refill;
  LISA_TRY(configure_launch(r));
  if (r.graph_exec) cudaGraphExecDestroy(r.graph_exec);  // launch shapes are baked into the graph
  r.graph_exec = nullptr;
  r.graph_key.clear();
  return Status();
}

}  // namespace

std::string tuning_key(const cudaDeviceProp& p, const lisa_renderer_params* sc, int n, const lisa_options& o) {
  uint64_t px = 0, tris = 0;
  uint32_t bounces = 0;
  for (int i = 0; i < n; ++i) {
    px += (uint64_t)sc[i].width * sc[i].height;
    tris += (uint64_t)std::max<int32_t>(sc[i].num_vertices, 0) / 3;
    bounces = std::max(bounces, sc[i].num_bounces);
  }
  std::string name(p.name);
  for (char& c : name)
    if (!std::isalnum((unsigned char)c)) c = '_';
  char buf[160];
  std::snprintf(buf, sizeof(buf), "%s|sm%d|cc%d.%d|mode%u|est%u|rng%u|px2^%u|tri2^%u|b%u|n2^%u", name.c_str(),
                p.multiProcessorCount, p.major, p.minor, o.mode, o.estimator, o.rng, log2_bucket(px),
                log2_bucket(tris), bounces, log2_bucket((uint64_t)n));
  return buf;
}

Status autotune(const lisa_renderer_params* scenes, int n, const lisa_options* base, const char* cache_path,
                lisa_tuning* out) {
  if (!scenes || n <= 0 || !out) return Status::invalid("no scenes");
  lisa_options o;
  lisa_options_default(&o);
  if (base) {
    if (base->struct_size != sizeof(lisa_options)) return Status::invalid("lisa_options.struct_size mismatch");
    o = *base;
  }
  o.stage_timing = 0;
  o.count_traversal = 0;
  o.use_graph = 1;
  int dev = 0, ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return Status(LISA_ERR_UNSUPPORTED, "no CUDA device");
  }
  LISA_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  LISA_CUDA(cudaGetDeviceProperties(&prop, dev));
  const std::string key = tuning_key(prop, scenes, n, o);
  std::map<std::string, Entry> cache;
  if (cache_path) {
    LISA_TRY(load_cache(cache_path, cache));
    auto it = cache.find(key);
    if (it != cache.end()) {
      to_tuning(key, it->second, out);
      out->candidates = 0;
      return Status();
    }
  }
  uint64_t px = 0;
  for (int i = 0; i < n; ++i) px += (uint64_t)scenes[i].width * scenes[i].height;
  if (px == 0) return Status::invalid("empty images");
  // the probe covers about 2^24 paths, so the larger queue sizes are exercised
  const uint32_t probe_spp = (uint32_t)std::min<uint64_t>(64, std::max<uint64_t>(1, ((1ull << 24) + px - 1) / px));
  const uint64_t probe_paths = px * probe_spp;
  size_t free_b = 0, total_b = 0;
  LISA_CUDA(cudaMemGetInfo(&free_b, &total_b));
  uint32_t maxd = 1;
  for (int i = 0; i < n; ++i) maxd = std::max(maxd, scenes[i].num_bounces);
  // queue bytes per path: rays (2 x 32), hit 8, path state 36, emitter queue
  // 48; guided mode adds 160 B of network outputs and 80 B per depth of
  // training records
  const uint64_t per_path = 156 + (o.mode == LISA_MODE_GUIDED ? 160ull + 80ull * maxd : 0ull);
  std::vector<uint32_t> Ws;
  for (uint32_t w = 1u << 20; w <= (1u << 24); w <<= 1) {
    if (w > probe_paths && !Ws.empty()) break;
    if ((uint64_t)w * per_path > free_b / 2 && !Ws.empty()) break;
    Ws.push_back(w);
  }
  Entry best;
  uint32_t tried = 0;
  const uint32_t t0 = o.threads_per_block ? o.threads_per_block : 128;
  const uint32_t f0 = o.refill_idle ? o.refill_idle : 12;
  std::unique_ptr<Renderer> keep;
  for (uint32_t w : Ws) {
    lisa_options c = o;
    c.paths_in_flight = w;
    c.threads_per_block = t0;
    c.refill_idle = f0;
    Renderer* raw = nullptr;
    LISA_TRY(renderer_create(scenes, n, &c, &raw));
    std::unique_ptr<Renderer> r(raw);
    double m = 0.0;
    LISA_TRY(probe(*r, probe_spp, &m));
    ++tried;
    if (m > best.mrays_per_s) {
      best.paths_in_flight = r->capacity;
      best.threads_per_block = t0;
      best.refill_idle = f0;
      best.mrays_per_s = m;
      keep = std::move(r);
    }
  }
  if (!keep) return Status(LISA_ERR_DEVICE, "autotune: no configuration rendered");
  for (uint32_t t : {64u, 96u, 128u}) {
    if (t == (uint32_t)best.threads_per_block) continue;
    LISA_TRY(apply_launch(*keep, t, (uint32_t)best.refill_idle));
    double m = 0.0;
    LISA_TRY(probe(*keep, probe_spp, &m));
    ++tried;
    if (m > best.mrays_per_s) {
      best.threads_per_block = t;
      best.mrays_per_s = m;
    }
  }
  for (uint32_t f : {8u, 12u, 16u}) {
    if (f == (uint32_t)best.refill_idle) continue;
    LISA_TRY(apply_launch(*keep, (uint32_t)best.threads_per_block, f));
    double m = 0.0;
    LISA_TRY(probe(*keep, probe_spp, &m));
    ++tried;
    if (m > best.mrays_per_s) {
      best.refill_idle = f;
      best.mrays_per_s = m;
    }
  }
  best.blocks_per_sm = 0;
  best.probe_spp = probe_spp;
  keep.reset();
  if (cache_path) {
    std::map<std::string, Entry> again;  // re-read: another process may have added entries
    LISA_TRY(load_cache(cache_path, again));
    again[key] = best;
    LISA_TRY(store_cache(cache_path, again));
  }
  to_tuning(key, best, out);
  out->candidates = tried;
  return Status();
}

}  // namespace lisa

using namespace lisa;

extern "C" {

int lisa_autotune(const lisa_renderer_params* scenes, int32_t n, const lisa_options* base, const char* cache_path,
                  lisa_tuning* out) {
  Status s;
  try {
    s = autotune(scenes, n, base, cache_path, out);
  } catch (const std::bad_alloc&) {
    s = Status(LISA_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    s = Status(LISA_ERR_INVALID, e.what());
  }
  set_last_error(s);
  return s.code;
}

void lisa_tuning_apply(const lisa_tuning* t, lisa_options* o) {
  if (!t || !o) return;
  o->paths_in_flight = t->paths_in_flight;
  o->threads_per_block = t->threads_per_block;
  o->blocks_per_sm = t->blocks_per_sm;
  o->refill_idle = t->refill_idle;
}

int lisa_tuning_cache_lookup(const char* cache_path, const char* key, lisa_tuning* out, int32_t* found) {
  Status s;
  try {
    if (found) *found = 0;
    if (!cache_path || !key || !out || !found) {
      s = Status::invalid("null argument");
    } else {
      std::map<std::string, Entry> m;
      s = load_cache(cache_path, m);
      if (s.ok()) {
        auto it = m.find(key);
        if (it != m.end()) {
          to_tuning(it->first, it->second, out);
          *found = 1;
        }
      }
    }
  } catch (const std::exception& e) {
    s = Status(LISA_ERR_INVALID, e.what());
  }
  set_last_error(s);
  return s.code;
}

int lisa_tuning_cache_store(const char* cache_path, const lisa_tuning* t) {
  Status s;
  try {
    if (!cache_path || !t) {
      s = Status::invalid("null argument");
    } else if (!key_ok(t->key)) {
      s = Status::invalid("tuning key must be non-empty printable text without quotes or backslashes");
    } else {
      std::map<std::string, Entry> m;
      s = load_cache(cache_path, m);
      if (s.ok()) {
        m[t->key] = from_tuning(t);
        s = store_cache(cache_path, m);
      }
    }
  } catch (const std::exception& e) {
    s = Status(LISA_ERR_INVALID, e.what());
  }
  set_last_error(s);
  return s.code;
}

}  // extern "C"

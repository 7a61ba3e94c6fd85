// .rto scene parser and parallel OBJ loader (host side of the boundary).
//
// The grammar is LiSA's (src/LiSA/src/scene_parser.cc:35-261): the reference
// finds every key with std::regex searches over the comment-stripped file.
// This file implements the same language with a hand-written scanner: each
// search below states the reference pattern it is equivalent to, including
// its quirks (leftmost substring matches, "roughness " needing a space before
// '=', " n" needing a space before 'n', colours above 1 divided by 255,
// trailing blanks kept in output_image, a '\r' inside a comment keeping the
// comment).  Errors return LISA_ERR_PARSE / LISA_ERR_IO with the reference's
// message instead of exit(1).
//
// The OBJ reader follows parse_obj (src/LiSA/src/parse_obj.cc:24-69): lines
// split on single spaces, "v" / "vn" / "f a/b/c" records, faces de-indexed
// into a flat soup (three vertices + three normals per triangle), only the
// first three corners of a face used.  It runs on all host threads: chunks
// at line boundaries are classified and counted, prefix-summed, then parsed
// in place.
#include "lisa_internal.h"

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

namespace lisa {

namespace {

// ECMAScript \s over bytes.
inline bool is_ws(char c) {
  return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}
inline bool is_digit(char c) { return c >= '0' && c <= '9'; }
inline bool is_name(char c) {
  return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z') || is_digit(c) || c == '_';
}
// ECMAScript '.' : anything but a line terminator.
inline bool is_dot(char c) { return c != '\n' && c != '\r'; }

size_t skip_ws(const std::string& s, size_t i) {
  while (i < s.size() && is_ws(s[i])) ++i;
  return i;
}

// Float token of the grammar, [+-]?([0-9]*[.])?[0-9]+ (scene_parser.cc:71),
// matched greedily at i.  Returns the end position or npos.
size_t match_float_tok(const std::string& s, size_t i) {
  size_t p = i;
  if (p < s.size() && (s[p] == '+' || s[p] == '-')) ++p;
  size_t d1 = p;
  while (d1 < s.size() && is_digit(s[d1])) ++d1;
  if (d1 < s.size() && s[d1] == '.' && d1 + 1 < s.size() && is_digit(s[d1 + 1])) {
    size_t d2 = d1 + 1;
    while (d2 < s.size() && is_digit(s[d2])) ++d2;
    return d2;
  }
  if (d1 > p) return d1;
  return std::string::npos;
}

// stof of a grammar token: the token is plain decimal, so strtof's correctly
// rounded result is what std::stof returns.
float tok_to_float(const std::string& s, size_t b, size_t e) {
  std::string t = s.substr(b, e - b);
  return std::strtof(t.c_str(), nullptr);
}

// Leftmost match of  key \s* = \s* F   (search_float, scene_parser.cc:81-83).
bool search_float(const std::string& s, const std::string& key, float* out) {
  for (size_t at = s.find(key); at != std::string::npos; at = s.find(key, at + 1)) {
    size_t p = skip_ws(s, at + key.size());
    if (p >= s.size() || s[p] != '=') continue;
    p = skip_ws(s, p + 1);
    size_t e = match_float_tok(s, p);
    if (e == std::string::npos) continue;
    *out = tok_to_float(s, p, e);
    return true;
  }
  return false;
}

// Leftmost match of  key \s* = \s* \( \s*F\s* (, \s*F\s*){n-1} \)
// (search_vector, scene_parser.cc:66-79).
bool search_vector(const std::string& s, const std::string& key, int n, float* out) {
  for (size_t at = s.find(key); at != std::string::npos; at = s.find(key, at + 1)) {
    size_t p = skip_ws(s, at + key.size());
    if (p >= s.size() || s[p] != '=') continue;
    p = skip_ws(s, p + 1);
    if (p >= s.size() || s[p] != '(') continue;
    ++p;
    bool ok = true;
    float vals[8];
    for (int k = 0; k < n && ok; ++k) {
      p = skip_ws(s, p);
      size_t e = match_float_tok(s, p);
      if (e == std::string::npos) {
        ok = false;
        break;
      }
      vals[k] = tok_to_float(s, p, e);
      p = skip_ws(s, e);
      const char want = (k == n - 1) ? ')' : ',';
      if (p >= s.size() || s[p] != want) {
        ok = false;
        break;
      }
      ++p;
    }
    if (!ok) continue;
    std::memcpy(out, vals, sizeof(float) * n);
    return true;
  }
  return false;
}

// Leftmost match of  param \s* = \s* ([0-9]+)  (search_int, :85-87), or for
// output_image  param \s* = \s* (([a-zA-Z0-9]|_|\/|.)+)  (:94), whose '.'
// is unescaped and so takes the rest of the line, trailing blanks included.
bool search_param(const std::string& s, const std::string& key, bool is_string, std::string* out) {
  for (size_t at = s.find(key); at != std::string::npos; at = s.find(key, at + 1)) {
    size_t p = skip_ws(s, at + key.size());
    if (p >= s.size() || s[p] != '=') continue;
    const size_t eq = p;
    p = skip_ws(s, p + 1);
    if (!is_string) {
      size_t e = p;
      while (e < s.size() && is_digit(s[e])) ++e;
      if (e == p) continue;
      *out = s.substr(p, e - p);
      return true;
    }
    // greedy \s* backs off one character at a time until the capture can
    // start on a non-line-terminator
    for (size_t start = p; start > eq; --start) {
      if (start < s.size() && is_dot(s[start])) {
        size_t e = start;
        while (e < s.size() && is_dot(s[e])) ++e;
        *out = s.substr(start, e - start);
        return true;
      }
    }
  }
  return false;
}

// Comment removal: \/\*((.|\n)*?)\*\/ (scene_parser.cc:59-64).  The body may
// hold '\n' but not '\r' ('.' excludes it), in which case that "/*" opens no
// comment.
std::string remove_comments(const std::string& f) {
  std::string out;
  out.reserve(f.size());
  size_t i = 0;
  while (i < f.size()) {
    if (f[i] == '/' && i + 1 < f.size() && f[i + 1] == '*') {
      size_t j = i + 2;
      bool closed = false;
      while (j < f.size()) {
        if (f[j] == '\r') break;
        if (f[j] == '*' && j + 1 < f.size() && f[j + 1] == '/') {
          closed = true;
          break;
        }
        ++j;
      }
      if (closed) {
        i = j + 2;
        continue;
      }
    }
    out.push_back(f[i]);
    ++i;
  }
  return out;
}

// All non-overlapping matches, left to right, of  head \s*\{ [^}]*  where
// head is "mesh" / "camera" (scene_parser.cc:37-38) or, for materials,
// material \s+ NAME \s* \{ [^}]*  (:36).  Returns [begin, end) spans.
struct Block {
  size_t b, e;
  std::string name;  // materials only
};

std::vector<Block> find_blocks(const std::string& s, const std::string& head, bool named) {
  std::vector<Block> out;
  size_t from = 0;
  while (true) {
    bool found = false;
    for (size_t at = s.find(head, from); at != std::string::npos; at = s.find(head, at + 1)) {
      size_t p = at + head.size();
      std::string name;
      if (named) {
        size_t q = p;
        while (q < s.size() && is_ws(s[q])) ++q;
        if (q == p) continue;  // \s+
        size_t ne = q;
        while (ne < s.size() && is_name(s[ne])) ++ne;
        if (ne == q) continue;
        name = s.substr(q, ne - q);
        p = ne;
      }
      p = skip_ws(s, p);
      if (p >= s.size() || s[p] != '{') continue;
      size_t e = s.find('}', p + 1);
      if (e == std::string::npos) e = s.size();
      out.push_back({at, e, name});
      from = e;
      found = true;
      break;
    }
    if (!found) break;
  }
  return out;
}

bool contains_emit_true(const std::string& s) {
  // emit \s* = \s* true
  for (size_t at = s.find("emit"); at != std::string::npos; at = s.find("emit", at + 1)) {
    size_t p = skip_ws(s, at + 4);
    if (p >= s.size() || s[p] != '=') continue;
    p = skip_ws(s, p + 1);
    if (s.compare(p, 4, "true") == 0) return true;
  }
  return false;
}

// Leftmost match of (roughness | n)\s*=\s*F  (scene_parser.cc:151-152): the
// alternatives are "roughness " (trailing blank) and " n" (leading blank).
bool search_roughness_or_n(const std::string& s, float* out) {
  for (size_t i = 0; i < s.size(); ++i) {
    size_t p;
    if (s.compare(i, 10, "roughness ") == 0) {
      p = i + 10;
    } else if (s.compare(i, 2, " n") == 0) {
      p = i + 2;
    } else {
      continue;
    }
    p = skip_ws(s, p);
    if (p >= s.size() || s[p] != '=') continue;
    p = skip_ws(s, p + 1);
    size_t e = match_float_tok(s, p);
    if (e == std::string::npos) continue;
    *out = tok_to_float(s, p, e);
    return true;
  }
  return false;
}

// material \s* = \s* (NAME)  (scene_parser.cc:177)
bool search_mesh_material(const std::string& s, std::string* out) {
  for (size_t at = s.find("material"); at != std::string::npos; at = s.find("material", at + 1)) {
    size_t p = skip_ws(s, at + 8);
    if (p >= s.size() || s[p] != '=') continue;
    p = skip_ws(s, p + 1);
    size_t e = p;
    while (e < s.size() && is_name(s[e])) ++e;
    if (e == p) continue;
    *out = s.substr(p, e - p);
    return true;
  }
  return false;
}

// obj_file \s* = \s* (.+\.obj)  (scene_parser.cc:190): greedy, so the
// capture runs to the last ".obj" on the line.
bool search_obj_file(const std::string& s, std::string* out) {
  for (size_t at = s.find("obj_file"); at != std::string::npos; at = s.find("obj_file", at + 1)) {
    size_t p = skip_ws(s, at + 8);
    if (p >= s.size() || s[p] != '=') continue;
    const size_t eq = p;
    p = skip_ws(s, p + 1);
    for (size_t start = p; start > eq; --start) {
      if (start >= s.size() || !is_dot(s[start])) continue;
      size_t le = start;
      while (le < s.size() && is_dot(s[le])) ++le;
      // last ".obj" beginning at least one character after start
      for (size_t k = le; k >= start + 5; --k) {
        if (s.compare(k - 4, 4, ".obj") == 0) {
          *out = s.substr(start, k - start);
          return true;
        }
      }
    }
  }
  return false;
}

lisa_material mk_material_emit(lisa_float3 color) {
  // structs.hh:25-31; the fields the reference leaves unset are zeroed.
  lisa_material m;
  std::memset(&m, 0, sizeof(m));
  m.emit = 1;
  m.emission_color = color;
  m.alpha = 1.0f;
  return m;
}

lisa_material mk_material_diffuse(lisa_float3 color, float alpha, float param) {
  // structs.hh:41-52
  lisa_material m;
  std::memset(&m, 0, sizeof(m));
  if (alpha < 1.0f)
    m.n = param;
  else
    m.roughness = param;
  m.alpha = alpha;
  m.diffuse_color = color;
  m.emit = 0;
  return m;
}

bool read_whole_file(const std::string& path, std::string* out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out->resize(n > 0 ? (size_t)n : 0);
  size_t got = n > 0 ? std::fread(&(*out)[0], 1, (size_t)n, f) : 0;
  std::fclose(f);
  return got == out->size();
}

// read_file (scene_parser.cc:5-19) keeps each line and appends '\n', so a
// last line without a newline gains one.
std::string normalise_lines(const std::string& raw) {
  if (!raw.empty() && raw.back() != '\n') return raw + "\n";
  return raw;
}

bool file_exists(const std::string& p) {
  FILE* f = std::fopen(p.c_str(), "rb");
  if (!f) return false;
  std::fclose(f);
  return true;
}

// ---------------------------------------------------------------------------
// OBJ

// stof / stoi of one space-separated token (parse_obj.cc:51-60): leading
// blanks skipped, longest numeric prefix converted, nothing converted is an
// error.
bool obj_float(const char* b, const char* e, float* out) {
  while (b < e && is_ws(*b)) ++b;
  if (b < e && *b == '+') {
    // std::from_chars has no '+'; strtof accepts it
    ++b;
    if (b < e && (*b == '+' || *b == '-')) return false;
  }
  auto r = std::from_chars(b, e, *out, std::chars_format::general);
  if (r.ec == std::errc()) return true;
  if (r.ec == std::errc::result_out_of_range) {
    std::string t(b, e);
    *out = std::strtof(t.c_str(), nullptr);
    return true;
  }
  // hexadecimal floats and other strtof-only forms
  std::string t(b, e);
  char* endp = nullptr;
  errno = 0;
  *out = std::strtof(t.c_str(), &endp);
  return endp != t.c_str();
}

bool obj_int(const char* b, const char* e, long* out) {
  while (b < e && is_ws(*b)) ++b;
  if (b < e && *b == '+') ++b;
  auto r = std::from_chars(b, e, *out);
  return r.ec == std::errc();
}

struct ObjChunk {
  size_t b, e;
  size_t nv = 0, nn = 0, nf = 0;
};

// Line kinds by first space-separated token.
enum { LINE_OTHER = 0, LINE_V = 1, LINE_VN = 2, LINE_F = 3 };
inline int line_kind(const char* p, const char* e) {
  // first space-separated token compared with "v", "vn", "f" (parse_obj.cc:51-56)
  const char* t = p;
  while (t < e && *t != ' ') ++t;
  const size_t n = (size_t)(t - p);
  if (n == 1 && p[0] == 'v') return LINE_V;
  if (n == 2 && p[0] == 'v' && p[1] == 'n') return LINE_VN;
  if (n == 1 && p[0] == 'f') return LINE_F;
  return LINE_OTHER;
}

// Tokens of a line split on ' ' (parse_obj.cc:4-22): empty tokens kept.
inline int split_tokens(const char* p, const char* e, const char** tb, const char** te, int maxt) {
  int n = 0;
  const char* s = p;
  for (const char* q = p;; ++q) {
    if (q == e || *q == ' ') {
      if (n < maxt) {
        tb[n] = s;
        te[n] = q;
      }
      ++n;
      if (q == e) break;
      s = q + 1;
    }
  }
  return n;
}

}  // namespace

namespace {

// One OBJ file as a de-indexed soup: three vertices and three normals per
// face.  A file of at least 1 MB is split over up to `max_threads` threads.
struct ObjSoup {
  std::vector<lisa_float3> vertices, normals;
};

// Runs fn(t) for t in [0, n): on this thread when n is 1.
template <class F>
void run_threads(unsigned n, F&& fn) {
  if (n <= 1) {
    fn(0u);
    return;
  }
  std::vector<std::thread> th;
  for (unsigned t = 0; t < n; ++t) th.emplace_back([&fn, t] { fn(t); });
  for (auto& x : th) x.join();
}

// The whole file into an uninitialised buffer; a file of at least 8 MB is
// read by `nth` threads, each its own byte range (pread).
bool read_file_parallel(const std::string& path, unsigned nth, std::unique_ptr<char[]>* buf, size_t* size) {
  const int fd = ::open(path.c_str(), O_RDONLY);
  if (fd < 0) return false;
  struct stat sb;
  if (::fstat(fd, &sb) != 0 || sb.st_size < 0) {
    ::close(fd);
    return false;
  }
  const size_t n = (size_t)sb.st_size;
  buf->reset(new char[n > 0 ? n : 1]);
  if (n < (8u << 20)) nth = 1;
  std::atomic<bool> ok{true};
  run_threads(nth, [&](unsigned t) {
    size_t off = n * t / nth;
    const size_t end = n * (t + 1) / nth;
    while (off < end) {
      const ssize_t r = ::pread(fd, buf->get() + off, end - off, (off_t)off);
      if (r <= 0) {
        ok = false;
        return;
      }
      off += (size_t)r;
    }
  });
  ::close(fd);
  *size = n;
  return ok;
}

Status obj_parse(const std::string& path, unsigned max_threads, ObjSoup& out) {
  std::unique_ptr<char[]> data;
  size_t n = 0;
  if (!read_file_parallel(path, std::max(1u, std::min(64u, max_threads)), &data, &n))
    return Status::io(path + " not found.");
  const char* base = data.get();
  unsigned nth = std::max(1u, std::min(64u, max_threads));
  if (n < (1u << 20)) nth = 1;
  std::vector<ObjChunk> ch(nth);
  for (unsigned t = 0; t < nth; ++t) {
    size_t b = n * t / nth, e = n * (t + 1) / nth;
    ch[t].b = b;
    ch[t].e = e;
  }
  // align chunk borders to line starts
  for (unsigned t = 1; t < nth; ++t) {
    size_t b = ch[t].b;
    while (b < n && base[b - 1] != '\n') ++b;
    ch[t].b = b;
    ch[t - 1].e = b;
  }
  ch[nth - 1].e = n;
  auto for_lines = [&](const ObjChunk& c, auto&& fn) {
    size_t i = c.b;
    while (i < c.e) {
      size_t j = i;
      while (j < c.e && base[j] != '\n') ++j;
      if (!fn(base + i, base + j)) return false;
      i = j + 1;
    }
    return true;
  };
  // pass 1: count records per chunk
  run_threads(nth, [&](unsigned t) {
    for_lines(ch[t], [&](const char* p, const char* e) {
      int k = line_kind(p, e);
      if (k == LINE_V) ch[t].nv++;
      else if (k == LINE_VN) ch[t].nn++;
      else if (k == LINE_F) ch[t].nf++;
      return true;
    });
  });
  std::vector<size_t> ov(nth + 1, 0), on(nth + 1, 0), of(nth + 1, 0);
  for (unsigned t = 0; t < nth; ++t) {
    ov[t + 1] = ov[t] + ch[t].nv;
    on[t + 1] = on[t] + ch[t].nn;
    of[t + 1] = of[t] + ch[t].nf;
  }
  std::vector<float> vt(ov[nth] * 3), nt(on[nth] * 3);
  std::vector<long> fv(of[nth] * 3), fn(of[nth] * 3);
  std::atomic<bool> bad{false};
  std::vector<std::string> errs(nth);
  // pass 2: parse in place
  {
    run_threads(nth, [&](unsigned t) {
        size_t iv = ov[t], in = on[t], iff = of[t];
        bool ok = for_lines(ch[t], [&](const char* p, const char* e) {
          int k = line_kind(p, e);
          if (k == LINE_OTHER) return true;
          const char* tb[5];
          const char* te[5];
          int nt_ = split_tokens(p, e, tb, te, 5);
          if (k == LINE_V || k == LINE_VN) {
            float* dst = (k == LINE_V) ? &vt[3 * iv++] : &nt[3 * in++];
            if (nt_ < 4) {
              errs[t] = "OBJ record with fewer than 3 coordinates";
              return false;
            }
            for (int c = 0; c < 3; ++c)
              if (!obj_float(tb[1 + c], te[1 + c], &dst[c])) {
                errs[t] = "bad number in OBJ vertex record";
                return false;
              }
            return true;
          }
          // face: first three corners, v/vt/vn
          if (nt_ < 4) {
            errs[t] = "OBJ face with fewer than 3 corners";
            return false;
          }
          for (int c = 0; c < 3; ++c) {
            const char* sb = tb[1 + c];
            const char* se = te[1 + c];
            const char* s1 = (const char*)std::memchr(sb, '/', se - sb);
            const char* s2 = s1 ? (const char*)std::memchr(s1 + 1, '/', se - s1 - 1) : nullptr;
            if (!s2) {
              errs[t] = "OBJ face corner without v/vt/vn indices";
              return false;
            }
            const char* s3 = (const char*)std::memchr(s2 + 1, '/', se - s2 - 1);
            long a, b;
            if (!obj_int(sb, s1, &a) || !obj_int(s2 + 1, s3 ? s3 : se, &b)) {
              errs[t] = "bad index in OBJ face";
              return false;
            }
            fv[3 * iff + c] = a - 1;
            fn[3 * iff + c] = b - 1;
          }
          ++iff;
          return true;
        });
        if (!ok) bad = true;
      });
  }
  if (bad) {
    for (auto& e : errs)
      if (!e.empty()) return Status::parse(path + ": " + e);
  }
  // de-index (parse_obj.cc:56-61)
  const size_t nfaces = of[nth];
  out.vertices.resize(3 * nfaces);
  out.normals.resize(3 * nfaces);
  const long nvt = (long)ov[nth], nnt = (long)on[nth];
  std::atomic<bool> range_bad{false};
  const unsigned nt2 = nfaces > 100000 ? nth : 1;
  run_threads(nt2, [&](unsigned t) {
    size_t b = nfaces * t / nt2, e = nfaces * (t + 1) / nt2;
    for (size_t f = b; f < e; ++f)
      for (int c = 0; c < 3; ++c) {
        long a = fv[3 * f + c], q = fn[3 * f + c];
        if (a < 0 || a >= nvt || q < 0 || q >= nnt) {
          range_bad = true;
          return;
        }
        out.vertices[3 * f + c] = {vt[3 * a], vt[3 * a + 1], vt[3 * a + 2]};
        out.normals[3 * f + c] = {nt[3 * q], nt[3 * q + 1], nt[3 * q + 2]};
      }
  });
  if (range_bad) return Status::parse(path + ": face index out of range");
  return Status();
}

unsigned host_threads() { return std::max(1u, std::min(64u, std::thread::hardware_concurrency())); }

void soup_append(Scene& sc, const ObjSoup& o, int32_t mat_idx) {
  sc.vertices.insert(sc.vertices.end(), o.vertices.begin(), o.vertices.end());
  sc.normals.insert(sc.normals.end(), o.normals.begin(), o.normals.end());
  sc.mat_indices.resize(sc.mat_indices.size() + o.vertices.size() / 3, mat_idx);
}

// The OBJ files of a scene's meshes, appended in declaration order.  Files
// under 1 MB are parsed side by side, one file per thread (a scene of many
// small meshes); larger ones one at a time on all threads.  The error
// reported is that of the first failing file in declaration order, as the
// reference, which loads them one after the other, would report.
struct ObjJob {
  std::string path;
  int32_t mat_idx;
};

Status obj_append_all(Scene& sc, const std::vector<ObjJob>& jobs) {
  const size_t n = jobs.size();
  std::vector<ObjSoup> soups(n);
  std::vector<Status> st(n);
  std::vector<size_t> small, large;
  for (size_t i = 0; i < n; ++i) {
    FILE* f = std::fopen(jobs[i].path.c_str(), "rb");
    long sz = 0;
    if (f) {
      std::fseek(f, 0, SEEK_END);
      sz = std::ftell(f);
      std::fclose(f);
    }
    (sz >= (1l << 20) ? large : small).push_back(i);
  }
  const unsigned nth = host_threads();
  std::atomic<size_t> next{0};
  run_threads(std::min<size_t>(nth, small.size()), [&](unsigned) {
    for (size_t k = next++; k < small.size(); k = next++) {
      const size_t i = small[k];
      st[i] = obj_parse(jobs[i].path, 1, soups[i]);
    }
  });
  for (size_t i : large) st[i] = obj_parse(jobs[i].path, nth, soups[i]);
  for (size_t i = 0; i < n; ++i)
    if (!st[i].ok()) return st[i];
  size_t tv = sc.vertices.size();
  for (const ObjSoup& o : soups) tv += o.vertices.size();
  sc.vertices.reserve(tv);
  sc.normals.reserve(tv);
  sc.mat_indices.reserve(tv / 3);
  for (size_t i = 0; i < n; ++i) {
    soup_append(sc, soups[i], jobs[i].mat_idx);
    ObjSoup().vertices.swap(soups[i].vertices);  // free as we go
    ObjSoup().normals.swap(soups[i].normals);
  }
  return Status();
}

}  // namespace

Status obj_append(Scene& sc, const std::string& path, int32_t mat_idx) {
  ObjSoup o;
  LISA_TRY(obj_parse(path, host_threads(), o));
  soup_append(sc, o, mat_idx);
  return Status();
}

Status parse_scene_text(const std::string& raw, const std::string& base_dir, Scene& sc) {
  const std::string file = remove_comments(normalise_lines(raw));
  std::string v;
  auto int_param = [&](const char* key, uint32_t* dst) -> Status {
    if (!search_param(file, key, false, &v)) return Status::parse(std::string("Param ") + key + " not found.");
    errno = 0;
    char* endp = nullptr;
    long long x = std::strtoll(v.c_str(), &endp, 10);
    if (errno == ERANGE || x > 2147483647LL) return Status::parse(std::string("Param ") + key + " out of range.");
    *dst = (uint32_t)x;
    return Status();
  };
  Status st;
  if (!(st = int_param("width", &sc.width)).ok()) return st;
  if (!(st = int_param("height", &sc.height)).ok()) return st;
  if (!(st = int_param("num_samples", &sc.num_samples)).ok()) return st;
  if (!(st = int_param("num_bounces", &sc.num_bounces)).ok()) return st;
  if (!search_param(file, "output_image", true, &sc.output_image))
    return Status::parse("Param output_image not found.");

  // materials (scene_parser.cc:106-163)
  auto mats = find_blocks(file, "material", true);
  if (mats.empty()) return Status::parse("Error in materials declaration: no valid materials declared.");
  for (const Block& b : mats) {
    const std::string s = file.substr(b.b, b.e - b.b);
    const bool is_light = contains_emit_true(s);
    float c4[4];
    if (!search_vector(s, "color", 4, c4))
      return Status::parse("Error in materials declaration: no valid color provided in material " + b.name + ".");
    lisa_float3 color = {c4[0], c4[1], c4[2]};
    const float alpha = c4[3];
    if (color.x > 1 || color.y > 1 || color.z > 1) {
      color.x = (float)((double)color.x / 255.0);
      color.y = (float)((double)color.y / 255.0);
      color.z = (float)((double)color.z / 255.0);
    }
    lisa_material m;
    if (is_light) {
      m = mk_material_emit(color);
    } else {
      float param;
      if (!search_roughness_or_n(s, &param))
        return Status::parse("Error in materials declaration: no valid roughness|refractive index in material " +
                             b.name + ".");
      m = mk_material_diffuse(color, alpha, param);
    }
    if (sc.mat_name_idx.find(b.name) == sc.mat_name_idx.end()) {
      sc.materials.push_back(m);
      sc.mat_name_idx[b.name] = (int)sc.materials.size() - 1;
    }
  }

  // meshes (scene_parser.cc:165-198): declarations in order up to the first
  // bad one, then their OBJ files; an OBJ error before that declaration
  // comes first, as in the reference's one-by-one loading
  std::vector<ObjJob> jobs;
  Status decl;
  for (const Block& b : find_blocks(file, "mesh", false)) {
    const std::string s = file.substr(b.b, b.e - b.b);
    std::string mname;
    if (!search_mesh_material(s, &mname)) {
      decl = Status::parse("Error in mesh declaration: no valid material provided");
      break;
    }
    auto it = sc.mat_name_idx.find(mname);
    if (it == sc.mat_name_idx.end()) {
      decl = Status::parse("Error in mesh declaration: " + mname + " material not found");
      break;
    }
    std::string path;
    if (!search_obj_file(s, &path)) {
      decl = Status::parse("Error in mesh declaration: no valid obj_file provided");
      break;
    }
    // The reference opens the path relative to the working directory.  A
    // relative path that does not exist there is also tried relative to the
    // directory of the .rto file.
    std::string use = path;
    if (!file_exists(use) && !base_dir.empty() && !path.empty() && path[0] != '/') {
      std::string alt = base_dir + "/" + path;
      if (file_exists(alt)) use = alt;
    }
    jobs.push_back({use, it->second});
  }
  if (!(st = obj_append_all(sc, jobs)).ok()) return st;
  if (!decl.ok()) return decl;

  // camera (scene_parser.cc:200-245)
  auto cams = find_blocks(file, "camera", false);
  if (cams.size() != 1) return Status::parse("Error in camera declaration: no valid camera declared.");
  const std::string s = file.substr(cams[0].b, cams[0].e - cams[0].b);
  float p3[3];
  if (!search_vector(s, "position", 3, p3))
    return Status::parse("Error in camera declaration: no valid position provided.");
  sc.camera.eye = {p3[0], p3[1], p3[2]};
  if (!search_vector(s, "look_at", 3, p3))
    return Status::parse("Error in camera declaration: no valid look_at provided.");
  sc.camera.look_at = {p3[0], p3[1], p3[2]};
  if (!search_float(s, "fov", &sc.camera.fov))
    return Status::parse("Error in camera declaration: no valid fov provided.");
  return Status();
}

Status parse_scene_file(const std::string& path, Scene& sc) {
  std::string raw;
  if (!read_whole_file(path, &raw)) return Status::io(path + " not found");
  std::string dir;
  size_t slash = path.find_last_of('/');
  if (slash != std::string::npos) dir = path.substr(0, slash);
  return parse_scene_text(raw, dir, sc);
}

void scene_fill_params(const Scene& sc, lisa_renderer_params* p) {
  // mk_params (scene_parser.cc:247-261): borrowed pointers into the scene
  std::memset(p, 0, sizeof(*p));
  p->vertices = sc.vertices.data();
  p->normals = sc.normals.data();
  p->materials = sc.materials.data();
  p->mat_indices = sc.mat_indices.data();
  p->num_vertices = (int32_t)sc.vertices.size();
  p->num_materials = (int32_t)sc.materials.size();
  p->width = sc.width;
  p->height = sc.height;
  p->camera = sc.camera;
  p->num_samples = sc.num_samples;
  p->num_bounces = sc.num_bounces;
  p->output_image = sc.output_image.c_str();
}

}  // namespace lisa

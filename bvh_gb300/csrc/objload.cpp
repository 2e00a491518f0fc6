// objload.cpp -- parallel Wavefront OBJ reader straight to the 9 SoA triangle arrays.
//
// Reference: loadOBJ, src/loader.cpp:10-74.  Same rules: lines that are empty or start with '#'
// are skipped; the first whitespace-separated token is the prefix; "v" reads three floats; "f"
// reads vertex indices (the text before the first '/', parsed like std::stoi), negative ones
// counting back from the vertices read so far, positive ones 1-based; faces are fan-triangulated
// and a triangle with an index outside the vertices read so far is skipped; other prefixes are
// ignored.
//
// The file is split at line boundaries into one chunk per thread.  Pass 1 counts each chunk's
// vertices, pass 2 parses vertices into their global slots and faces into vertex-index triples
// (each chunk knows how many vertices precede it, which is all a relative index or the
// "read so far" check needs), pass 3 gathers the triangles' corners into the SoA arrays.
#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bvh_gb300.h"

namespace {

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f'; }

struct Chunk {
  const char* b;
  const char* e;
  size_t vertices = 0;   // 'v' lines in the chunk
  size_t vbase = 0;      // vertices before the chunk
  std::vector<int32_t> tri;  // 3 vertex indices per triangle
  bool bad = false;      // an index the reference's std::stoi would reject
};

// One line [p, end): its prefix token and the rest.
inline const char* skip_space(const char* p, const char* end) {
  while (p < end && is_space(*p)) ++p;
  return p;
}
inline const char* token_end(const char* p, const char* end) {
  while (p < end && !is_space(*p)) ++p;
  return p;
}

// Three floats as `std::istream >> float` reads them (strtof on each whitespace token); a missing
// or unreadable value leaves 0 (C++11 extraction failure writes 0), and after a token with
// trailing characters the next extraction fails, so the remaining values stay 0 (well-formed
// numbers parse identically).
inline void parse_vertex(const char* p, const char* end, float out[3]) {
  char buf[128];
  for (int k = 0; k < 3; ++k) {
    out[k] = 0.0f;
    p = skip_space(p, end);
    const char* q = token_end(p, end);
    if (p == q) {
      for (int j = k + 1; j < 3; ++j) out[j] = 0.0f;
      return;
    }
    const size_t len = (size_t)(q - p) < sizeof(buf) - 1 ? (size_t)(q - p) : sizeof(buf) - 1;
    memcpy(buf, p, len);
    buf[len] = 0;
    char* stop = nullptr;
    const float v = strtof(buf, &stop);
    if (stop == buf) {  // extraction failed: the rest stay 0
      for (int j = k + 1; j < 3; ++j) out[j] = 0.0f;
      return;
    }
    out[k] = v;
    if (stop != buf + len) return;  // trailing characters: the following extractions fail
    p = q;
  }
}

// std::stoi on the text before the first '/': leading spaces, sign, digits; false where stoi
// would throw (no digits, or out of int range).
inline bool parse_index(const char* p, const char* q, long* out) {
  const char* slash = (const char*)memchr(p, '/', (size_t)(q - p));
  const char* e = slash ? slash : q;
  char buf[64];
  const size_t len = (size_t)(e - p) < sizeof(buf) - 1 ? (size_t)(e - p) : sizeof(buf) - 1;
  memcpy(buf, p, len);
  buf[len] = 0;
  errno = 0;
  char* stop = nullptr;
  const long v = strtol(buf, &stop, 10);
  if (stop == buf || errno == ERANGE || v < INT_MIN || v > INT_MAX) return false;
  *out = v;
  return true;
}

void count_chunk(Chunk& c) {
  const char* p = c.b;
  while (p < c.e) {
    const char* nl = (const char*)memchr(p, '\n', (size_t)(c.e - p));
    const char* end = nl ? nl : c.e;
    if (end > p && *p != '#') {
      const char* t = skip_space(p, end);
      const char* te = token_end(t, end);
      if (te - t == 1 && *t == 'v') ++c.vertices;
    }
    p = end + 1;
  }
}

void parse_chunk(Chunk& c, float* vx) {
  const char* p = c.b;
  size_t vi = c.vbase;  // vertices read so far
  std::vector<int> face;
  while (p < c.e) {
    const char* nl = (const char*)memchr(p, '\n', (size_t)(c.e - p));
    const char* end = nl ? nl : c.e;
    if (end > p && *p != '#') {
      const char* t = skip_space(p, end);
      const char* te = token_end(t, end);
      if (te - t == 1 && *t == 'v') {
        parse_vertex(te, end, vx + 3 * vi);
        ++vi;
      } else if (te - t == 1 && *t == 'f') {
        face.clear();
        const char* q = te;
        while (true) {
          q = skip_space(q, end);
          if (q >= end) break;
          const char* qe = token_end(q, end);
          long raw = 0;
          if (!parse_index(q, qe, &raw)) {
            c.bad = true;
            return;
          }
          face.push_back(raw < 0 ? (int)((long)vi + raw) : (int)(raw - 1));
          q = qe;
        }
        for (size_t i = 1; i + 1 < face.size(); ++i) {
          const int a = face[0], b = face[i], d = face[i + 1];
          if (a < 0 || (size_t)a >= vi || b < 0 || (size_t)b >= vi || d < 0 || (size_t)d >= vi) continue;
          c.tri.push_back(a);
          c.tri.push_back(b);
          c.tri.push_back(d);
        }
      }
    }
    p = end + 1;
  }
}

template <typename F>
void parallel(int threads, F f) {
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(f, t);
  f(0);
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" bvh_status bvh_load_obj(const char* path, int32_t threads, int32_t pinned, bvh_obj_mesh* out) {
  if (!path || !out) return BVH_ERR_INVALID_ARG;
  memset(out, 0, sizeof(*out));
  FILE* f = fopen(path, "rb");
  if (!f) return BVH_ERR_INVALID_ARG;
  std::string data;
  if (fseek(f, 0, SEEK_END) == 0) {
    const long size = ftell(f);
    if (size > 0) {
      data.resize((size_t)size);
      fseek(f, 0, SEEK_SET);
      if (fread(&data[0], 1, (size_t)size, f) != (size_t)size) data.clear();
    }
  }
  fclose(f);
  if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
  if (threads <= 0) threads = 1;
  if (threads > 256) threads = 256;
  if (data.size() < (size_t)threads * 4096) threads = 1;
  // chunks at line boundaries
  std::vector<Chunk> ch((size_t)threads);
  const char* base = data.data();
  const char* stop = base + data.size();
  const char* p = base;
  for (int t = 0; t < threads; ++t) {
    ch[t].b = p;
    const char* q = t + 1 == threads ? stop : base + data.size() * (size_t)(t + 1) / (size_t)threads;
    if (q < p) q = p;
    if (q < stop) {
      const char* nl = (const char*)memchr(q, '\n', (size_t)(stop - q));
      q = nl ? nl + 1 : stop;
    }
    ch[t].e = q;
    p = q;
  }
  parallel(threads, [&](int t) { count_chunk(ch[t]); });
  size_t nv = 0;
  for (auto& c : ch) {
    c.vbase = nv;
    nv += c.vertices;
  }
  std::vector<float> vx(3 * (nv ? nv : 1));
  parallel(threads, [&](int t) { parse_chunk(ch[t], vx.data()); });
  size_t nt = 0;
  std::vector<size_t> tbase(ch.size());
  for (size_t t = 0; t < ch.size(); ++t) {
    if (ch[t].bad) return BVH_ERR_INVALID_ARG;  // the reference throws (std::stoi)
    tbase[t] = nt;
    nt += ch[t].tri.size() / 3;
  }
  if (nt > 0xffffffffu) return BVH_ERR_INVALID_ARG;
  out->n = (uint32_t)nt;
  out->vertices = nv;
  out->pinned = pinned ? 1 : 0;
  for (int k = 0; k < 9; ++k) {
    void* mem = nullptr;
    const size_t bytes = (nt ? nt : 1) * sizeof(float);
    if (pinned) {
      if (cudaMallocHost(&mem, bytes) != cudaSuccess) mem = nullptr;
    } else {
      mem = malloc(bytes);
    }
    if (!mem) {
      bvh_obj_free(out);
      return BVH_ERR_OUT_OF_MEMORY;
    }
    out->v[k] = static_cast<float*>(mem);
  }
  // corners: v0x v0y v0z v1x v1y v1z v2x v2y v2z
  parallel(threads, [&](int t) {
    const Chunk& c = ch[(size_t)t];
    const size_t tb = tbase[(size_t)t], m = c.tri.size() / 3;
    for (size_t i = 0; i < m; ++i)
      for (int corner = 0; corner < 3; ++corner) {
        const float* v = vx.data() + 3 * (size_t)c.tri[3 * i + corner];
        out->v[3 * corner + 0][tb + i] = v[0];
        out->v[3 * corner + 1][tb + i] = v[1];
        out->v[3 * corner + 2][tb + i] = v[2];
      }
  });
  return BVH_OK;
}

extern "C" void bvh_obj_free(bvh_obj_mesh* m) {
  if (!m) return;
  for (int k = 0; k < 9; ++k) {
    if (!m->v[k]) continue;
    if (m->pinned) cudaFreeHost(m->v[k]);
    else free(m->v[k]);
    m->v[k] = nullptr;
  }
  m->n = 0;
}

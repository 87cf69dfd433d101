// Mesh and site files in the reference's formats (test_voronoi.cu:40-145),
// read into plain arrays with the numbers parsed on every host thread.
//
//   .tet  "<nv> vertices" line, "<nt> tets" line, then nv x y z and nt
//         "4 a b c d" (0-based);
//   .vtk  four header lines, "POINTS nv type", 3 nv coordinates, "CELLS nt
//         size", nt "4 a b c d" (1-based, stored 0-based);
//   .xyz  a count, then n x y z.
//
// The whole file is read once; its body is split at whitespace into one
// chunk per thread, each thread counts its tokens, a prefix sum gives every
// chunk the global index of its first token, and each thread parses its
// tokens straight into the output arrays (std::from_chars: the same correctly
// rounded floats as the reference's stream extraction).  A 100M-tet file is
// about 5 GB of text; the streams of the reference read it one token at a
// time on one thread.
#include <algorithm>
#include <atomic>
#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "voronoi_gb300.h"

namespace vgb {
void set_error(const char* fmt, ...);  // the library's last-error text (vgb_last_error)
}

namespace {

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

bool read_file(const char* path, std::string& text) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  bool ok = std::fseek(f, 0, SEEK_END) == 0;
  const long size = ok ? std::ftell(f) : -1;
  ok = ok && size >= 0 && std::fseek(f, 0, SEEK_SET) == 0;
  if (ok) {
    text.resize((size_t)size);
    ok = size == 0 || std::fread(&text[0], 1, (size_t)size, f) == (size_t)size;
  }
  std::fclose(f);
  return ok;
}

// Whitespace-separated tokens of [b, e), counted per chunk (one per thread).
struct Tokens {
  std::vector<const char*> cb, ce;  // chunk bounds (no token crosses one)
  std::vector<size_t> first;        // global index of each chunk's first token
  size_t total = 0;

  Tokens(const char* b, const char* e) {
    const size_t bytes = (size_t)(e - b);
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = std::max<size_t>(1, std::min<size_t>(std::min(hw, 64u), bytes >> 20));
    const char* p = b;
    for (size_t t = 0; t < nt; ++t) {
      const char* q = t + 1 == nt ? e : b + bytes / nt * (t + 1);
      if (q < p) q = p;
      while (q < e && !is_space(*q)) ++q;  // end the chunk at whitespace
      cb.push_back(p);
      ce.push_back(q);
      p = q;
    }
    std::vector<size_t> count(nt, 0);
    run([&](size_t t) {
      size_t c = 0;
      const char* s = cb[t];
      while (s < ce[t]) {
        while (s < ce[t] && is_space(*s)) ++s;
        if (s == ce[t]) break;
        ++c;
        while (s < ce[t] && !is_space(*s)) ++s;
      }
      count[t] = c;
    });
    first.resize(nt);
    for (size_t t = 0; t < nt; ++t) {
      first[t] = total;
      total += count[t];
    }
  }

  template <class F>
  void run(F&& fn) {
    const size_t nt = cb.size();
    if (nt == 1) {
      fn(0);
      return;
    }
    std::vector<std::thread> th;
    th.reserve(nt);
    for (size_t t = 0; t < nt; ++t) th.emplace_back([&, t] { fn(t); });
    for (auto& x : th) x.join();
  }

  // fn(global index, token begin, token end) for every token, chunk by chunk
  // on the threads; fn returns false to flag a malformed token
  template <class F>
  bool each(F&& fn) {
    std::atomic<bool> ok{true};
    run([&](size_t t) {
      size_t i = first[t];
      const char* s = cb[t];
      while (s < ce[t]) {
        while (s < ce[t] && is_space(*s)) ++s;
        if (s == ce[t]) break;
        const char* w = s;
        while (s < ce[t] && !is_space(*s)) ++s;
        if (!fn(i++, w, s)) ok.store(false, std::memory_order_relaxed);
      }
    });
    return ok.load();
  }

  // the token at global index i (sequential; for the few header tokens)
  bool at(size_t i, const char*& w, const char*& we) const {
    if (i >= total) return false;
    size_t t = std::upper_bound(first.begin(), first.end(), i) - first.begin() - 1;
    size_t k = first[t];
    const char* s = cb[t];
    while (s < ce[t]) {
      while (s < ce[t] && is_space(*s)) ++s;
      const char* b0 = s;
      while (s < ce[t] && !is_space(*s)) ++s;
      if (k++ == i) {
        w = b0;
        we = s;
        return true;
      }
    }
    return false;
  }
};

bool parse_float(const char* b, const char* e, float& v) {
  if (b < e && *b == '+') ++b;  // stream extraction takes a leading '+'
  const auto r = std::from_chars(b, e, v);
  return r.ec == std::errc() && r.ptr == e;
}
bool parse_int(const char* b, const char* e, long long& v) {
  if (b < e && *b == '+') ++b;
  const auto r = std::from_chars(b, e, v);
  return r.ec == std::errc() && r.ptr == e;
}
bool token_int(const Tokens& T, size_t i, long long& v) {
  const char *w, *we;
  return T.at(i, w, we) && parse_int(w, we, v);
}
bool token_is(const Tokens& T, size_t i, const char* word) {
  const char *w, *we;
  return T.at(i, w, we) && (size_t)(we - w) == std::strlen(word) && std::memcmp(w, word, (size_t)(we - w)) == 0;
}

// The next integer from p, then the rest of its line is skipped (the
// reference's `input >> n; getline(input, s)`); p moves past that line.
bool line_count(const char*& p, const char* e, long long& v) {
  const char* s = p;
  while (s < e && is_space(*s)) ++s;
  const char* w = s;
  while (s < e && !is_space(*s)) ++s;
  const bool ok = parse_int(w, s, v);
  while (s < e && *s != '\n') ++s;
  p = s < e ? s + 1 : s;
  return ok;
}

template <class T>
T* take(std::vector<T>& v) {
  T* p = static_cast<T*>(std::malloc(sizeof(T) * std::max<size_t>(v.size(), 1)));
  if (p && !v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}

}  // namespace

extern "C" {

int vgb_read_tet(const char* path, float** verts, int* n_vert, int** tets, int* n_tet) {
  if (!path || !verts || !n_vert || !tets || !n_tet) { vgb::set_error("NULL argument"); return VGB_ERR_INVALID; }
  std::string text;
  if (!read_file(path, text)) { vgb::set_error("%s: cannot read", path); return VGB_ERR_INVALID; }
  const char* p = text.data();
  const char* e = p + text.size();
  const std::string spath(path);
  const std::string ext = spath.substr(spath.find_last_of('.') + 1);
  long long nv = 0, nt = 0;
  size_t v0 = 0, t0 = 0;  // global token index of the first coordinate / cell
  int base = 0;           // the file's first vertex index
  const char* body = p;
  if (ext == "tet") {
    if (!line_count(body, e, nv) || !line_count(body, e, nt)) {
      vgb::set_error("%s: bad .tet header", path);
      return VGB_ERR_INVALID;
    }
    t0 = 3 * (size_t)nv;
  } else if (ext == "vtk") {
    for (int i = 0; i < 4 && body < e; ++i) {
      while (body < e && *body != '\n') ++body;
      if (body < e) ++body;
    }
  } else {
    vgb::set_error("%s: not a .tet or .vtk file", path);
    return VGB_ERR_INVALID;
  }
  Tokens T(body, e);
  if (ext == "vtk") {
    // POINTS nv type | coordinates | CELLS nt size | cells
    if (!token_is(T, 0, "POINTS") || !token_int(T, 1, nv) || nv < 0 ||
        !token_is(T, 3 + 3 * (size_t)nv, "CELLS") || !token_int(T, 4 + 3 * (size_t)nv, nt)) {
      vgb::set_error("%s: bad .vtk layout", path);
      return VGB_ERR_INVALID;
    }
    v0 = 3;
    t0 = 6 + 3 * (size_t)nv;
    base = 1;
  }
  if (nv <= 0 || nt <= 0 || nv > (1LL << 31) - 1 || nt > (1LL << 31) - 1 ||
      T.total < t0 + 5 * (size_t)nt || (ext == "tet" && T.total < 3 * (size_t)nv)) {
    vgb::set_error("%s: %lld vertices, %lld tets, %zu numbers", path, nv, nt, T.total);
    return VGB_ERR_INVALID;
  }
  std::vector<float> v(3 * (size_t)nv);
  std::vector<int> t(4 * (size_t)nt);
  const size_t v1 = v0 + 3 * (size_t)nv, t1 = t0 + 5 * (size_t)nt;
  const bool ok = T.each([&](size_t i, const char* w, const char* we) {
    if (i >= v0 && i < v1) return parse_float(w, we, v[i - v0]);
    if (i >= t0 && i < t1) {
      long long x = 0;
      if (!parse_int(w, we, x)) return false;
      const size_t k = i - t0;
      if (k % 5 == 0) return x == 4;  // tetrahedral cells only
      x -= base;
      if (x < 0 || x >= nv) return false;
      t[4 * (k / 5) + (k % 5) - 1] = (int)x;
    }
    return true;
  });
  if (!ok) {
    vgb::set_error("%s: malformed number, non-tetrahedral cell or vertex index out of range", path);
    return VGB_ERR_INVALID;
  }
  *verts = take(v);
  *tets = take(t);
  if (!*verts || !*tets) {
    std::free(*verts);
    std::free(*tets);
    *verts = nullptr;
    *tets = nullptr;
    vgb::set_error("host allocation failed");
    return VGB_ERR_NOMEM;
  }
  *n_vert = (int)nv;
  *n_tet = (int)nt;
  return VGB_OK;
}

int vgb_read_xyz(const char* path, float** xyz, int* n) {
  if (!path || !xyz || !n) { vgb::set_error("NULL argument"); return VGB_ERR_INVALID; }
  std::string text;
  if (!read_file(path, text)) { vgb::set_error("%s: cannot read", path); return VGB_ERR_INVALID; }
  Tokens T(text.data(), text.data() + text.size());
  long long m = 0;
  if (!token_int(T, 0, m) || m <= 0 || m > (1LL << 31) - 1 || T.total < 1 + 3 * (size_t)m) {
    vgb::set_error("%s: bad count or too few coordinates", path);
    return VGB_ERR_INVALID;
  }
  std::vector<float> s(3 * (size_t)m);
  const bool ok = T.each([&](size_t i, const char* w, const char* we) {
    if (i >= 1 && i < 1 + 3 * (size_t)m) return parse_float(w, we, s[i - 1]);
    return true;
  });
  if (!ok) {
    vgb::set_error("%s: malformed coordinate", path);
    return VGB_ERR_INVALID;
  }
  *xyz = take(s);
  if (!*xyz) { vgb::set_error("host allocation failed"); return VGB_ERR_NOMEM; }
  *n = (int)m;
  return VGB_OK;
}

void vgb_free_array(void* p) { std::free(p); }

}  // extern "C"

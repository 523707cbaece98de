// Scene I/O on the host: Wavefront OBJ meshes (v / f records) in and out,
// the reference's model-file lookup with a case-insensitive name match, and
// the reference's sphere scene built from a model file.
//
// The reference's loader (createScene_new, main.cpp:599-721) reads only `v`
// records, stops at the first other token and turns every vertex into a
// small sphere; its model names are lower case ("igea.obj") while one of its
// files is not ("Igea.obj"), so that model fails to open on case-sensitive
// file systems.  rq_obj_load reads full meshes; rq_reference_spheres keeps
// the reference's semantics for its sphere scenes; rq_model_path resolves the
// file name case-insensitively.
#include <dirent.h>
#include <strings.h>

#include <charconv>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "rq.h"

namespace {

bool read_file(const char* path, std::string& out) {
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  long size = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (size < 0) {
    std::fclose(f);
    return false;
  }
  out.resize((size_t)size);
  const size_t got = size ? std::fread(&out[0], 1, (size_t)size, f) : 0;
  std::fclose(f);
  return got == (size_t)size;
}

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r'; }

struct Cursor {
  const char* p;
  const char* end;  // end of the current line
  void skip_space() {
    while (p < end && is_space(*p)) ++p;
  }
  bool at_end() {
    skip_space();
    return p >= end;
  }
  bool read_float(float& v) {
    skip_space();
    if (p < end && *p == '+') ++p;  // from_chars takes no leading '+'
    auto r = std::from_chars(p, end, v);
    if (r.ec != std::errc()) return false;
    p = r.ptr;
    return true;
  }
  // One face corner: v, v/vt, v/vt/vn or v//vn; returns the vertex index.
  bool read_corner(long long& v) {
    skip_space();
    if (p < end && *p == '+') ++p;
    auto r = std::from_chars(p, end, v);
    if (r.ec != std::errc()) return false;
    p = r.ptr;
    while (p < end && !is_space(*p)) ++p;  // the /vt/vn parts are not used
    return true;
  }
};

template <typename T>
T* copy_out(const std::vector<T>& v) {
  T* p = static_cast<T*>(std::malloc(v.empty() ? 1 : v.size() * sizeof(T)));
  if (p && !v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
  return p;
}

}  // namespace

extern "C" {

void rq_free(void* p) { std::free(p); }

rq_status_t rq_obj_load(const char* path, float** verts, uint32_t* nv, uint32_t** idx, uint32_t* nt) {
  if (!path || !verts || !nv || !idx || !nt) return RQ_ERROR_INVALID_ARGUMENT;
  *verts = nullptr;
  *idx = nullptr;
  *nv = *nt = 0;
  std::string text;
  if (!read_file(path, text)) return RQ_ERROR_INVALID_ARGUMENT;
  std::vector<float> v;
  std::vector<uint32_t> f;
  std::vector<long long> corners;
  const char* p = text.data();
  const char* stop = p + text.size();
  while (p < stop) {
    const char* eol = static_cast<const char*>(std::memchr(p, '\n', (size_t)(stop - p)));
    if (!eol) eol = stop;
    Cursor c{p, eol};
    c.skip_space();
    if (c.p + 1 < eol && c.p[0] == 'v' && is_space(c.p[1])) {
      c.p += 1;
      float x, y, z;
      if (!c.read_float(x) || !c.read_float(y) || !c.read_float(z)) return RQ_ERROR_INVALID_ARGUMENT;
      if (v.size() / 3 >= 0xFFFFFFFFull) return RQ_ERROR_INVALID_ARGUMENT;
      v.push_back(x);
      v.push_back(y);
      v.push_back(z);
    } else if (c.p + 1 < eol && c.p[0] == 'f' && is_space(c.p[1])) {
      c.p += 1;
      corners.clear();
      while (!c.at_end()) {
        long long k;
        if (!c.read_corner(k)) return RQ_ERROR_INVALID_ARGUMENT;
        const long long count = (long long)(v.size() / 3);
        // 1-based, or negative = relative to the vertices read so far
        const long long abs_k = k > 0 ? k - 1 : count + k;
        if (k == 0 || abs_k < 0 || abs_k >= count) return RQ_ERROR_INVALID_ARGUMENT;
        corners.push_back(abs_k);
      }
      if (corners.size() < 3) return RQ_ERROR_INVALID_ARGUMENT;
      for (size_t j = 1; j + 1 < corners.size(); ++j) {  // fan around the first corner
        f.push_back((uint32_t)corners[0]);
        f.push_back((uint32_t)corners[j]);
        f.push_back((uint32_t)corners[j + 1]);
      }
      if (f.size() / 3 >= (1u << 30)) return RQ_ERROR_INVALID_ARGUMENT;
    }
    p = eol + 1;
  }
  *verts = copy_out(v);
  *idx = copy_out(f);
  if (!*verts || !*idx) {
    std::free(*verts);
    std::free(*idx);
    *verts = nullptr;
    *idx = nullptr;
    return RQ_ERROR_OUT_OF_MEMORY;
  }
  *nv = (uint32_t)(v.size() / 3);
  *nt = (uint32_t)(f.size() / 3);
  return RQ_SUCCESS;
}

rq_status_t rq_obj_save(const char* path, const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt) {
  if (!path || (nv && !verts) || (nt && !idx)) return RQ_ERROR_INVALID_ARGUMENT;
  for (size_t i = 0; i < (size_t)nt * 3; ++i)
    if (idx[i] >= nv) return RQ_ERROR_INVALID_ARGUMENT;
  std::FILE* out = std::fopen(path, "wb");
  if (!out) return RQ_ERROR_INVALID_ARGUMENT;
  char buf[96];
  bool ok = true;
  for (size_t i = 0; i < nv && ok; ++i) {
    // shortest text that reads back to the same float
    char* q = buf;
    *q++ = 'v';
    for (int k = 0; k < 3; ++k) {
      *q++ = ' ';
      auto r = std::to_chars(q, buf + sizeof(buf) - 2, verts[3 * i + k]);
      q = r.ptr;
    }
    *q++ = '\n';
    ok = std::fwrite(buf, 1, (size_t)(q - buf), out) == (size_t)(q - buf);
  }
  for (size_t i = 0; i < nt && ok; ++i)
    ok = std::fprintf(out, "f %u %u %u\n", idx[3 * i] + 1, idx[3 * i + 1] + 1, idx[3 * i + 2] + 1) > 0;
  ok = (std::fclose(out) == 0) && ok;
  return ok ? RQ_SUCCESS : RQ_ERROR_INVALID_ARGUMENT;
}

rq_status_t rq_model_path(const char* dir, int32_t scene_model, char* out, uint32_t cap) {
  if (!dir || !out || cap == 0) return RQ_ERROR_INVALID_ARGUMENT;
  // the file names of createScene_new's switch (main.cpp:605-643)
  const char* name;
  switch (scene_model) {
    case RQ_IGEA: name = "igea.obj"; break;
    case RQ_ARMADILLO: name = "armadillo.obj"; break;
    case RQ_BUNNIES: name = "bunnies.obj"; break;
    case RQ_CITY: name = "city.obj"; break;
    case RQ_GRASS: name = "grass.obj"; break;
    case RQ_BUNNY: name = "bunny.obj"; break;
    case RQ_BUDDHA: name = "buddha.obj"; break;
    default: name = "test.obj"; break;
  }
  std::string found;
  if (DIR* d = opendir(dir)) {
    while (dirent* e = readdir(d)) {
      if (strcasecmp(e->d_name, name) == 0) {
        found = e->d_name;
        if (std::strcmp(e->d_name, name) == 0) break;  // an exact match wins
      }
    }
    closedir(d);
  }
  if (found.empty()) return RQ_ERROR_INVALID_ARGUMENT;
  std::string path = std::string(dir) + "/" + found;
  if (path.size() + 1 > cap) return RQ_ERROR_INVALID_ARGUMENT;
  std::memcpy(out, path.c_str(), path.size() + 1);
  return RQ_SUCCESS;
}

rq_status_t rq_reference_spheres(const char* path, int32_t clones, float** spheres, uint32_t* n) {
  if (!path || !spheres || !n || clones < 1) return RQ_ERROR_INVALID_ARGUMENT;
  *spheres = nullptr;
  *n = 0;
  std::vector<float> s;
  for (int clone = 0; clone < clones; ++clone) {
    const float shift = clone * 20.f;
    std::ifstream file(path);
    if (!file.good()) return RQ_ERROR_INVALID_ARGUMENT;
    std::string tok;
    // every `v x y z` up to the first other token (main.cpp:657-698)
    while (file >> tok && tok == "v") {
      float x, y, z;
      if (!(file >> x >> y >> z)) return RQ_ERROR_INVALID_ARGUMENT;
      float cx = x * 100 + shift, cy = y * 100 + shift, cz = z * 100 + shift;
      cy += -10;
      cz += -60;
      s.insert(s.end(), {cx, cy, cz, (float)(0.01 * 5)});  // radius: a double product stored to float
    }
  }
  // the ground sphere (main.cpp:701-703)
  s.insert(s.end(), {0.93591022f, -105.47120094f, -43.2363205f, 100.f});
  *spheres = copy_out(s);
  if (!*spheres) return RQ_ERROR_OUT_OF_MEMORY;
  *n = (uint32_t)(s.size() / 4);
  return RQ_SUCCESS;
}

}  // extern "C"

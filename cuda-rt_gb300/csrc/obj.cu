// obj.cu -- host-side scene input and image output for the drop-in CLI:
// a Wavefront OBJ/MTL reader with the conventions of the reference's loader
// (Scene_h::LoadObj, src/scene.cpp:6-58, over its vendored tinyobjloader)
// and the reference's 24-bit BMP writer (writeBMP, src/bitmap.cpp:99-154).
// Host code only; no CUDA calls.
//
// OBJ: "v x y z", "vn x y z", "f" with v, v/t, v//n or v/t/n corners
// (1-based or negative indices), polygons fan-triangulated (0, k, k+1),
// "mtllib" (read from mtl_dir, or the OBJ's directory), "usemtl" (unknown
// or absent names give material 0).  Coordinates are rounded to FP32, the
// precision of crt_mesh_desc.  MTL: newmtl, Ka, Kd, Ks, Kt/Tf, Ke, Ns, Ni
// (tinyobjloader's defaults: colours 0, shininess 1, ior 1).  A missing MTL file
// is skipped, as tinyobjloader warns and goes on; a mesh without materials
// gets one Lambert material (kd 0.8).  Every face corner must name a normal:
// the reference reads normals[-1] otherwise, so such files are rejected.
//
// The OBJ is read in chunks of whole lines on all host cores, in two passes:
// the first counts each chunk's lines, vertices, normals and triangles and
// lists its mtllib/usemtl lines; a serial step reads the MTL files and
// resolves every usemtl in file order and gives each chunk its starting
// offsets; the second parses each chunk into its place in the output arrays
// (a relative index counts back from the vertices before its line, as in a
// serial read).  The result does not depend on the chunking; the first error
// in file order is the one reported.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "crt.h"

namespace crt {
void set_last_error(const char* msg);
}

struct crt_obj {
  std::vector<float> v, n;
  std::vector<int32_t> vi, ni, mid;
  std::vector<crt_material> mats;
  std::vector<double> ior;  // per material: MTL Ni
};

namespace {

crt_status fail(const std::string& m) {
  crt::set_last_error(m.c_str());
  return CRT_INVALID_ARG;
}

bool parse_double(const std::string& s, double& out) {
  const char* b = s.c_str();
  char* e = nullptr;
  errno = 0;
  out = std::strtod(b, &e);
  return e != b && *e == '\0';
}

bool parse3(const std::vector<std::string>& t, double out[3]) {
  if (t.size() < 4) return false;
  for (int k = 0; k < 3; k++)
    if (!parse_double(t[1 + k], out[k])) return false;
  return true;
}

std::vector<std::string> split_ws(const std::string& line) {
  std::vector<std::string> t;
  std::istringstream is(line);
  std::string w;
  while (is >> w) t.push_back(w);
  return t;
}

std::string dir_of(const std::string& path) {
  const size_t k = path.find_last_of('/');
  return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

void read_mtl(const std::string& file, std::map<std::string, int>& names, std::vector<crt_material>& mats,
              std::vector<double>& ior) {
  std::ifstream f(file);
  if (!f) return;  // tinyobjloader warns and goes on
  std::string line;
  crt_material* m = nullptr;
  while (std::getline(f, line)) {
    const std::vector<std::string> t = split_ws(line);
    if (t.empty()) continue;
    if (t[0] == "newmtl" && t.size() >= 2) {
      crt_material z;
      std::memset(&z, 0, sizeof(z));
      z.shininess = 1.0;
      names[t[1]] = (int)mats.size();
      mats.push_back(z);
      ior.push_back(1.0);
      m = &mats.back();
      continue;
    }
    if (!m) continue;
    double x[3];
    double* dst = nullptr;
    if (t[0] == "Ka") dst = m->ka;
    else if (t[0] == "Kd") dst = m->kd;
    else if (t[0] == "Ks") dst = m->ks;
    else if (t[0] == "Kt" || t[0] == "Tf") dst = m->kt;
    else if (t[0] == "Ke") dst = m->ke;
    if (dst && parse3(t, x)) {
      for (int k = 0; k < 3; k++) dst[k] = x[k];
    } else if (t[0] == "Ns" && t.size() >= 2) {
      double s;
      if (parse_double(t[1], s)) m->shininess = s;
    } else if (t[0] == "Ni" && t.size() >= 2) {
      double s;
      if (parse_double(t[1], s)) ior.back() = s;
    }
  }
}

// A line of the OBJ as whitespace-separated tokens [b, e) of the file
// buffer: no allocation per line (a 200,000-face file has a million lines).
struct Tok {
  const char* b;
  const char* e;
  bool is(const char* w) const {
    const size_t n = std::strlen(w);
    return (size_t)(e - b) == n && std::memcmp(b, w, n) == 0;
  }
  std::string str() const { return std::string(b, e); }
};
inline bool space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// A number that fills the token: strtod stops at the first character that is
// not part of it, which must be the token's end.
bool tok_double(const Tok& t, double& out) {
  char* e = nullptr;
  errno = 0;
  out = std::strtod(t.b, &e);
  return e != t.b && e == t.e;
}

// One face corner: "v", "v/t", "v//n" or "v/t/n"; indices resolved to
// 0-based (negative ones count back from the current end); ni = -1 when the
// corner names no normal.
bool tok_corner(const Tok& t, size_t nv, size_t nn, int& vi, int& ni) {
  const char* s1 = static_cast<const char*>(std::memchr(t.b, '/', t.e - t.b));
  const char* ve = s1 ? s1 : t.e;
  if (ve == t.b) return false;
  char* e = nullptr;
  const long v = std::strtol(t.b, &e, 10);
  if (e != ve || v == 0 || v > INT32_MAX || v < -(long)INT32_MAX) return false;
  vi = v > 0 ? (int)(v - 1) : (int)((long)nv + v);
  ni = -1;
  if (s1) {
    const char* s2 = static_cast<const char*>(std::memchr(s1 + 1, '/', t.e - (s1 + 1)));
    if (s2 && s2 + 1 < t.e) {
      const long n = std::strtol(s2 + 1, &e, 10);
      if (e != t.e || n == 0 || n > INT32_MAX || n < -(long)INT32_MAX) return false;
      ni = n > 0 ? (int)(n - 1) : (int)((long)nn + n);
    }
  }
  return true;
}

// Whole file into buf (NUL-terminated, so strtod never reads past it).
bool read_file(const char* path, std::string& buf) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  bool ok = std::fseek(f, 0, SEEK_END) == 0;
  const long size = ok ? std::ftell(f) : -1;
  ok = ok && size >= 0 && std::fseek(f, 0, SEEK_SET) == 0;
  if (ok) {
    buf.resize((size_t)size);
    ok = size == 0 || std::fread(&buf[0], 1, (size_t)size, f) == (size_t)size;
  }
  std::fclose(f);
  return ok;
}

// Whitespace-separated tokens of the line [q, le).
void tokenize(const char* q, const char* le, std::vector<Tok>& t) {
  t.clear();
  while (q < le) {
    while (q < le && space(*q)) q++;
    const char* tb = q;
    while (q < le && !space(*q)) q++;
    if (q > tb) t.push_back(Tok{tb, q});
  }
}

// A run of whole lines [b, e), its counts (first pass), its offsets in the
// file and the output arrays (serial step) and its first error (second pass).
struct Chunk {
  struct Event {  // an mtllib or usemtl line
    bool lib, has_name;
    std::string name;
  };
  const char* b;
  const char* e;
  int64_t lines = 0, nv = 0, nn = 0, ntri = 0;
  std::vector<Event> events;
  int64_t line0 = 0, v0 = 0, n0 = 0, t0 = 0;
  int mat0 = -1;
  std::vector<int> usemtl;  // the material each of its usemtl lines selects
  std::string err;
};

// Chunks of about CRT_OBJ_CHUNK_BYTES (environment; default 256 KiB), each
// ending just after a newline (the last at the end of the file).
std::vector<Chunk> split_chunks(const std::string& buf) {
  size_t want = (size_t)1 << 18;
  if (const char* ev = std::getenv("CRT_OBJ_CHUNK_BYTES")) {
    const long x = std::strtol(ev, nullptr, 10);
    if (x > 0) want = (size_t)x;
  }
  std::vector<Chunk> out;
  const char* p = buf.c_str();
  const char* const end = p + buf.size();
  while (p < end) {
    const char* q = (size_t)(end - p) > want ? p + want : end;
    if (q < end) {
      const char* nl = static_cast<const char*>(std::memchr(q - 1, '\n', end - (q - 1)));
      q = nl ? nl + 1 : end;
    }
    Chunk c;
    c.b = p, c.e = q;
    out.push_back(std::move(c));
    p = q;
  }
  return out;
}

// f(i) for i in [0, n) on nth threads (this one included).
template <typename F>
void parallel_for(size_t n, size_t nth, F f) {
  std::atomic<size_t> next(0);
  auto work = [&]() {
    for (size_t i; (i = next.fetch_add(1)) < n;) f(i);
  };
  std::vector<std::thread> pool;
  for (size_t k = 1; k < nth; k++) pool.emplace_back(work);
  work();
  for (std::thread& th : pool) th.join();
}

// First pass: counts and mtllib/usemtl lines.
void count_chunk(Chunk& c) {
  std::vector<Tok> t;
  for (const char* p = c.b; p < c.e;) {
    const char* le = static_cast<const char*>(std::memchr(p, '\n', c.e - p));
    if (!le) le = c.e;
    c.lines++;
    tokenize(p, le, t);
    p = le + 1;
    if (t.empty() || *t[0].b == '#') continue;
    if (t[0].is("v")) c.nv++;
    else if (t[0].is("vn")) c.nn++;
    else if (t[0].is("f")) c.ntri += t.size() >= 4 ? (int64_t)t.size() - 3 : 0;
    else if (t[0].is("mtllib") && t.size() >= 2) c.events.push_back(Chunk::Event{true, true, t[1].str()});
    else if (t[0].is("usemtl")) c.events.push_back(Chunk::Event{false, t.size() >= 2, t.size() >= 2 ? t[1].str() : ""});
  }
}

// Second pass: the chunk's vertices, normals and triangles into their places.
void parse_chunk(Chunk& c, crt_obj& o) {
  std::vector<Tok> t;
  std::vector<int> cv, cn;
  int64_t line = c.line0, lv = c.v0, ln = c.n0, lt = c.t0;
  int cur = c.mat0;
  size_t ue = 0;
  for (const char* p = c.b; p < c.e;) {
    const char* le = static_cast<const char*>(std::memchr(p, '\n', c.e - p));
    if (!le) le = c.e;
    line++;
    tokenize(p, le, t);
    p = le + 1;
    if (t.empty() || *t[0].b == '#') continue;
    if (t[0].is("v") || t[0].is("vn")) {
      double x[3];
      bool ok = t.size() >= 4;
      for (int k = 0; ok && k < 3; k++) ok = tok_double(t[1 + k], x[k]);
      if (!ok) {
        c.err = "bad vertex at line " + std::to_string(line);
        return;
      }
      float* dst = t[0].is("v") ? &o.v[3 * (size_t)lv++] : &o.n[3 * (size_t)ln++];
      for (int k = 0; k < 3; k++) dst[k] = (float)x[k];
    } else if (t[0].is("usemtl")) {
      cur = c.usemtl[ue++];
    } else if (t[0].is("f")) {
      cv.clear();
      cn.clear();
      for (size_t k = 1; k < t.size(); k++) {
        int vi, ni;
        if (!tok_corner(t[k], (size_t)lv, (size_t)ln, vi, ni)) {
          c.err = "bad face corner at line " + std::to_string(line);
          return;
        }
        if (ni < 0) {
          c.err = "face without a normal index at line " + std::to_string(line) + " (vn normals are required)";
          return;
        }
        cv.push_back(vi);
        cn.push_back(ni);
      }
      for (size_t k = 1; k + 1 < cv.size(); k++, lt++) {
        const size_t c3[3] = {0, k, k + 1};
        for (int j = 0; j < 3; j++) o.vi[3 * (size_t)lt + j] = cv[c3[j]], o.ni[3 * (size_t)lt + j] = cn[c3[j]];
        o.mid[(size_t)lt] = cur;
      }
    }
  }
}

}  // namespace

extern "C" {

crt_status crt_obj_load(const char* obj_path, const char* mtl_dir, crt_obj** out) {
  if (!obj_path || !out) return fail("null argument");
  *out = nullptr;
  std::string buf;
  if (!read_file(obj_path, buf)) return fail(std::string("cannot open ") + obj_path);
  const std::string base = mtl_dir ? std::string(mtl_dir) : dir_of(obj_path);
  std::vector<Chunk> chunks = split_chunks(buf);
  const size_t nth = std::min<size_t>(chunks.size(), std::max(1u, std::thread::hardware_concurrency()));
  parallel_for(chunks.size(), nth, [&](size_t c) { count_chunk(chunks[c]); });

  // serial: MTL files and usemtl in file order, each chunk's offsets
  crt_obj* o = new crt_obj;
  std::map<std::string, int> names;
  int cur = -1;
  int64_t L = 0, V = 0, N = 0, T = 0;
  for (Chunk& c : chunks) {
    c.line0 = L, c.v0 = V, c.n0 = N, c.t0 = T, c.mat0 = cur;
    for (const Chunk::Event& ev : c.events) {
      if (ev.lib) {
        std::string mp = base;
        if (!mp.empty() && mp.back() != '/') mp += '/';
        read_mtl(mp + ev.name, names, o->mats, o->ior);
      } else {
        const auto it = ev.has_name ? names.find(ev.name) : names.end();
        cur = it == names.end() ? -1 : it->second;
        c.usemtl.push_back(cur);
      }
    }
    L += c.lines, V += c.nv, N += c.nn, T += c.ntri;
  }
  if (V > CRT_MAX_VERTICES || N > CRT_MAX_VERTICES || T > CRT_MAX_TRIANGLES) {
    delete o;
    return fail("more than CRT_MAX_VERTICES vertices or normals, or CRT_MAX_TRIANGLES triangles");
  }
  o->v.resize(3 * (size_t)V);
  o->n.resize(3 * (size_t)N);
  o->vi.resize(3 * (size_t)T);
  o->ni.resize(3 * (size_t)T);
  o->mid.resize((size_t)T);
  parallel_for(chunks.size(), nth, [&](size_t c) { parse_chunk(chunks[c], *o); });
  for (const Chunk& c : chunks)
    if (!c.err.empty()) {
      delete o;
      return fail(c.err);
    }

  if (o->mats.empty()) {
    crt_material z;
    std::memset(&z, 0, sizeof(z));
    z.kd[0] = z.kd[1] = z.kd[2] = 0.8;
    o->mats.push_back(z);
    o->ior.push_back(1.0);
  }
  for (int32_t& m : o->mid)
    if (m < 0) m = 0;
  for (size_t k = 0; k < o->vi.size(); k++)
    if (o->vi[k] < 0 || o->vi[k] >= V || o->ni[k] < 0 || o->ni[k] >= N) {
      delete o;
      return fail("face index out of range");
    }
  *out = o;
  return CRT_OK;
}

crt_status crt_obj_mesh(const crt_obj* o, crt_mesh_desc* mesh) {
  if (!o || !mesh) return fail("null argument");
  mesh->vertices = o->v.data();
  mesh->num_vertices = (int32_t)(o->v.size() / 3);
  mesh->normals = o->n.data();
  mesh->num_normals = (int32_t)(o->n.size() / 3);
  mesh->vertex_indices = o->vi.data();
  mesh->normal_indices = o->ni.data();
  mesh->num_triangles = (int32_t)o->mid.size();
  mesh->materials = o->mats.data();
  mesh->num_materials = (int32_t)o->mats.size();
  mesh->material_ids = o->mid.data();
  return CRT_OK;
}

crt_status crt_obj_optics(const crt_obj* o, crt_optics* optics) {
  if (!o || !optics) return fail("null argument");
  for (size_t m = 0; m < o->mats.size(); m++) {
    for (int k = 0; k < 3; k++) optics[m].kr[k] = o->mats[m].ks[k];  // mat.kr = specular, src/scene.cpp:29
    optics[m].ior = o->ior[m];
  }
  return CRT_OK;
}

crt_status crt_obj_free(crt_obj* o) {
  delete o;
  return CRT_OK;
}

crt_status crt_write_bmp(const char* path, int32_t width, int32_t height, const uint8_t* rgb8) {
  if (!path || !rgb8 || width <= 0 || height <= 0) return fail("bad arguments");
  const int row = width * 3, pad = (row % 4) ? 4 - row % 4 : 0;
  const uint32_t image = (uint32_t)(row + pad) * (uint32_t)height;
  uint8_t h[54];
  std::memset(h, 0, sizeof(h));
  auto u16 = [&](int at, uint32_t v) { h[at] = v & 0xff, h[at + 1] = (v >> 8) & 0xff; };
  auto u32 = [&](int at, uint32_t v) {
    for (int k = 0; k < 4; k++) h[at + k] = (v >> (8 * k)) & 0xff;
  };
  u16(0, 0x4d42);       // "BM"
  u32(2, 54 + image);   // file size
  u32(10, 54);          // pixel data offset
  u32(14, 40);          // info header size
  u32(18, (uint32_t)width);
  u32(22, (uint32_t)height);
  u16(26, 1);           // planes
  u16(28, 24);          // bits per pixel
  u32(38, (uint32_t)(100 / 2.54 * 72));  // pixels per metre, x and y
  u32(42, (uint32_t)(100 / 2.54 * 72));
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(std::string("cannot write ") + path);
  bool ok = std::fwrite(h, 1, sizeof(h), f) == sizeof(h);
  std::vector<uint8_t> line(row + pad, 0);
  for (int j = 0; j < height && ok; j++) {  // rows bottom-up, as the image buffer
    const uint8_t* src = rgb8 + (size_t)j * row;
    for (int i = 0; i < width; i++) {
      line[3 * i] = src[3 * i + 2];
      line[3 * i + 1] = src[3 * i + 1];
      line[3 * i + 2] = src[3 * i];
    }
    ok = std::fwrite(line.data(), 1, line.size(), f) == line.size();
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? CRT_OK : fail(std::string("write failed: ") + path);
}

}  // extern "C"

// capi.cu -- the C ABI (include/crt.h): scene ownership, argument checks,
// host/device staging and error reporting around the kernels of build.cu and
// trace.cu.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "crt.h"
#include "crt_internal.h"

using namespace crt;

struct crt_scene {
  MeshBufs m;
  BuildBufs b;
  bool built = false;
  // borrowing scene (crt_scene_create_borrowed): m's arrays are the caller's,
  // except a material-id array of zeros allocated when none was given
  bool borrowed = false;
  int* own_matid = nullptr;
  unsigned* counter = nullptr;
  void* block = nullptr;  // one allocation backing the build arrays
  size_t block_bytes = 0;
};

namespace {

thread_local std::string g_err;

crt_status fail(crt_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

crt_status cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();
  return fail(e == cudaErrorMemoryAllocation ? CRT_OOM : CRT_CUDA_ERROR,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define CRT_CUDA(call, what)                     \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

DScene dscene(const crt_scene* s) {
  DScene d;
  d.ntri = s->m.ntri;
  d.root = s->m.ntri >= 2 ? 0 : ~0;
  d.verts = s->m.verts;
  d.normals = s->m.normals;
  d.vidx = s->m.vidx;
  d.nidx = s->m.nidx;
  d.matid = s->m.matid;
  d.mats = s->m.mats;
  d.wnodes = s->b.wnodes;
  d.leaves = s->b.leaves;
  d.g = s->b.g;
  return d;
}

// A device view of a caller buffer: the buffer itself when it is device
// memory, else a stream-ordered temporary that is copied in and/or out.
struct DevView {
  void* user = nullptr;
  void* dev = nullptr;
  size_t bytes = 0;
  bool temp = false;
  cudaError_t open(void* p, size_t n, bool copy_in, cudaStream_t st) {
    user = p;
    bytes = n;
    if (!p || n == 0) return cudaSuccess;
    if (is_device_ptr(p)) {
      dev = p;
      return cudaSuccess;
    }
    temp = true;
    cudaError_t e = cudaMallocAsync(&dev, n, st);
    if (e != cudaSuccess) return e;
    if (copy_in) return cudaMemcpyAsync(dev, p, n, cudaMemcpyDefault, st);
    return cudaSuccess;
  }
  cudaError_t close(bool copy_out, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    if (temp) {
      if (copy_out) e = cudaMemcpyAsync(user, dev, bytes, cudaMemcpyDefault, st);
      cudaError_t e2 = cudaFreeAsync(dev, st);
      if (e == cudaSuccess) e = e2;
      temp = false;
    }
    return e;
  }
};

crt_status check_globals(crt_scene* s, cudaStream_t st) {
  CRT_CUDA(cudaStreamSynchronize(st), "synchronize");
  if (!s->b.g) return CRT_OK;
  int err = 0;
  CRT_CUDA(cudaMemcpy(&err, &s->b.g->err, sizeof(int), cudaMemcpyDeviceToHost), "read error flags");
  if (err & kErrTimeout) return fail(CRT_TIMEOUT, "a radix-sort look-back wait timed out");
  if (err & kErrStack) return fail(CRT_STACK_OVERFLOW, "a traversal exceeded the 64-entry stack");
  if (err & kErrIndex) return fail(CRT_INVALID_ARG, "a vertex, normal or material index is out of range");
  if (err & kErrNonFinite) return fail(CRT_INVALID_ARG, "non-finite (or |x| > 1e37) vertex coordinate");
  return CRT_OK;
}

void free_scene(crt_scene* s) {
  if (!s->borrowed) {
    cudaFree(s->m.verts);
    cudaFree(s->m.normals);
    cudaFree(s->m.vidx);
    cudaFree(s->m.nidx);
    cudaFree(s->m.matid);
    cudaFree(s->m.mats);
  }
  cudaFree(s->own_matid);
  cudaFree(s->block);
  cudaFree(s->counter);
}

}  // namespace

namespace crt {
// Lets entry points in other translation units record their error message.
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace crt

extern "C" {

const char* crt_last_error_string(void) { return g_err.c_str(); }
const char* crt_version(void) { return "cuda-rt-gb300 0.1 (sm_103a)"; }

// crt_scene_create and crt_scene_create_borrowed: checks, device arrays
// (copies, or the caller's own when borrowing), build arrays, index checks of
// device-resident indices, then the build.
static crt_status create_scene(const crt_mesh_desc* d, void* stream, bool borrow, crt_scene** out) {
  if (!d || !out) return fail(CRT_INVALID_ARG, "null argument");
  *out = nullptr;
  const int n = d->num_triangles;
  if (n < 0 || n > CRT_MAX_TRIANGLES) return fail(CRT_INVALID_ARG, "num_triangles out of range");
  if (d->num_vertices < 0 || d->num_normals < 0) return fail(CRT_INVALID_ARG, "negative array size");
  if (d->num_vertices > CRT_MAX_VERTICES || d->num_normals > CRT_MAX_VERTICES)
    return fail(CRT_INVALID_ARG, "more than CRT_MAX_VERTICES vertices or normals");
  if (n > 0 && (!d->vertices || !d->vertex_indices || d->num_vertices <= 0))
    return fail(CRT_INVALID_ARG, "triangles need vertices and vertex_indices");
  if (n > 0 && (!d->normals || d->num_normals <= 0)) return fail(CRT_INVALID_ARG, "normals are required");
  if (!d->materials || d->num_materials <= 0) return fail(CRT_INVALID_ARG, "at least one material is required");
  if (borrow) {
    const void* arrays[6] = {d->vertices, d->normals, d->vertex_indices, d->normal_indices, d->materials,
                             d->material_ids};
    for (const void* p : arrays)
      if (p && !is_device_ptr(p)) return fail(CRT_INVALID_ARG, "a borrowing scene takes device pointers only");
  }
  // Index checks when the indices are host memory (device ones: k_check_indices).
  if (n > 0 && !is_device_ptr(d->vertex_indices)) {
    for (int64_t i = 0; i < 3 * (int64_t)n; i++)
      if (d->vertex_indices[i] < 0 || d->vertex_indices[i] >= d->num_vertices)
        return fail(CRT_INVALID_ARG, "vertex index out of range");
    const int32_t* ni = d->normal_indices ? d->normal_indices : d->vertex_indices;
    if (!is_device_ptr(ni))
      for (int64_t i = 0; i < 3 * (int64_t)n; i++)
        if (ni[i] < 0 || ni[i] >= d->num_normals) return fail(CRT_INVALID_ARG, "normal index out of range");
    if (d->material_ids && !is_device_ptr(d->material_ids))
      for (int i = 0; i < n; i++)
        if (d->material_ids[i] < 0 || d->material_ids[i] >= d->num_materials)
          return fail(CRT_INVALID_ARG, "material id out of range");
  }
  cudaStream_t st = S(stream);
  crt_scene* s = new crt_scene;
  MeshBufs& m = s->m;
  m.nv = d->num_vertices;
  m.nn = d->num_normals;
  m.ntri = n;
  m.nmat = d->num_materials;
  auto bail = [&](cudaError_t e, const char* what) {
    crt_status r = cuda_fail(e, what);
    free_scene(s);
    delete s;
    return r;
  };
  cudaError_t e;
#define ALLOC(ptr, bytes)                                                 \
  if ((bytes) > 0 && (e = cudaMalloc(&(ptr), (bytes))) != cudaSuccess) \
    return bail(e, "cudaMalloc");
  s->borrowed = borrow;
  if (borrow) {
    m.verts = const_cast<float*>(d->vertices);
    m.normals = const_cast<float*>(d->normals);
    m.vidx = const_cast<int*>(d->vertex_indices);
    m.nidx = const_cast<int*>(d->normal_indices ? d->normal_indices : d->vertex_indices);
    m.mats = reinterpret_cast<DMat*>(const_cast<crt_material*>(d->materials));
    if (d->material_ids) {
      m.matid = const_cast<int*>(d->material_ids);
    } else {
      ALLOC(s->own_matid, sizeof(int) * (size_t)(n > 0 ? n : 1));
      m.matid = s->own_matid;
    }
  } else {
    ALLOC(m.verts, sizeof(float) * 3 * (size_t)m.nv);
    ALLOC(m.normals, sizeof(float) * 3 * (size_t)m.nn);
    ALLOC(m.vidx, sizeof(int) * 3 * (size_t)n);
    ALLOC(m.nidx, sizeof(int) * 3 * (size_t)n);
    ALLOC(m.matid, sizeof(int) * (size_t)n);
    ALLOC(m.mats, sizeof(DMat) * (size_t)m.nmat);
  }
  ALLOC(s->counter, sizeof(unsigned) * kMaxTileRegions);
  // build arrays, one block
  BuildBufs& b = s->b;
  b.n = n;
  const int tiles = sort_tiles(n > 0 ? n : 1);
  const size_t nn = n > 0 ? 2 * (size_t)n - 1 : 0;
  const size_t n1 = n > 0 ? (size_t)n : 1;
  size_t off[13], total = 0;
  const size_t sizes[13] = {4 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n, 4 * (size_t)n, 4 * 3 * (size_t)kRadix,
                            4 * 3 * (size_t)tiles * kRadix, 4 * nn, sizeof(uint4) * n1,
                            sizeof(float) * 6 * n1, sizeof(float) * 6 * n1, sizeof(int) * 6 * span_groups(n),
                            sizeof(LeafTri) * n1, sizeof(WNode) * n1};
  for (int i = 0; i < 13; i++) off[i] = total, total += align256(sizes[i]);
  const size_t goff = total;
  total += align256(sizeof(SceneGlobals));
  ALLOC(s->block, total);
  s->block_bytes = total;
#undef ALLOC
  char* base = static_cast<char*>(s->block);
  b.keys_a = reinterpret_cast<uint32_t*>(base + off[0]);
  b.keys_b = reinterpret_cast<uint32_t*>(base + off[1]);
  b.vals_a = reinterpret_cast<uint32_t*>(base + off[2]);
  b.vals_b = reinterpret_cast<uint32_t*>(base + off[3]);
  b.hist = reinterpret_cast<uint32_t*>(base + off[4]);
  b.status = reinterpret_cast<uint32_t*>(base + off[5]);
  b.parent = reinterpret_cast<uint32_t*>(base + off[6]);
  b.spans = reinterpret_cast<uint4*>(base + off[7]);
  b.suf = reinterpret_cast<float*>(base + off[8]);
  b.pre = reinterpret_cast<float*>(base + off[9]);
  b.gbox = reinterpret_cast<int*>(base + off[10]);
  b.leaves = reinterpret_cast<LeafTri*>(base + off[11]);
  b.wnodes = reinterpret_cast<WNode*>(base + off[12]);
  b.g = reinterpret_cast<SceneGlobals*>(base + goff);
  if ((e = cudaMemsetAsync(b.g, 0, sizeof(SceneGlobals), st)) != cudaSuccess) return bail(e, "memset");
  // upload
  auto up = [&](void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, st) : cudaSuccess;
  };
  static_assert(sizeof(DMat) == sizeof(crt_material), "material layout");
  if (!borrow) {
    if ((e = up(m.verts, d->vertices, sizeof(float) * 3 * (size_t)m.nv)) != cudaSuccess) return bail(e, "upload");
    if ((e = up(m.normals, d->normals, sizeof(float) * 3 * (size_t)m.nn)) != cudaSuccess) return bail(e, "upload");
    if ((e = up(m.vidx, d->vertex_indices, sizeof(int) * 3 * (size_t)n)) != cudaSuccess) return bail(e, "upload");
    if ((e = up(m.nidx, d->normal_indices ? d->normal_indices : d->vertex_indices, sizeof(int) * 3 * (size_t)n)) !=
        cudaSuccess)
      return bail(e, "upload");
    if (d->material_ids && (e = up(m.matid, d->material_ids, sizeof(int) * (size_t)n)) != cudaSuccess)
      return bail(e, "upload");
    if ((e = up(m.mats, d->materials, sizeof(DMat) * (size_t)m.nmat)) != cudaSuccess) return bail(e, "upload");
  }
  if (!d->material_ids && n > 0 && (e = cudaMemsetAsync(m.matid, 0, sizeof(int) * (size_t)n, st)) != cudaSuccess)
    return bail(e, "memset");
  // device-resident indices are checked on the device before the build reads them
  const bool dev_idx = n > 0 && (is_device_ptr(d->vertex_indices) || (d->normal_indices && is_device_ptr(d->normal_indices)) ||
                                 (d->material_ids && is_device_ptr(d->material_ids)));
  if (dev_idx) {
    if ((e = launch_check_indices(m, b, st)) != cudaSuccess) return bail(e, "index check launch");
    crt_status r = check_globals(s, st);
    if (r != CRT_OK) {
      std::string msg = g_err;
      free_scene(s);
      delete s;
      return fail(r, msg);
    }
  }
  if ((e = launch_build(m, b, st)) != cudaSuccess) return bail(e, "build launch");
  s->built = true;
  crt_status r = check_globals(s, st);
  if (r != CRT_OK) {
    std::string msg = g_err;
    free_scene(s);
    delete s;
    return fail(r, msg);
  }
  *out = s;
  return CRT_OK;
}

crt_status crt_scene_create(const crt_mesh_desc* d, void* stream, crt_scene** out) {
  return create_scene(d, stream, false, out);
}

crt_status crt_scene_create_borrowed(const crt_mesh_desc* d, void* stream, crt_scene** out) {
  return create_scene(d, stream, true, out);
}

crt_status crt_scene_destroy(crt_scene* s) {
  if (!s) return CRT_OK;
  cudaDeviceSynchronize();
  free_scene(s);
  delete s;
  return CRT_OK;
}

crt_status crt_scene_set_vertices(crt_scene* s, const float* v, int rebuild, void* stream) {
  if (!s) return fail(CRT_INVALID_ARG, "null scene");
  if (s->borrowed && v)
    return fail(CRT_INVALID_ARG, "a borrowing scene reads the caller's vertex array: update it in place, pass NULL");
  if (!s->borrowed && !v && s->m.nv > 0) return fail(CRT_INVALID_ARG, "null argument");
  cudaStream_t st = S(stream);
  if (!s->borrowed && s->m.nv > 0)
    CRT_CUDA(cudaMemcpyAsync(s->m.verts, v, sizeof(float) * 3 * (size_t)s->m.nv, cudaMemcpyDefault, st), "upload");
  if (rebuild || !s->built) {
    CRT_CUDA(launch_build(s->m, s->b, st), "build launch");
    s->built = true;
  } else {
    CRT_CUDA(launch_refit(s->m, s->b, st), "refit launch");
  }
  return CRT_OK;
}

crt_status crt_bvh_build(crt_scene* s, void* stream) {
  if (!s) return fail(CRT_INVALID_ARG, "null scene");
  CRT_CUDA(launch_build(s->m, s->b, S(stream)), "build launch");
  s->built = true;
  return CRT_OK;
}

crt_status crt_bvh_refit(crt_scene* s, void* stream) {
  if (!s) return fail(CRT_INVALID_ARG, "null scene");
  if (!s->built) return fail(CRT_NOT_BUILT, "refit needs a built BVH");
  CRT_CUDA(launch_refit(s->m, s->b, S(stream)), "refit launch");
  return CRT_OK;
}

crt_status crt_scene_check(crt_scene* s, void* stream) {
  if (!s) return fail(CRT_INVALID_ARG, "null scene");
  return check_globals(s, S(stream));
}

crt_status crt_bvh_export(crt_scene* s, float* scene_box, int32_t* codes, uint32_t* ids, int32_t* nodes3,
                          float* node_boxes, void* stream) {
  if (!s) return fail(CRT_INVALID_ARG, "null scene");
  if (!s->built) return fail(CRT_NOT_BUILT, "no BVH");
  cudaStream_t st = S(stream);
  CRT_CUDA(cudaStreamSynchronize(st), "synchronize");
  const int n = s->m.ntri;
  const size_t nn = n > 0 ? 2 * (size_t)n - 1 : 0;
  SceneGlobals g;
  CRT_CUDA(cudaMemcpy(&g, s->b.g, sizeof(g), cudaMemcpyDeviceToHost), "download");
  auto ord2f_h = [](int i) {
    int bits = i >= 0 ? i : i ^ 0x7FFFFFFF;
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
  };
  std::vector<float> box(6);
  for (int k = 0; k < 3; k++) box[k] = ord2f_h(g.bmin[k]), box[3 + k] = ord2f_h(g.bmax[k]);
  std::vector<uint32_t> hk(n), hv(n);
  std::vector<int> parent(nn);
  std::vector<WNode> wn(n > 1 ? n : 0);
  if (n > 0) {
    CRT_CUDA(cudaMemcpy(hk.data(), s->b.keys_b, 4 * (size_t)n, cudaMemcpyDeviceToHost), "download");
    CRT_CUDA(cudaMemcpy(hv.data(), s->b.vals_b, 4 * (size_t)n, cudaMemcpyDeviceToHost), "download");
    CRT_CUDA(cudaMemcpy(parent.data(), s->b.parent, 4 * nn, cudaMemcpyDeviceToHost), "download");
  }
  if (n > 1) CRT_CUDA(cudaMemcpy(wn.data(), s->b.wnodes, sizeof(WNode) * (size_t)n, cudaMemcpyDeviceToHost), "download");
  std::vector<int> n3(3 * nn);
  std::vector<float> nb(6 * nn);
  auto ref = [n](int code) { return code >= 0 ? code : (n - 1) + ~code; };
  for (size_t i = 0; i < nn; i++) n3[3 * i] = (i == 0) ? -1 : (int)((uint32_t)parent[i] & ((1u << 30) - 1));
  for (int k = 0; k < n; k++) {
    n3[3 * ((n - 1) + k) + 1] = (int)hv[k];
    n3[3 * ((n - 1) + k) + 2] = (int)hv[k];
  }
  // the children of internal node i sit in the wide node of its parent (the
  // root's in the virtual node n - 1), slots 2*side(i) and 2*side(i) + 1
  for (int i = 0; i < n - 1; i++) {
    const uint32_t w = (uint32_t)parent[i];
    const int gp = i == 0 ? n - 1 : (int)(w & ((1u << 30) - 1));
    if (gp < 0 || gp >= n) return fail(CRT_CUDA_ERROR, "inconsistent tree");
    const int s0 = (i == 0 || (w >> 31)) ? 0 : 2;
    for (int c = 0; c < 2; c++) {
      const WSlot& q = wn[gp].s[s0 + c];
      int code;
      std::memcpy(&code, &q.lo_code.w, 4);
      const int r = ref(code);
      if (code == kNoChild || r < 0 || (size_t)r >= nn) return fail(CRT_CUDA_ERROR, "inconsistent tree");
      n3[3 * i + 1 + c] = r;
      const float box[6] = {q.lo_code.x, q.lo_code.y, q.lo_code.z, q.hi.x, q.hi.y, q.hi.z};
      std::memcpy(&nb[6 * (size_t)r], box, sizeof(box));
    }
  }
  if (nn > 0) std::memcpy(&nb[0], g.root_box, 6 * sizeof(float));
  auto put = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    if (!dst || !bytes) return cudaSuccess;
    return cudaMemcpy(dst, src, bytes, cudaMemcpyDefault);
  };
  CRT_CUDA(put(scene_box, box.data(), 6 * sizeof(float)), "export");
  CRT_CUDA(put(codes, hk.data(), 4 * (size_t)n), "export");
  CRT_CUDA(put(ids, hv.data(), 4 * (size_t)n), "export");
  CRT_CUDA(put(nodes3, n3.data(), 4 * n3.size()), "export");
  CRT_CUDA(put(node_boxes, nb.data(), 4 * nb.size()), "export");
  return CRT_OK;
}

static crt_status trace_common(crt_scene* s, const double* rays, int64_t n, int32_t* ids, double* t,
                               double* normals, bool any, void* stream) {
  if (!s || n < 0 || (n > 0 && (!rays || !ids))) return fail(CRT_INVALID_ARG, "bad trace arguments");
  if (!s->built) return fail(CRT_NOT_BUILT, "no BVH");
  if (n == 0) return CRT_OK;
  cudaStream_t st = S(stream);
  DevView vr, vi, vt, vn;
  CRT_CUDA(vr.open(const_cast<double*>(rays), 6 * sizeof(double) * (size_t)n, true, st), "stage rays");
  CRT_CUDA(vi.open(ids, sizeof(int32_t) * (size_t)n, false, st), "stage ids");
  CRT_CUDA(vt.open(t, sizeof(double) * (size_t)n, false, st), "stage t");
  CRT_CUDA(vn.open(any ? nullptr : normals, 3 * sizeof(double) * (size_t)n, false, st), "stage normals");
  CRT_CUDA(launch_trace(dscene(s), static_cast<const double*>(vr.dev), n, any, static_cast<int*>(vi.dev),
                        static_cast<double*>(vt.dev), static_cast<double*>(vn.dev), st),
           "trace launch");
  const bool host_out = vi.temp || vt.temp || vn.temp;
  CRT_CUDA(vr.close(false, st), "unstage");
  CRT_CUDA(vi.close(true, st), "unstage");
  CRT_CUDA(vt.close(true, st), "unstage");
  CRT_CUDA(vn.close(true, st), "unstage");
  if (host_out) return check_globals(s, st);
  return CRT_OK;
}

crt_status crt_trace_closest(crt_scene* s, const double* rays, int64_t n, int32_t* ids, double* t, double* normals,
                             void* stream) {
  return trace_common(s, rays, n, ids, t, normals, false, stream);
}

crt_status crt_trace_shadow(crt_scene* s, const double* rays, int64_t n, int32_t* ids, double* t, void* stream) {
  return trace_common(s, rays, n, ids, t, nullptr, true, stream);
}

// The checks and the RenderArgs shared by crt_render, crt_render_recursive
// and crt_adjoint_lambert (the constants of raytracer.cu:126-130, 144; tan on
// the host).  Outputs start unset.
static crt_status render_args(crt_scene* s, const crt_camera* cam, const crt_light* light,
                              const crt_render_params* p, cudaStream_t st, RenderArgs& a) {
  if (!s->built) return fail(CRT_NOT_BUILT, "no BVH");
  if (p->width <= 0 || p->height <= 0 || p->spp <= 0) return fail(CRT_INVALID_ARG, "width, height, spp must be > 0");
  if (p->spp > CRT_MAX_SPP) return fail(CRT_INVALID_ARG, "spp above CRT_MAX_SPP");
  if ((int64_t)p->width * p->height > (int64_t)1 << 30) return fail(CRT_INVALID_ARG, "image too large");
  int row0 = p->row_begin, row1 = p->row_end;
  if (row0 == 0 && row1 == 0) row1 = p->height;
  if (row0 < 0 || row1 > p->height || row0 >= row1) return fail(CRT_INVALID_ARG, "bad row range");
  a = RenderArgs{};
  a.W = p->width, a.H = p->height, a.spp = p->spp, a.row0 = row0, a.row1 = row1;
  a.group = lanes_per_pixel(p->spp, kDefaultLanesPerPixel);
  a.angle = std::tan(M_PI * 0.5 * cam->fov / 180.0f);
  a.aspect = double(p->width) / double(p->height);
  a.invW = 1.0 / double(p->width);
  a.invH = 1.0 / double(p->height);
  a.aperture = 1 / cam->fstop;
  a.focal = cam->focal_point;
  for (int k = 0; k < 3; k++) {
    a.eye[k] = cam->eye[k];
    a.lpos[k] = light->position[k];
    a.lcol[k] = light->color[k];
  }
  a.lradius = light->radius;
  a.latt[0] = light->constant_term, a.latt[1] = light->linear_term, a.latt[2] = light->quadratic_term;
  a.counter = s->counter;
  a.seed_mix = p->seed * 0x9E3779B1u;
  if (a.aperture != 0.0) {
    const LensTables t = lens_tables(st);
    a.lens_cs = t.cs, a.lens_sqrt = t.sq;
  }
  return CRT_OK;
}

crt_status crt_render(crt_scene* s, const crt_camera* cam, const crt_light* light, const crt_render_params* p,
                      const crt_render_out* o, void* stream) {
  if (!s || !cam || !light || !p || !o) return fail(CRT_INVALID_ARG, "null argument");
  RenderArgs a;
  cudaStream_t st = S(stream);
  if (crt_status e = render_args(s, cam, light, p, st, a)) return e;
  const size_t npx = (size_t)p->width * p->height;
  const size_t nsm = npx * (size_t)p->spp;
  // outputs: whole-image buffers; a row band writes only its rows
  DevView v8, vf, vh, vt, vs, vr, vst, vd, vdp, vsi;
  const bool band = !(a.row0 == 0 && a.row1 == p->height);
  CRT_CUDA(v8.open(o->rgb8, 3 * npx, band, st), "stage rgb8");
  CRT_CUDA(vf.open(o->rgb_f32, 3 * sizeof(float) * npx, band, st), "stage rgb_f32");
  CRT_CUDA(vh.open(o->hit_id, sizeof(int32_t) * nsm, band, st), "stage hit_id");
  CRT_CUDA(vt.open(o->hit_t, sizeof(double) * nsm, band, st), "stage hit_t");
  CRT_CUDA(vs.open(o->shadow, sizeof(int32_t) * nsm, band, st), "stage shadow");
  CRT_CUDA(vr.open(o->rays, 6 * sizeof(double) * nsm, band, st), "stage rays");
  CRT_CUDA(vst.open(o->traversal_stats, 2 * sizeof(uint64_t), false, st), "stage stats");
  CRT_CUDA(vd.open(o->rgb_f64, 3 * sizeof(double) * npx, band, st), "stage rgb_f64");
  CRT_CUDA(vdp.open(o->depth, sizeof(double) * npx, band, st), "stage depth");
  CRT_CUDA(vsi.open(o->shadow_id, sizeof(int32_t) * nsm, band, st), "stage shadow_id");
  if (vst.dev) CRT_CUDA(cudaMemsetAsync(vst.dev, 0, 2 * sizeof(uint64_t), st), "memset");
  a.rgb8 = static_cast<uint8_t*>(v8.dev);
  a.rgbf = static_cast<float*>(vf.dev);
  a.hit_id = static_cast<int*>(vh.dev);
  a.hit_t = static_cast<double*>(vt.dev);
  a.shadow = static_cast<int*>(vs.dev);
  a.rays = static_cast<double*>(vr.dev);
  a.stats = static_cast<unsigned long long*>(vst.dev);
  a.rgbd = static_cast<double*>(vd.dev);
  a.depth = static_cast<double*>(vdp.dev);
  a.shadow_id = static_cast<int*>(vsi.dev);
  CRT_CUDA(launch_render(dscene(s), a, st), "render launch");
  const bool host_out = v8.temp || vf.temp || vh.temp || vt.temp || vs.temp || vr.temp || vst.temp || vd.temp ||
                        vdp.temp || vsi.temp;
  CRT_CUDA(v8.close(true, st), "unstage");
  CRT_CUDA(vf.close(true, st), "unstage");
  CRT_CUDA(vh.close(true, st), "unstage");
  CRT_CUDA(vt.close(true, st), "unstage");
  CRT_CUDA(vs.close(true, st), "unstage");
  CRT_CUDA(vr.close(true, st), "unstage");
  CRT_CUDA(vst.close(true, st), "unstage");
  CRT_CUDA(vd.close(true, st), "unstage");
  CRT_CUDA(vdp.close(true, st), "unstage");
  CRT_CUDA(vsi.close(true, st), "unstage");
  if (host_out) return check_globals(s, st);
  return CRT_OK;
}

crt_status crt_render_recursive(crt_scene* s, const crt_camera* cam, const crt_light* light,
                                const crt_render_params* p, int32_t depth, const crt_optics* optics,
                                const crt_render_out* o, void* stream) {
  if (!s || !cam || !light || !p || !o) return fail(CRT_INVALID_ARG, "null argument");
  if (depth < 0 || depth > CRT_MAX_DEPTH) return fail(CRT_INVALID_ARG, "depth must be in [0, CRT_MAX_DEPTH]");
  if (o->shadow || o->shadow_id || o->depth)
    return fail(CRT_INVALID_ARG,
                "crt_render_recursive writes rgb8, rgb_f32, rgb_f64, hit_id, hit_t, rays and traversal_stats only");
  RenderArgs a;
  cudaStream_t st = S(stream);
  if (crt_status e = render_args(s, cam, light, p, st, a)) return e;
  // kr and ior per material (host or device array); NULL: the kernel takes
  // kr = ks and ior = 1
  static_assert(sizeof(DOptics) == sizeof(crt_optics) && kMaxRecDepth == CRT_MAX_DEPTH, "crt_optics layout");
  DevView vo;
  CRT_CUDA(vo.open(const_cast<crt_optics*>(optics), sizeof(DOptics) * (size_t)s->m.nmat, true, st), "stage optics");
  const size_t npx = (size_t)p->width * p->height;
  const size_t nsm = npx * (size_t)p->spp;
  const bool band = !(a.row0 == 0 && a.row1 == p->height);
  DevView v8, vf, vh, vt, vr, vd, vst;
  CRT_CUDA(vst.open(o->traversal_stats, 2 * sizeof(uint64_t), false, st), "stage stats");
  if (vst.dev) CRT_CUDA(cudaMemsetAsync(vst.dev, 0, 2 * sizeof(uint64_t), st), "memset");
  CRT_CUDA(v8.open(o->rgb8, 3 * npx, band, st), "stage rgb8");
  CRT_CUDA(vf.open(o->rgb_f32, 3 * sizeof(float) * npx, band, st), "stage rgb_f32");
  CRT_CUDA(vh.open(o->hit_id, sizeof(int32_t) * nsm, band, st), "stage hit_id");
  CRT_CUDA(vt.open(o->hit_t, sizeof(double) * nsm, band, st), "stage hit_t");
  CRT_CUDA(vr.open(o->rays, 6 * sizeof(double) * nsm, band, st), "stage rays");
  CRT_CUDA(vd.open(o->rgb_f64, 3 * sizeof(double) * npx, band, st), "stage rgb_f64");
  a.rgb8 = static_cast<uint8_t*>(v8.dev);
  a.rgbf = static_cast<float*>(vf.dev);
  a.hit_id = static_cast<int*>(vh.dev);
  a.hit_t = static_cast<double*>(vt.dev);
  a.rays = static_cast<double*>(vr.dev);
  a.rgbd = static_cast<double*>(vd.dev);
  a.stats = static_cast<unsigned long long*>(vst.dev);
  CRT_CUDA(launch_render_recursive(dscene(s), a, static_cast<const DOptics*>(vo.dev), depth, st),
           "recursive render launch");
  CRT_CUDA(vo.close(false, st), "unstage");
  const bool host_out = v8.temp || vf.temp || vh.temp || vt.temp || vr.temp || vd.temp || vst.temp;
  CRT_CUDA(vst.close(true, st), "unstage");
  CRT_CUDA(v8.close(true, st), "unstage");
  CRT_CUDA(vf.close(true, st), "unstage");
  CRT_CUDA(vh.close(true, st), "unstage");
  CRT_CUDA(vt.close(true, st), "unstage");
  CRT_CUDA(vr.close(true, st), "unstage");
  CRT_CUDA(vd.close(true, st), "unstage");
  if (host_out) return check_globals(s, st);
  return CRT_OK;
}

crt_status crt_scene_set_materials(crt_scene* s, const crt_material* mats, int32_t num, void* stream) {
  if (!s || !mats) return fail(CRT_INVALID_ARG, "null argument");
  if (s->borrowed) return fail(CRT_INVALID_ARG, "a borrowing scene reads the caller's material array");
  if (num != s->m.nmat) return fail(CRT_INVALID_ARG, "material count differs from the scene's");
  CRT_CUDA(cudaMemcpyAsync(s->m.mats, mats, sizeof(DMat) * (size_t)num, cudaMemcpyDefault, S(stream)), "upload");
  return CRT_OK;
}

crt_status crt_adjoint_lambert(crt_scene* s, const crt_camera* cam, const crt_light* light,
                               const crt_render_params* p, const double* grad_rgb, const double* grad_depth,
                               double* grad_vertices, double* grad_light, double* grad_kd, void* stream) {
  if (!s || !cam || !light || !p || !grad_rgb) return fail(CRT_INVALID_ARG, "null argument");
  RenderArgs a;
  cudaStream_t st = S(stream);
  if (crt_status e = render_args(s, cam, light, p, st, a)) return e;
  const size_t npx = (size_t)p->width * p->height;
  DevView vg, vgd;
  CRT_CUDA(vg.open(const_cast<double*>(grad_rgb), 3 * sizeof(double) * npx, true, st), "stage grad_rgb");
  CRT_CUDA(vgd.open(const_cast<double*>(grad_depth), sizeof(double) * npx, true, st), "stage grad_depth");
  // gradient outputs: always through device scratch (they are accumulated atomically)
  const size_t nv3 = 3 * (size_t)s->m.nv, nk3 = 3 * (size_t)s->m.nmat;
  double* acc = nullptr;
  CRT_CUDA(cudaMallocAsync(&acc, sizeof(double) * (nv3 + 3 + nk3), st), "scratch");
  CRT_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * (nv3 + 3 + nk3), st), "memset");
  a.grad_rgb = static_cast<const double*>(vg.dev);
  a.grad_depth = static_cast<const double*>(vgd.dev);
  a.grad_verts = acc;
  a.grad_light = acc + nv3;
  a.grad_albedo = acc + nv3 + 3;
  CRT_CUDA(launch_render(dscene(s), a, st), "adjoint launch");
  auto out = [&](double* dst, const double* src, size_t n) -> cudaError_t {
    return (dst && n) ? cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDefault, st) : cudaSuccess;
  };
  CRT_CUDA(out(grad_vertices, acc, nv3), "download");
  CRT_CUDA(out(grad_light, acc + nv3, 3), "download");
  CRT_CUDA(out(grad_kd, acc + nv3 + 3, nk3), "download");
  CRT_CUDA(cudaFreeAsync(acc, st), "free");
  CRT_CUDA(vg.close(false, st), "unstage");
  CRT_CUDA(vgd.close(false, st), "unstage");
  return check_globals(s, st);
}

crt_status crt_morton(const float* verts, int32_t num_vertices, const int32_t* vidx, int32_t n, const float* box6,
                      int32_t* codes, void* stream) {
  if (n < 0 || n > CRT_MAX_TRIANGLES || num_vertices < 0 || num_vertices > CRT_MAX_VERTICES ||
      (n > 0 && (!verts || !vidx || !box6 || !codes)))
    return fail(CRT_INVALID_ARG, "bad arguments");
  if (n == 0) return CRT_OK;
  if (!(is_device_ptr(verts) && is_device_ptr(vidx) && is_device_ptr(box6) && is_device_ptr(codes)))
    return fail(CRT_INVALID_ARG, "crt_morton takes device pointers");
  cudaStream_t st = S(stream);
  int* scratch = nullptr;  // error bit
  CRT_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&scratch), sizeof(int), st), "scratch");
  CRT_CUDA(cudaMemsetAsync(scratch, 0, sizeof(int), st), "memset");
  const cudaError_t e =
      launch_morton(verts, num_vertices, vidx, n, box6, reinterpret_cast<uint32_t*>(codes), scratch, st);
  int err = 0;
  if (e == cudaSuccess) CRT_CUDA(cudaMemcpyAsync(&err, scratch, sizeof(int), cudaMemcpyDeviceToHost, st), "read");
  CRT_CUDA(cudaFreeAsync(scratch, st), "free");
  CRT_CUDA(e, "morton launch");
  CRT_CUDA(cudaStreamSynchronize(st), "synchronize");
  if (err) return fail(CRT_INVALID_ARG, "a vertex index is out of range");
  return CRT_OK;
}

crt_status crt_hierarchy(const uint32_t* codes, const uint32_t* ids, int32_t n, int32_t* nodes3, void* stream) {
  if (n < 0 || n > CRT_MAX_TRIANGLES || (n > 0 && (!codes || !ids || !nodes3))) return fail(CRT_INVALID_ARG, "bad arguments");
  if (n == 0) return CRT_OK;
  if (!(is_device_ptr(codes) && is_device_ptr(ids) && is_device_ptr(nodes3)))
    return fail(CRT_INVALID_ARG, "crt_hierarchy takes device pointers");
  cudaStream_t st = S(stream);
  const size_t nn = 2 * (size_t)n - 1;
  const size_t bytes = align256(4 * nn) + sizeof(WNode) * (size_t)n;
  char* scratch = nullptr;
  CRT_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&scratch), bytes, st), "scratch");
  uint32_t* parent = reinterpret_cast<uint32_t*>(scratch);
  WNode* wnodes = reinterpret_cast<WNode*>(scratch + align256(4 * nn));
  const cudaError_t e = launch_stage_hierarchy(codes, ids, n, nodes3, parent, wnodes, st);
  CRT_CUDA(cudaFreeAsync(scratch, st), "free");
  CRT_CUDA(e, "hierarchy launch");
  return CRT_OK;
}

crt_status crt_refit(const float* vertices, int32_t num_vertices, const int32_t* vertex_indices, int32_t n,
                     const uint32_t* ids, const int32_t* nodes3, float* node_boxes, void* stream) {
  if (n < 0 || n > CRT_MAX_TRIANGLES || num_vertices < 0 || num_vertices > CRT_MAX_VERTICES ||
      (n > 0 && (!vertices || !vertex_indices || !ids || !nodes3 || !node_boxes)))
    return fail(CRT_INVALID_ARG, "bad arguments");
  if (n == 0) return CRT_OK;
  if (!(is_device_ptr(vertices) && is_device_ptr(vertex_indices) && is_device_ptr(ids) && is_device_ptr(nodes3) &&
        is_device_ptr(node_boxes)))
    return fail(CRT_INVALID_ARG, "crt_refit takes device pointers");
  cudaStream_t st = S(stream);
  int* scratch = nullptr;  // [0] error bits, [1..n-1] arrival flags
  CRT_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&scratch), 4 * (size_t)n, st), "scratch");
  CRT_CUDA(cudaMemsetAsync(scratch, 0, 4 * (size_t)n, st), "memset");
  const cudaError_t e = launch_stage_refit(vertices, num_vertices, vertex_indices, n, ids, nodes3, node_boxes,
                                           scratch + 1, scratch, st);
  int err = 0;
  if (e == cudaSuccess) CRT_CUDA(cudaMemcpyAsync(&err, scratch, sizeof(int), cudaMemcpyDeviceToHost, st), "read");
  CRT_CUDA(cudaFreeAsync(scratch, st), "free");
  CRT_CUDA(e, "refit launch");
  CRT_CUDA(cudaStreamSynchronize(st), "synchronize");
  if (err) return fail(CRT_INVALID_ARG, "an id, vertex index or node index is out of range");
  return CRT_OK;
}

crt_status crt_sort_pairs(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, int32_t n,
                          int32_t key_bits, void* stream) {
  if (n < 0 || n > CRT_MAX_TRIANGLES || key_bits < 1 || key_bits > 32) return fail(CRT_INVALID_ARG, "bad sizes");
  if (n == 0) return CRT_OK;
  if (const char* why = sort_args_problem(kin, vin, kout, vout, n))
    return fail(CRT_INVALID_ARG, std::string("crt_sort_pairs: ") + why);
  cudaStream_t st = S(stream);
  const size_t bytes = sort_scratch_bytes(n, key_bits) + 256;
  void* scratch = nullptr;
  CRT_CUDA(cudaMallocAsync(&scratch, bytes, st), "scratch");
  int* err = reinterpret_cast<int*>(static_cast<char*>(scratch) + bytes - 256);
  cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e == cudaSuccess) e = launch_sort_pairs(kin, vin, kout, vout, n, key_bits, scratch, err, st);
  int herr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaError_t e2 = cudaFreeAsync(scratch, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(e, "sort");
  if (herr & kErrTimeout) return fail(CRT_TIMEOUT, "a radix-sort look-back wait timed out");
  return CRT_OK;
}

}  // extern "C"

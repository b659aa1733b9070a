// batch.cu -- the batched form: many meshes, each with its own camera and
// light, built and rendered together by the persistent kernels of
// batch_kernel.cuh (one launch, or the render in a second one), captured once
// into a CUDA graph and replayed.  The block size, the lanes each pixel
// takes, the shared-memory part of the traversal stack and the number of
// launches are chosen by crt_batch_autotune.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "crt.h"
#include "batch_kernel.cuh"

namespace crt {
void set_last_error(const char* msg);
}

using namespace crt;

struct crt_batch {
  int M = 0, N = 0, V = 0, Nn = 0, Mat = 0;
  std::vector<int> tri_off, px_off;  // host copies
  std::vector<int> item_off;           // kLaneOptions x (M + 1): work-item prefix per lanes option
  int* d_item_off = nullptr;
  std::vector<crt_batch_view> views;
  void* block = nullptr;  // one allocation for everything
  BatchBufs b;
  BatchView v;
  uint8_t* image = nullptr;  // concatenated rgb8 images
  size_t image_bytes = 0;
  RenderArgs* args = nullptr;
  BatchTuning tuning;
  unsigned* bar = nullptr;     // the grid barrier of the persistent kernel (2 words)
  cudaStream_t cap = nullptr;  // capture stream (the legacy stream cannot be captured)
  cudaGraphExec_t graph = nullptr;
};

namespace {

crt_status fail(crt_status s, const std::string& m) {
  crt::set_last_error(m.c_str());
  return s;
}
crt_status cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();
  return fail(e == cudaErrorMemoryAllocation ? CRT_OOM : CRT_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CRT_CUDA(call, what)                               \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(e_, what);     \
  } while (0)

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

bool on_device(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Work-item prefixes are kept for every lanes-per-pixel option.
constexpr int kLaneOptions = 6;
constexpr int kLanes[kLaneOptions] = {1, 2, 4, 8, 16, 32};

int option_of(const BatchTuning& t) {
  for (int s = 0; s < kLaneOptions; s++)
    if (kLanes[s] == t.lanes) return s;
  return 0;
}

// The device view for tuning t (the work-item prefix depends on the lanes per pixel).
BatchView view_for(const crt_batch* b, const BatchTuning& t) {
  BatchView v = b->v;
  const int s = option_of(t);
  v.item_off = b->d_item_off + (size_t)s * (b->M + 1);
  v.items = b->item_off[(size_t)s * (b->M + 1) + b->M];
  return v;
}

// One launch of k_batch<TH, SHORT> over phases [first, last]: as many
// blocks as can be resident at once (the launch is cooperative, so the grid
// barrier between phases cannot wait on a block that is not running).
template <int TH, int SHORT>
cudaError_t launch_batch_kernel(const BatchLaunch& L, cudaStream_t st) {
  const size_t smem = batch_smem_bytes<TH>(SHORT, L.first < kPhRender);
  void (*k)(const BatchBufs, const BatchView, int, int, unsigned*, int, int) = k_batch<TH, SHORT>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int bps = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, TH, smem);
  if (e != cudaSuccess) return e;
  if (bps <= 0) return cudaErrorInvalidConfiguration;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(num_sms() * bps));
  cfg.blockDim = dim3(TH);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, L.b, L.v, L.gmax, L.sort_tiles, L.bar, L.first, L.last);
}

// The render phase alone, in k_batch_render (persistent, not cooperative:
// it has no grid barrier).
template <int TH, int SHORT>
cudaError_t launch_render_kernel(const BatchLaunch& L, cudaStream_t st) {
  const size_t smem = batch_smem_bytes<TH>(SHORT, false);
  void (*k)(const BatchView, int) = k_batch_render<TH, SHORT>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int bps = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k, TH, smem);
  if (e != cudaSuccess) return e;
  k<<<num_sms() * (bps > 0 ? bps : 1), TH, smem, st>>>(L.v, L.gmax);
  return cudaGetLastError();
}

template <int TH, int SHORT>
cudaError_t launch_phases(const BatchLaunch& L, bool render_kernel, cudaStream_t st) {
  return render_kernel ? launch_render_kernel<TH, SHORT>(L, st) : launch_batch_kernel<TH, SHORT>(L, st);
}

template <int TH>
cudaError_t launch_batch_stack(const BatchLaunch& L, int stack, bool render_kernel, cudaStream_t st) {
  switch (stack) {
    case 8:
      return launch_phases<TH, 8>(L, render_kernel, st);
    case 16:
      return launch_phases<TH, 16>(L, render_kernel, st);
    default:
      return launch_phases<TH, 0>(L, render_kernel, st);
  }
}

// Enqueue phases [first, last] with tuning t.  With t.launches == 2 the
// render phase runs in k_batch_render after k_batch has run the others.
// The barrier words are cleared before each k_batch launch, and the render's
// item counter before a render that the init phase of the same launch does
// not precede.
cudaError_t enqueue_phases(crt_batch* b, const BatchTuning& t, int first, int last, cudaStream_t st) {
  BatchLaunch L;
  L.b = b->b;
  L.v = view_for(b, t);
  L.gmax = t.lanes;
  L.sort_tiles = sort_tiles(b->N);
  L.bar = b->bar;
  auto run = [&](int f, int l, bool render_kernel) -> cudaError_t {
    L.first = f, L.last = l;
    cudaError_t e = cudaSuccess;
    if (!render_kernel) e = cudaMemsetAsync(b->bar, 0, 2 * sizeof(unsigned), st);
    if (e == cudaSuccess && l == kPhRender && (f > kPhInit || render_kernel))
      e = cudaMemsetAsync(b->v.counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    return t.block == 128 ? launch_batch_stack<128>(L, t.stack, render_kernel, st)
                          : launch_batch_stack<256>(L, t.stack, render_kernel, st);
  };
  if (t.launches == 2 && last == kPhRender) {
    if (first < kPhRender) {
      const cudaError_t e = run(first, kPhRefitTop, false);
      if (e != cudaSuccess) return e;
    }
    return run(kPhRender, kPhRender, true);
  }
  return run(first, last, false);
}

cudaError_t enqueue(crt_batch* b, cudaStream_t st) { return enqueue_phases(b, b->tuning, kPhInit, kPhRender, st); }

void drop_graph(crt_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
}

}  // namespace

extern "C" {

crt_status crt_batch_create(const crt_mesh_desc* meshes, const crt_batch_view* views, int32_t M, void* stream,
                            crt_batch** out) {
  if (!meshes || !views || !out || M <= 0) return fail(CRT_INVALID_ARG, "bad arguments");
  *out = nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  crt_batch* b = new crt_batch;
  b->M = M;
  b->tri_off.assign(M + 1, 0);
  if (M > kRadix) {
    delete b;
    return fail(CRT_INVALID_ARG, "at most " + std::to_string(kRadix) + " meshes in a batch");
  }
  b->item_off.assign((size_t)kLaneOptions * (M + 1), 0);
  b->px_off.assign(M + 1, 0);
  std::vector<int> vert_off(M + 1, 0), nrm_off(M + 1, 0), mat_off(M + 1, 0);
  for (int m = 0; m < M; m++) {
    const crt_mesh_desc& d = meshes[m];
    const crt_batch_view& w = views[m];
    if (d.num_triangles <= 0 || !d.vertices || !d.vertex_indices || !d.normals || !d.materials ||
        d.num_materials <= 0 || w.width <= 0 || w.height <= 0 || w.spp <= 0) {
      delete b;
      return fail(CRT_INVALID_ARG, "batch mesh " + std::to_string(m) + ": bad description");
    }
    if (on_device(d.vertices) || on_device(d.vertex_indices)) {
      delete b;
      return fail(CRT_INVALID_ARG, "crt_batch_create takes host meshes");
    }
    // sizes, one mesh and the running totals (the offsets below are int32)
    if (d.num_vertices <= 0 || d.num_normals <= 0 || (int64_t)vert_off[m] + d.num_vertices > CRT_MAX_VERTICES ||
        (int64_t)nrm_off[m] + d.num_normals > CRT_MAX_VERTICES ||
        (int64_t)b->tri_off[m] + d.num_triangles > CRT_MAX_TRIANGLES ||
        (int64_t)mat_off[m] + d.num_materials > INT32_MAX || (int64_t)w.width * w.height > ((int64_t)1 << 30) ||
        (int64_t)b->px_off[m] + (int64_t)w.width * w.height > INT32_MAX || w.spp > CRT_MAX_SPP) {
      delete b;
      return fail(CRT_INVALID_ARG, "batch mesh " + std::to_string(m) + ": a size is out of range");
    }
    for (int64_t i = 0; i < 3 * (int64_t)d.num_triangles; i++) {
      const int32_t* ni = d.normal_indices ? d.normal_indices : d.vertex_indices;
      if (d.vertex_indices[i] < 0 || d.vertex_indices[i] >= d.num_vertices || ni[i] < 0 || ni[i] >= d.num_normals) {
        delete b;
        return fail(CRT_INVALID_ARG, "batch mesh " + std::to_string(m) + ": index out of range");
      }
    }
    for (int t = 0; d.material_ids && t < d.num_triangles; t++)
      if (d.material_ids[t] < 0 || d.material_ids[t] >= d.num_materials) {
        delete b;
        return fail(CRT_INVALID_ARG, "batch mesh " + std::to_string(m) + ": material id out of range");
      }
    b->tri_off[m + 1] = b->tri_off[m] + d.num_triangles;
    vert_off[m + 1] = vert_off[m] + d.num_vertices;
    nrm_off[m + 1] = nrm_off[m] + d.num_normals;
    mat_off[m + 1] = mat_off[m] + d.num_materials;
    for (int sh = 0; sh < kLaneOptions; sh++) {  // warp tiles of 32 / G pixels
      const int G = lanes_per_pixel(w.spp, kLanes[sh]), tw = group_tile_w(G), th = group_tile_h(G);
      int* io = &b->item_off[(size_t)sh * (M + 1)];
      io[m + 1] = io[m] + ((w.width + tw - 1) / tw) * ((w.height + th - 1) / th);
    }
    b->px_off[m + 1] = b->px_off[m] + w.width * w.height;
    b->views.push_back(w);
  }
  const int N = b->tri_off[M], V = vert_off[M], Nn = nrm_off[M], Mat = mat_off[M];
  b->N = N, b->V = V, b->Nn = Nn, b->Mat = Mat;
  // host staging of the concatenated arrays (indices made global)
  std::vector<float> hv(3 * (size_t)V), hn(3 * (size_t)Nn);
  std::vector<int> hvi(3 * (size_t)N), hni(3 * (size_t)N), hmat(N), hmesh(N);
  std::vector<crt_material> hm(Mat);
  for (int m = 0; m < M; m++) {
    const crt_mesh_desc& d = meshes[m];
    std::memcpy(&hv[3 * (size_t)vert_off[m]], d.vertices, 12 * (size_t)d.num_vertices);
    std::memcpy(&hn[3 * (size_t)nrm_off[m]], d.normals, 12 * (size_t)d.num_normals);
    std::memcpy(&hm[mat_off[m]], d.materials, sizeof(crt_material) * d.num_materials);
    const int32_t* ni = d.normal_indices ? d.normal_indices : d.vertex_indices;
    for (int t = 0; t < d.num_triangles; t++) {
      const size_t g = (size_t)b->tri_off[m] + t;
      for (int k = 0; k < 3; k++) {
        hvi[3 * g + k] = vert_off[m] + d.vertex_indices[3 * t + k];
        hni[3 * g + k] = nrm_off[m] + ni[3 * t + k];
      }
      hmat[g] = mat_off[m] + (d.material_ids ? d.material_ids[t] : 0);
      hmesh[g] = m;
    }
  }
  // one device block
  const int tiles = sort_tiles(N);
  const int NI = N - M;
  b->image_bytes = 3 * (size_t)b->px_off[M];
  const size_t sz[] = {12 * (size_t)V, 12 * (size_t)Nn, 12 * (size_t)N, 12 * (size_t)N, 4 * (size_t)N,
                       sizeof(DMat) * (size_t)Mat, 4 * (size_t)N, 4 * (size_t)(M + 1), 4 * (size_t)kLaneOptions * (M + 1),
                       5 * 4 * (size_t)N, 4 * 4 * (size_t)kRadix, 4 * 4 * (size_t)tiles * kRadix,
                       4 * (size_t)(NI + N), 4 * (size_t)(NI > 0 ? NI : 1), 0,
                       sizeof(LeafTri) * (size_t)N, sizeof(SceneGlobals) * (size_t)M, 128, b->image_bytes,
                       sizeof(RenderArgs) * (size_t)M, sizeof(WNode) * (size_t)(NI + M), sizeof(uint2) * (size_t)N};
  const int K = sizeof(sz) / sizeof(sz[0]);
  std::vector<size_t> off(K);
  size_t total = 0;
  for (int i = 0; i < K; i++) off[i] = total, total += al(sz[i]);
  cudaError_t e = cudaMalloc(&b->block, total);
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "cudaMalloc");
  }
  char* base = static_cast<char*>(b->block);
  auto at = [&](int i) { return base + off[i]; };
  float* d_v = (float*)at(0);
  float* d_n = (float*)at(1);
  int* d_vi = (int*)at(2);
  int* d_ni = (int*)at(3);
  int* d_mat = (int*)at(4);
  DMat* d_mats = (DMat*)at(5);
  int* d_mesh = (int*)at(6);
  int* d_toff = (int*)at(7);
  int* d_ioff = (int*)at(8);
  uint32_t* keys = (uint32_t*)at(9);
  BatchBufs& bb = b->b;
  bb.M = M, bb.N = N, bb.NI = NI;
  bb.verts = d_v, bb.vidx = d_vi, bb.mesh_of = d_mesh, bb.tri_off = d_toff;
  bb.keys_a = keys, bb.keys_b = keys + N, bb.vals_a = keys + 2 * (size_t)N, bb.vals_b = keys + 3 * (size_t)N;
  bb.codes0 = keys + 4 * (size_t)N;
  bb.hist = (uint32_t*)at(10);
  bb.status = (uint32_t*)at(11);
  bb.parent = (uint32_t*)at(12);
  bb.flags = (int*)at(13);
  bb.leaves = (LeafTri*)at(15);
  bb.g = (SceneGlobals*)at(16);
  bb.counters = (unsigned*)at(17);
  bb.err = (int*)(at(17) + 32);
  b->bar = (unsigned*)(at(17) + 64);
  b->image = (uint8_t*)at(18);
  b->args = (RenderArgs*)at(19);
  bb.wnodes = (WNode*)at(20);
  bb.arrivals = (uint2*)at(21);
  BatchView& v = b->v;
  b->d_item_off = d_ioff;
  v.M = M, v.tri_off = d_toff;
  v.verts = d_v, v.normals = d_n, v.vidx = d_vi, v.nidx = d_ni, v.matid = d_mat, v.mats = d_mats;
  v.wnodes = bb.wnodes, v.leaves = bb.leaves, v.g = bb.g, v.args = b->args;
  v.counter = bb.counters + 4;
  // per-mesh render arguments
  bool lens = false;
  for (int m = 0; m < M; m++) lens = lens || 1 / views[m].camera.fstop != 0.0;
  const LensTables lt = lens ? lens_tables(st) : LensTables{};
  std::vector<RenderArgs> ha(M);
  for (int m = 0; m < M; m++) {
    const crt_batch_view& w = views[m];
    RenderArgs& a = ha[m];
    a = RenderArgs{};  // every field zero or null
    a.W = w.width, a.H = w.height, a.spp = w.spp, a.row0 = 0, a.row1 = w.height;
    a.angle = std::tan(M_PI * 0.5 * w.camera.fov / 180.0f);
    a.aspect = double(w.width) / double(w.height);
    a.invW = 1.0 / double(w.width);
    a.invH = 1.0 / double(w.height);
    a.aperture = 1 / w.camera.fstop;
    a.focal = w.camera.focal_point;
    for (int k = 0; k < 3; k++) {
      a.eye[k] = w.camera.eye[k];
      a.lpos[k] = w.light.position[k];
      a.lcol[k] = w.light.color[k];
    }
    a.lradius = w.light.radius;
    a.latt[0] = w.light.constant_term, a.latt[1] = w.light.linear_term, a.latt[2] = w.light.quadratic_term;
    a.rgb8 = b->image + 3 * (size_t)b->px_off[m];
    a.lens_cs = lt.cs, a.lens_sqrt = lt.sq;
  }
  static_assert(sizeof(DMat) == sizeof(crt_material), "material layout");
  auto up = [&](void* dst, const void* src, size_t n) {
    return n ? cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, st) : cudaSuccess;
  };
  if ((e = up(d_v, hv.data(), 4 * hv.size())) != cudaSuccess || (e = up(d_n, hn.data(), 4 * hn.size())) != cudaSuccess ||
      (e = up(d_vi, hvi.data(), 4 * hvi.size())) != cudaSuccess ||
      (e = up(d_ni, hni.data(), 4 * hni.size())) != cudaSuccess ||
      (e = up(d_mat, hmat.data(), 4 * hmat.size())) != cudaSuccess ||
      (e = up(d_mats, hm.data(), sizeof(crt_material) * hm.size())) != cudaSuccess ||
      (e = up(d_mesh, hmesh.data(), 4 * hmesh.size())) != cudaSuccess ||
      (e = up(d_toff, b->tri_off.data(), 4 * (M + 1))) != cudaSuccess ||
      (e = up(d_ioff, b->item_off.data(), 4 * b->item_off.size())) != cudaSuccess ||
      (e = up(b->args, ha.data(), sizeof(RenderArgs) * M)) != cudaSuccess ||
      (e = cudaMemsetAsync(bb.flags, 0, sz[13], st)) != cudaSuccess ||
      (e = cudaMemsetAsync(at(17), 0, sz[17], st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking)) != cudaSuccess) {
    cudaFree(b->block);
    delete b;
    return cuda_fail(e, "batch upload");
  }
  *out = b;
  return CRT_OK;
}

crt_status crt_batch_destroy(crt_batch* b) {
  if (!b) return CRT_OK;
  cudaDeviceSynchronize();
  drop_graph(b);
  if (b->cap) cudaStreamDestroy(b->cap);
  cudaFree(b->block);
  delete b;
  return CRT_OK;
}

crt_status crt_batch_set_tuning(crt_batch* b, const crt_batch_tuning* t) {
  if (!b || !t) return fail(CRT_INVALID_ARG, "null argument");
  bool lanes_ok = false;
  for (int s = 0; s < kLaneOptions; s++) lanes_ok = lanes_ok || t->lanes_per_pixel == kLanes[s];
  const bool ok = (t->block_size == 128 || t->block_size == 256) && lanes_ok &&
                  (t->stack == 0 || t->stack == 8 || t->stack == 16) && (t->launches == 1 || t->launches == 2);
  if (!ok) return fail(CRT_INVALID_ARG, "unsupported tuning");
  b->tuning.block = t->block_size, b->tuning.lanes = t->lanes_per_pixel, b->tuning.stack = t->stack;
  b->tuning.launches = t->launches;
  drop_graph(b);
  return CRT_OK;
}

crt_status crt_batch_run(crt_batch* b, int use_graph, uint8_t* rgb8, void* stream) {
  if (!b) return fail(CRT_INVALID_ARG, "null batch");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (use_graph) {
    if (!b->graph) {
      cudaGraph_t g = nullptr;
      CRT_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
      cudaError_t e = enqueue(b, b->cap);
      cudaError_t e2 = cudaStreamEndCapture(b->cap, &g);
      if (e != cudaSuccess) return cuda_fail(e, "capture");
      if (e2 != cudaSuccess) return cuda_fail(e2, "end capture");
      e = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "instantiate");
    }
    CRT_CUDA(cudaGraphLaunch(b->graph, st), "graph launch");
  } else {
    CRT_CUDA(enqueue(b, st), "batch launch");
  }
  if (rgb8) CRT_CUDA(cudaMemcpyAsync(rgb8, b->image, b->image_bytes, cudaMemcpyDefault, st), "download");
  if (rgb8 && !on_device(rgb8)) CRT_CUDA(cudaStreamSynchronize(st), "synchronize");
  return CRT_OK;
}

crt_status crt_batch_check(crt_batch* b, void* stream) {
  if (!b) return fail(CRT_INVALID_ARG, "null batch");
  CRT_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "synchronize");
  int err = 0;
  CRT_CUDA(cudaMemcpy(&err, b->b.err, sizeof(int), cudaMemcpyDeviceToHost), "read");
  std::vector<SceneGlobals> g(b->M);
  CRT_CUDA(cudaMemcpy(g.data(), b->b.g, sizeof(SceneGlobals) * b->M, cudaMemcpyDeviceToHost), "read");
  for (auto& x : g) err |= x.err;
  if (err & kErrTimeout) return fail(CRT_TIMEOUT, "a radix-sort look-back wait timed out");
  if (err & kErrStack) return fail(CRT_STACK_OVERFLOW, "a traversal exceeded the 64-entry stack");
  if (err & kErrNonFinite) return fail(CRT_INVALID_ARG, "non-finite (or |x| > 1e37) vertex coordinate");
  return CRT_OK;
}

// Times the supported tunings on the batch (build once, then the render
// phase alone per tuning after a warm-up render, in k_batch for the
// one-launch form and in k_batch_render for the two-launch form; lanes
// options that give every mesh the same lanes per pixel as a smaller option
// are skipped) and keeps the fastest.
crt_status crt_batch_autotune(crt_batch* b, crt_batch_tuning* chosen, void* stream) {
  if (!b) return fail(CRT_INVALID_ARG, "null batch");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int blocks[] = {128, 256};
  const int stacks[] = {0, 8, 16};
  cudaEvent_t e0, e1;
  CRT_CUDA(cudaEventCreate(&e0), "event");
  CRT_CUDA(cudaEventCreate(&e1), "event");
  BatchTuning best = b->tuning;
  float best_ms = 1e30f;
  CRT_CUDA(enqueue_phases(b, best, kPhInit, kPhRefitTop, st), "build");
  CRT_CUDA(enqueue_phases(b, best, kPhRender, kPhRender, st), "render");  // warm-up
  for (int li = 0; li < kLaneOptions; li++) {
    bool same = li > 0;
    for (int m = 0; m < b->M && same; m++)
      same = lanes_per_pixel(b->views[m].spp, kLanes[li]) == lanes_per_pixel(b->views[m].spp, kLanes[li - 1]);
    if (same) continue;
    for (int bs : blocks)
      for (int sk : stacks)
        for (int nl = 1; nl <= 2; nl++) {
          BatchTuning t;
          t.block = bs, t.lanes = kLanes[li], t.stack = sk, t.launches = nl;
          CRT_CUDA(cudaEventRecord(e0, st), "event");
          CRT_CUDA(enqueue_phases(b, t, kPhRender, kPhRender, st), "render");
          CRT_CUDA(cudaEventRecord(e1, st), "event");
          CRT_CUDA(cudaEventSynchronize(e1), "event");
          float ms = 0.f;
          CRT_CUDA(cudaEventElapsedTime(&ms, e0, e1), "event");
          if (ms < best_ms) best_ms = ms, best = t;
        }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->tuning = best;
  drop_graph(b);
  if (chosen) {
    chosen->block_size = best.block, chosen->lanes_per_pixel = best.lanes, chosen->stack = best.stack;
    chosen->launches = best.launches;
    chosen->render_ms = best_ms;
  }
  return CRT_OK;
}

// The build products of one mesh of the batch, in crt_bvh_export's layout.
crt_status crt_batch_export(crt_batch* b, int32_t m, float* scene_box, int32_t* codes, uint32_t* ids,
                            int32_t* nodes3, float* node_boxes, void* stream) {
  if (!b || m < 0 || m >= b->M) return fail(CRT_INVALID_ARG, "bad mesh index");
  CRT_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "synchronize");
  const int t0 = b->tri_off[m], n = b->tri_off[m + 1] - t0, NI = b->b.NI, ib = t0 - m;
  const size_t nn = 2 * (size_t)n - 1;
  SceneGlobals g;
  CRT_CUDA(cudaMemcpy(&g, b->b.g + m, sizeof(g), cudaMemcpyDeviceToHost), "download");
  auto ord2f_h = [](int i) {
    int bits = i >= 0 ? i : i ^ 0x7FFFFFFF;
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
  };
  std::vector<uint32_t> hk(n), hv(n), par_i(n > 1 ? n - 1 : 0), par_l(n);
  std::vector<WNode> wn(n > 1 ? n - 1 : 0);
  WNode wroot;
  CRT_CUDA(cudaMemcpy(hk.data(), b->b.keys_b + t0, 4 * (size_t)n, cudaMemcpyDeviceToHost), "download");
  CRT_CUDA(cudaMemcpy(hv.data(), b->b.vals_a + t0, 4 * (size_t)n, cudaMemcpyDeviceToHost), "download");
  CRT_CUDA(cudaMemcpy(par_l.data(), b->b.parent + NI + t0, 4 * (size_t)n, cudaMemcpyDeviceToHost), "download");
  if (n > 1) {
    CRT_CUDA(cudaMemcpy(par_i.data(), b->b.parent + ib, 4 * (size_t)(n - 1), cudaMemcpyDeviceToHost), "download");
    CRT_CUDA(cudaMemcpy(wn.data(), b->b.wnodes + ib, sizeof(WNode) * (n - 1), cudaMemcpyDeviceToHost), "download");
    CRT_CUDA(cudaMemcpy(&wroot, b->b.wnodes + NI + m, sizeof(WNode), cudaMemcpyDeviceToHost), "download");
  }
  const uint32_t mask = (1u << 30) - 1;
  std::vector<int> n3(3 * nn);
  std::vector<float> nb(6 * nn);
  auto ref = [n](int code) { return code >= 0 ? code : (n - 1) + ~code; };
  for (int i = 0; i < n - 1; i++) n3[3 * i] = i == 0 ? -1 : (int)(par_i[i] & mask) - ib;
  for (int k = 0; k < n; k++) {
    n3[3 * ((n - 1) + k)] = n > 1 ? (int)(par_l[k] & mask) - ib : -1;
    n3[3 * ((n - 1) + k) + 1] = n3[3 * ((n - 1) + k) + 2] = (int)hv[k] - t0;
  }
  // the children of internal node i sit in the wide node of its parent (the
  // root's in the mesh's virtual node), slots 2*side(i) and 2*side(i) + 1
  for (int i = 0; i < n - 1; i++) {
    const int pl = (int)(par_i[i] & mask) - ib;
    if (i > 0 && (pl < 0 || pl >= n - 1)) return fail(CRT_CUDA_ERROR, "inconsistent tree");
    const WNode& gw = i == 0 ? wroot : wn[pl];
    const int s0 = (i == 0 || (par_i[i] >> 31)) ? 0 : 2;
    for (int c = 0; c < 2; c++) {
      const WSlot& q = gw.s[s0 + c];
      int code;
      std::memcpy(&code, &q.lo_code.w, 4);
      const int r = ref(code);
      if (code == kNoChild || r < 0 || (size_t)r >= nn) return fail(CRT_CUDA_ERROR, "inconsistent tree");
      n3[3 * i + 1 + c] = r;
      const float box[6] = {q.lo_code.x, q.lo_code.y, q.lo_code.z, q.hi.x, q.hi.y, q.hi.z};
      std::memcpy(&nb[6 * (size_t)r], box, sizeof(box));
    }
  }
  std::memcpy(&nb[0], g.root_box, 6 * sizeof(float));
  float box[6];
  for (int k = 0; k < 3; k++) box[k] = ord2f_h(g.bmin[k]), box[3 + k] = ord2f_h(g.bmax[k]);
  std::vector<int32_t> ids_local(n);
  for (int k = 0; k < n; k++) ids_local[k] = (int32_t)hv[k] - t0;
  auto put = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    return (dst && bytes) ? cudaMemcpy(dst, src, bytes, cudaMemcpyDefault) : cudaSuccess;
  };
  CRT_CUDA(put(scene_box, box, sizeof(box)), "export");
  CRT_CUDA(put(codes, hk.data(), 4 * (size_t)n), "export");
  CRT_CUDA(put(ids, ids_local.data(), 4 * (size_t)n), "export");
  CRT_CUDA(put(nodes3, n3.data(), 4 * n3.size()), "export");
  CRT_CUDA(put(node_boxes, nb.data(), 4 * nb.size()), "export");
  return CRT_OK;
}

}  // extern "C"

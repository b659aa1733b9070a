// harness.cpp -- drives the reference's own device code on the CPU.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle).  build_ref.py compiles this
// file together with the reference's kernel sources (device functions taken
// as they are in the reference checkout, host launch wrappers left out) into
// oracle/_ref/libcrtref.so.  The harness plays the role of the host code the
// reference would run: it allocates the arrays, "launches" each __global__
// function as a loop over simulated blocks and threads, and reads back.
//
// Exported functions mirror crt_oracle.cpp's (ref_* for orc_*), so the tests
// can check the restatement against the reference itself.
#define private public  // BVH_d keeps its arrays private (inc/bvh.cuh:32-49)
#include "scene.h"
#include "Light.h"
#include "camera.h"
#include "bvh.cuh"
#undef private

#include <algorithm>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

// Kernels defined in the reference sources (same signatures as there).
void computeBoundingBoxes_kernel(int numTriangles, Vec3d* vertices, TriangleIndices* t_indices, BoundingBox* BBoxs);
void computeMortonCodesKernel(int* mortonCodes, unsigned int* object_ids, BoundingBox* BBoxs,
                              TriangleIndices* t_indices, Vec3d* vertices, int numTriangles, Vec3d mMin, Vec3d mMax);
void BuildHierarchy(int* mortoncodes, BoundingBox* bounds, unsigned int* indices, int numprims, HNode* nodes,
                    BoundingBox* boundssorted, int* flags);
void RefitBounds(BoundingBox* bounds, int numprims, HNode* nodes, int* flags);
void runRayTracerKernelRec(Scene_d* scene, int depth);
void initLight(Scene_d* scene, Light_h hostLight, Light* light);
void AverageSuperSamplingKernel(Vec3d* smallImage, Vec3d* deviceImage, int imageWidth, int imageHeight,
                                int superSampling);

// Definitions the reference keeps in host files that are not compiled here
// (src/scene.cpp:163-171, src/bvh.cpp:35-41).  The harness owns the memory.
Scene_d::~Scene_d() {}
BVH_d::~BVH_d() {}

namespace {

// Run a 1-D kernel body over `n` simulated threads, blocks of `bs`,
// one simulated thread after another.
template <class F>
void launch1d(int n, int bs, F body) {
  gridDim = dim3((n + bs - 1) / bs);
  blockDim = dim3(bs);
  for (unsigned b = 0; b < gridDim.x; b++)
    for (unsigned t = 0; t < (unsigned)bs; t++) {
      blockIdx = make_uint3(b, 0, 0);
      threadIdx = make_uint3(t, 0, 0);
      body();
    }
}

struct RefScene {
  std::vector<Vec3d> verts, normals;
  std::vector<TriangleIndices> tidx;
  std::vector<int> matid;
  std::vector<Material> mats;
  std::vector<BoundingBox> bbox;
  Vec3d mMin, mMax;
  std::vector<int> codes_unsorted, codes, flags;
  std::vector<unsigned> ids;
  std::vector<HNode> nodes;
  std::vector<BoundingBox> sorted;
  Scene_d sd;
  int n = 0;
};

// The upload + build sequence of Scene_d::operator= (src/scene.cpp:82-160)
// and BVH_d::setUp (src/bvh.cpp:3-32), minus the device allocations.
void build(RefScene& s) {
  const int n = s.n;
  s.bbox.assign(n, BoundingBox());
  launch1d(n, 256, [&] { computeBoundingBoxes_kernel(n, s.verts.data(), s.tidx.data(), s.bbox.data()); });
  // findMinMax (kernels/scene.cu:72-85): thrust::transform_reduce of the
  // reference's minimum/maximum from (+1e9)/(-1e9).
  Vec3d mn(1e9, 1e9, 1e9), mx(-1e9, -1e9, -1e9);
  for (int i = 0; i < n; i++) {
    mn = minimum(mn, s.bbox[i].bmin);
    mx = maximum(mx, s.bbox[i].bmax);
  }
  s.mMin = mn;
  s.mMax = mx;
  s.codes.assign(n, 0);
  s.ids.assign(n, 0);
  launch1d(n, 256, [&] {
    computeMortonCodesKernel(s.codes.data(), s.ids.data(), s.bbox.data(), s.tidx.data(), s.verts.data(), n, mn, mx);
  });
  s.codes_unsorted = s.codes;
  // thrust::sort_by_key (kernels/bvh.cu:267-273) is a stable ascending sort
  // of (code, id); thrust is not part of the reference checkout.
  std::vector<std::pair<int, unsigned>> kv(n);
  for (int i = 0; i < n; i++) kv[i] = {s.codes[i], s.ids[i]};
  std::stable_sort(kv.begin(), kv.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  for (int i = 0; i < n; i++) s.codes[i] = kv[i].first, s.ids[i] = kv[i].second;
  const int nn = n > 0 ? 2 * n - 1 : 0;
  HNode zero{-1, 0, 0, 0};
  s.nodes.assign(nn, zero);
  s.sorted.assign(nn, BoundingBox());
  s.flags.assign(n > 1 ? n - 1 : 1, 0);
  launch1d(n, 256, [&] {
    BuildHierarchy(s.codes.data(), s.bbox.data(), s.ids.data(), n, s.nodes.data(), s.sorted.data(), s.flags.data());
  });
  // With one triangle RefitBounds would follow the root's unwritten parent.
  if (n >= 2) launch1d(n, 256, [&] { RefitBounds(s.sorted.data(), n, s.nodes.data(), s.flags.data()); });
  s.sd.bvh.mortonCodes = s.codes.data();
  s.sd.bvh.object_ids = s.ids.data();
  s.sd.bvh.nodes = s.nodes.data();
  s.sd.bvh.sortedBBoxs = s.sorted.data();
  s.sd.bvh.flags = s.flags.data();
  s.sd.bvh.numTriangles = n;
  s.sd.bvh.vertices = s.verts.data();
  s.sd.bvh.normals = s.normals.data();
  s.sd.bvh.BBoxs = s.bbox.data();
  s.sd.bvh.t_indices = s.tidx.data();
  s.sd.bvh.materials = s.mats.data();
  s.sd.bvh.material_ids = s.matid.data();
}

}  // namespace

extern "C" {

struct ref_material {  // same layout as orc_material
  double ka[3], kd[3], ks[3], kt[3], ke[3];
  double shininess;
};
struct ref_camera {  // same layout as orc_camera
  double fov, focal_point, fstop;
  double eye[3];
};
struct ref_light {  // same layout as orc_light
  double color[3], position[3];
  double radius, constant_term, linear_term, quadratic_term;
};

void* ref_scene_create(int nv, const float* verts, int nn, const float* normals, int ntri, const int* vidx,
                       const int* nidx, int nmat, const ref_material* mats, const int* matid) {
  RefScene* s = new RefScene;
  s->n = ntri;
  s->verts.resize(nv);
  for (int i = 0; i < nv; i++) s->verts[i] = Vec3d(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  s->normals.resize(nn);
  for (int i = 0; i < nn; i++) s->normals[i] = Vec3d(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
  s->tidx.resize(ntri);
  for (int t = 0; t < ntri; t++) {
    index_t* c[3] = {&s->tidx[t].a, &s->tidx[t].b, &s->tidx[t].c};
    for (int k = 0; k < 3; k++) {
      c[k]->vertex_index = vidx[3 * t + k];
      c[k]->normal_index = nidx ? nidx[3 * t + k] : vidx[3 * t + k];
      c[k]->texcoord_index = -1;
    }
  }
  s->matid.resize(ntri);
  for (int t = 0; t < ntri; t++) s->matid[t] = matid ? matid[t] : 0;
  // Material set-up as in Scene_h::LoadObj (src/scene.cpp:22-37).
  s->mats.resize(nmat);
  for (int m = 0; m < nmat; m++) {
    Material& M = s->mats[m];
    M.ka = Vec3d((double*)mats[m].ka);
    M.kd = Vec3d((double*)mats[m].kd);
    M.ks = Vec3d((double*)mats[m].ks);
    M.kt = Vec3d((double*)mats[m].kt);
    M.ke = Vec3d((double*)mats[m].ke);
    M.kr = M.ks;
    M.shininess = mats[m].shininess;
    M.ior = 1.0;
    M.dissolve = 1.0;
    M.setBools();
  }
  build(*s);
  return s;
}

void ref_scene_destroy(void* h) { delete (RefScene*)h; }

// Returns 0 if every exported box value is a float (as it must be), else 1.
int ref_export(void* h, double* smin3, double* smax3, int* codes_unsorted, int* codes, unsigned* ids, int* nodes3,
               float* node_boxes, float* tri_boxes) {
  RefScene* s = (RefScene*)h;
  const int n = s->n, nn = n > 0 ? 2 * n - 1 : 0;
  int bad = 0;
  if (smin3) smin3[0] = s->mMin.x, smin3[1] = s->mMin.y, smin3[2] = s->mMin.z;
  if (smax3) smax3[0] = s->mMax.x, smax3[1] = s->mMax.y, smax3[2] = s->mMax.z;
  if (codes_unsorted) std::memcpy(codes_unsorted, s->codes_unsorted.data(), n * sizeof(int));
  if (codes) std::memcpy(codes, s->codes.data(), n * sizeof(int));
  if (ids) std::memcpy(ids, s->ids.data(), n * sizeof(unsigned));
  auto put = [&](float* dst, const BoundingBox& b) {
    double v[6] = {b.bmin.x, b.bmin.y, b.bmin.z, b.bmax.x, b.bmax.y, b.bmax.z};
    for (int k = 0; k < 6; k++) {
      dst[k] = (float)v[k];
      if ((double)dst[k] != v[k]) bad = 1;
    }
  };
  for (int i = 0; i < nn; i++) {
    if (nodes3) {
      nodes3[3 * i] = (i == 0) ? -1 : s->nodes[i].parent;
      nodes3[3 * i + 1] = s->nodes[i].left;
      nodes3[3 * i + 2] = s->nodes[i].right;
    }
    if (node_boxes) put(node_boxes + 6 * i, s->sorted[i]);
  }
  if (tri_boxes)
    for (int i = 0; i < n; i++) put(tri_boxes + 6 * i, s->bbox[i]);
  return bad;
}

// BVH_d::intersect / BVH_d::intersectAny on n rays (6 doubles each).
void ref_trace(void* h, const double* rays, int n, int any, int* ids, double* t, double* normal3, int nthreads) {
  RefScene* s = (RefScene*)h;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (int i = 0; i < n; i++) {
    const double* r = rays + 6 * (size_t)i;
    ray R(Vec3d(r[0], r[1], r[2]), Vec3d(r[3], r[4], r[5]));
    isect is;
    bool hit = (s->n > 0) && (any ? s->sd.bvh.intersectAny(R, is) : s->sd.bvh.intersect(R, is));
    ids[i] = hit ? is.object_id : -1;
    if (t) t[i] = hit ? is.t : 0.0;
    if (normal3 && hit && !any) normal3[3 * i] = is.N.x, normal3[3 * i + 1] = is.N.y, normal3[3 * i + 2] = is.N.z;
  }
}

// RayTracer::run (kernels/raytracer.cu:55-92) for the 16x16-block rows that
// cover [row0, row1), then AverageSuperSampling (SS = 1) and
// pullRaytracedImage's quantisation (inc/raytracer.h:53-63).  The reference
// kernel always takes 20 samples per pixel (raytracer.cu:138).  Outputs use
// the reference's memory order (idx = (H-py-1)*W + px) for rows in range.
void ref_render(void* h, const ref_camera* cam, const ref_light* light, int W, int H, int row0, int row1,
                unsigned char* rgb8, double* color, int nthreads) {
  RefScene* s = (RefScene*)h;
  Camera camera;  // Camera() (kernels/camera.cu:9-22), then main.cpp's setters
  camera.setfov(cam->fov);
  camera.setFstop(cam->fstop);
  camera.setFocalPoint(cam->focal_point);
  camera.setEye(Vec3d(cam->eye[0], cam->eye[1], cam->eye[2]));
  Light_h hl;
  hl.color = Vec3d(light->color[0], light->color[1], light->color[2]);
  hl.position = Vec3d(light->position[0], light->position[1], light->position[2]);
  hl.radius = light->radius;
  hl.constantTerm = light->constant_term;
  hl.linearTerm = light->linear_term;
  hl.quadraticTerm = light->quadratic_term;
  std::vector<Vec3d> image((size_t)W * H);
  std::vector<uint32_t> seeds((size_t)256 * ((W + 15) / 16) * ((H + 15) / 16));
  Scene_d& sd = s->sd;
  sd.numVertices = (int)s->verts.size();
  sd.imageWidth = W;
  sd.imageHeight = H;
  sd.numTriangles = s->n;
  sd.numMaterials = (int)s->mats.size();
  sd.vertices = s->verts.data();
  sd.normals = s->normals.data();
  sd.texcoords = nullptr;
  sd.materials = s->mats.data();
  sd.material_ids = s->matid.data();
  sd.BBoxs = s->bbox.data();
  sd.t_indices = s->tidx.data();
  sd.image = image.data();
  sd.camera = &camera;
  sd.seeds = seeds.data();
  Light light_obj(&sd, Vec3d(1, 1, 1));
  blockIdx = make_uint3(0, 0, 0);
  threadIdx = make_uint3(0, 0, 0);
  initLight(&sd, hl, &light_obj);  // initLight<<<1,1>>> (raytracer.cu:70)
  const int gx = (W + 15) / 16, gy = (H + 15) / 16;
  const int by0 = row0 / 16, by1 = (row1 + 15) / 16;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
#endif
  for (int by = by0; by < by1; by++)
    for (int bx = 0; bx < gx; bx++) {
      gridDim = dim3(gx, gy);
      blockDim = dim3(16, 16);
      for (int ty = 0; ty < 16; ty++)
        for (int tx = 0; tx < 16; tx++) {
          blockIdx = make_uint3(bx, by, 0);
          threadIdx = make_uint3(tx, ty, 0);
          runRayTracerKernelRec(&sd, 1);
        }
    }
  // AverageSuperSamplingKernel maps buffer index r*W + c to itself; pixel
  // (px, py) lives at buffer row r = H - py - 1.
  std::vector<Vec3d> small((size_t)W * H);
  for (int py = row0; py < row1; py++)
    for (int px = 0; px < W; px++) {
      const int r = H - py - 1;
      gridDim = dim3(gx, gy);
      blockDim = dim3(16, 16);
      blockIdx = make_uint3(px / 16, r / 16, 0);
      threadIdx = make_uint3(px % 16, r % 16, 0);
      AverageSuperSamplingKernel(small.data(), image.data(), W, H, 1);
    }
  for (int py = row0; py < row1; py++)
    for (int px = 0; px < W; px++) {
      size_t idx = (size_t)(H - py - 1) * W + px;
      if (color) color[3 * idx] = image[idx].x, color[3 * idx + 1] = image[idx].y, color[3 * idx + 2] = image[idx].z;
      if (rgb8) {
        rgb8[3 * idx + 0] = (unsigned char)(255.0 * small[idx].x);
        rgb8[3 * idx + 1] = (unsigned char)(255.0 * small[idx].y);
        rgb8[3 * idx + 2] = (unsigned char)(255.0 * small[idx].z);
      }
    }
}

int ref_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"

// trace.cu -- traversal and the pixel kernel on sm_103a.
//
// k_trace<ANY>  closest hit (BVH_d::intersect) or first hit in left-first
//               DFS order (BVH_d::intersectAny) for a batch of double rays.
// k_pixels      runRayTracerKernelRec (kernels/raytracer.cu:95-166) with
//               traceRay (raytracer.cu:169-249), Material::shade
//               (kernels/material.cu:6-40) and the positional Light
//               (kernels/Light.cu:5-86); also its adjoint.  Persistent: each
//               warp claims tiles of 32 / G pixels (G lanes per pixel), first
//               from its SM's rectangle of the image, then from the others;
//               a pixel's lanes trace its samples in waves, speculating on
//               how the mrand stream couples them (a hit consumes three
//               extra draws).
#include <cmath>

#include "pixel.cuh"

namespace crt {

namespace {

template <bool ANY>
__global__ void __launch_bounds__(128) k_trace(DScene S, const double* __restrict__ rays, int64_t n,
                                               int* __restrict__ ids, double* __restrict__ tout,
                                               double* __restrict__ nout) {
  float rb[6], B, D;
  scene_consts(S, rb, B, D);
  const int lane = threadIdx.x & 31;
  // warp-uniform loop (the traversal is warp-synchronous): lanes past n ride along
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
    const int64_t i = base + lane;
    const bool live = i < n;
    RayC rc;
    if (live) {
      const double* r = rays + 6 * i;
      ray_setup(rc, r[0], r[1], r[2], r[3], r[4], r[5], B, D);
    } else {
      ray_setup(rc, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, B, D);
    }
    HitRec h;
    const int res = traverse<ANY>(S, rc, rb, h, live);
    if (res < 0) atomicOr(&S.g->err, kErrStack);
    if (!live) continue;
    const bool hit = res > 0;
    ids[i] = hit ? h.id : -1;
    if (tout) tout[i] = hit ? h.t : 0.0;
    if (!ANY && nout && hit) {
      const D3 N = hit_normal(S, h);
      nout[3 * i] = N.x, nout[3 * i + 1] = N.y, nout[3 * i + 2] = N.z;
    }
  }
}

// One scene: warps claim tiles of 32 / G pixels of rows [row0, row1).
// SHORT: traversal-stack entries kept in shared memory per thread.
constexpr int kPixelsShort = 0;
template <int MODE>
__global__ void __launch_bounds__(128, 9) k_pixels(DScene S, RenderArgs A) {
  extern __shared__ int2 s_ring[];
  int2* ring = kPixelsShort > 0 ? s_ring + threadIdx.x : nullptr;
  TravStats ts;
  D3 glight = d3(0, 0, 0);
  float rb[6], B, D;
  scene_consts(S, rb, B, D);
  const int lane = threadIdx.x & 31;
  const int G = A.group, tw = group_tile_w(G), th = group_tile_h(G);
  const int tiles_x = (A.W + tw - 1) / tw;
  const int tiles_y = (A.row1 - A.row0 + th - 1) / th;
  const int p = lane / G;  // this lane's pixel in the tile
  unsigned pred = 0xffffffffu;
  int region = home_region(A.regions_x, A.regions_y);
  bool home = true;
  while (true) {
    int tile = 0;
    if (lane == 0) tile = claim_tile(A.counter, tiles_x, tiles_y, A.regions_x, A.regions_y, region, home);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile < 0) break;
    const int px = (tile % tiles_x) * tw + (p % tw);
    const int py = A.row0 + (tile / tiles_x) * th + (p / tw);
    pixel<MODE, kPixelsShort>(S, A, px, py, px < A.W && py < A.row1, G, pred, rb, B, D, ts, glight, ring);
  }
  flush_stats<MODE>(A, ts, glight);
}

}  // namespace

template <int MODE>
static void launch_pixels(const DScene& S, const RenderArgs& a, cudaStream_t st) {
  const size_t smem = (size_t)kPixelsShort * 128 * sizeof(int2);
  int bps = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_pixels<MODE>, 128, smem);
  k_pixels<MODE><<<num_sms() * (bps > 0 ? bps : 1), 128, smem, st>>>(S, a);
}

cudaError_t set_tile_regions(RenderArgs& a, int tiles_x, int tiles_y, bool split, cudaStream_t st) {
  int rx = 1, ry = 1;
  const int R = min(num_sms(), kMaxTileRegions - 1);
  if (split && (int64_t)tiles_x * tiles_y >= (int64_t)kMinTilesPerRegion * R) {
    const double aspect = (double)max(tiles_x, 1) / (double)max(tiles_y, 1);
    rx = (int)(std::sqrt(R * aspect) + 0.5);
    rx = max(1, min(rx, min(R, tiles_x)));
    ry = max(1, min((R + rx - 1) / rx, tiles_y));
    while (rx * ry > kMaxTileRegions - 1) ry--;
  }
  a.regions_x = rx, a.regions_y = ry;
  return cudaMemsetAsync(a.counter, 0, sizeof(unsigned) * (size_t)(rx * ry + 1), st);
}

cudaError_t launch_render(const DScene& S, const RenderArgs& a0, cudaStream_t st) {
  RenderArgs a = a0;
  const int tw = group_tile_w(a.group), th = group_tile_h(a.group);
  cudaError_t e = set_tile_regions(a, (a.W + tw - 1) / tw, (a.row1 - a.row0 + th - 1) / th, true, st);
  if (e != cudaSuccess) return e;
  if (a.grad_rgb)
    launch_pixels<kAdjoint>(S, a, st);
  else if (a.stats)
    launch_pixels<kRenderStats>(S, a, st);
  else
    launch_pixels<kRender>(S, a, st);
  return cudaGetLastError();
}

cudaError_t launch_trace(const DScene& S, const double* rays, int64_t n, bool any, int* ids, double* t,
                         double* normals, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int bps = 0;
  if (any)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_trace<true>, 128, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_trace<false>, 128, 0);
  if (bps <= 0) bps = 1;
  const int64_t need = (n + 127) / 128;
  const int grid = (int)(need < (int64_t)num_sms() * bps ? need : (int64_t)num_sms() * bps);
  if (any)
    k_trace<true><<<grid, 128, 0, st>>>(S, rays, n, ids, t, nullptr);
  else
    k_trace<false><<<grid, 128, 0, st>>>(S, rays, n, ids, t, normals);
  return cudaGetLastError();
}

}  // namespace crt

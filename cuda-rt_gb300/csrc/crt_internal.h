// crt_internal.h -- host-side interfaces between the library's translation
// units (build.cu, trace.cu, capi.cu).  Not part of the public ABI.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "crt_device.cuh"

namespace crt {

// Sort geometry shared by the build and the standalone sort.
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kRadixBits = 10;
constexpr int kRadix = 1 << kRadixBits;

inline int sort_passes(int key_bits) { return (key_bits + kRadixBits - 1) / kRadixBits; }
// Tiles of the small shape: an upper bound on the tiles of a pass, for sizing.
inline int sort_tiles(int n) { return (n + kSortTile - 1) / kSortTile; }
// From 2^19 keys on, passes use 8192-key tiles of 1024 threads.
constexpr int kSortThreadsL = 1024;
constexpr int kSortTileL = kSortThreadsL * kSortItems;
inline bool sort_large(int n) { return n >= (1 << 19); }
inline int sort_tiles_used(int n) { return sort_large(n) ? (n + kSortTileL - 1) / kSortTileL : sort_tiles(n); }

// Leaves per block of the refit (a node whose leaf range crosses a multiple
// of it is a spanning node).
constexpr int kRefitBlock = 512;
// Refit blocks per group (the spanning-node pass reads a whole group's box at once).
constexpr int kSpanGroup = 32;
inline size_t refit_blocks(int n) { return n > 0 ? ((size_t)n + kRefitBlock - 1) / kRefitBlock : 1; }
inline size_t span_groups(int n) { return (refit_blocks(n) + kSpanGroup - 1) / kSpanGroup; }

// Device arrays of one scene's BVH build (owned by the scene).
struct BuildBufs {
  int n = 0;
  uint32_t *keys_a = nullptr, *keys_b = nullptr, *vals_a = nullptr, *vals_b = nullptr;
  uint32_t* hist = nullptr;    // 3 * kRadix
  uint32_t* status = nullptr;  // 3 * tiles * kRadix
  uint32_t* parent = nullptr;  // 2n - 1: parent index (reference numbering) | left-child and spanning bits
  uint4* spans = nullptr;      // n: the spanning internal nodes (node, first leaf, last leaf, parent word)
  float* suf = nullptr;        // 6n: box of leaves i..end of i's refit block (at first leaves of block tops;
                               // at a block's first leaf: the block's box)
  float* pre = nullptr;        // 6n: box of leaves start of i's refit block..i (at last leaves of block tops)
  int* gbox = nullptr;         // 6 per group of kSpanGroup refit blocks: the group's box (order-preserving ints)
  WNode* wnodes = nullptr;     // n (the last one virtual: the root's children)
  LeafTri* leaves = nullptr;   // n
  SceneGlobals* g = nullptr;
};

// Mesh arrays on the device.
struct MeshBufs {
  int nv = 0, nn = 0, ntri = 0, nmat = 0;
  float* verts = nullptr;
  float* normals = nullptr;
  int* vidx = nullptr;
  int* nidx = nullptr;
  int* matid = nullptr;
  DMat* mats = nullptr;
};

// Many meshes in concatenated arrays (see batch_kernel.cuh).
struct BatchBufs {
  int M = 0, N = 0, NI = 0;  // meshes, triangles, internal nodes (N - M)
  const float* verts = nullptr;
  const int* vidx = nullptr;  // global vertex indices
  const int* mesh_of = nullptr;
  const int* tri_off = nullptr;  // M + 1
  uint32_t *keys_a = nullptr, *keys_b = nullptr, *vals_a = nullptr, *vals_b = nullptr, *codes0 = nullptr;
  uint32_t* hist = nullptr;    // 4 * kRadix
  uint32_t* status = nullptr;  // 4 * tiles * kRadix
  uint32_t* parent = nullptr;  // NI + N
  int* flags = nullptr;        // NI
  WNode* wnodes = nullptr;     // NI + M (codes local to each mesh; NI + m: mesh m's virtual node)
  LeafTri* leaves = nullptr;   // N
  SceneGlobals* g = nullptr;   // M
  unsigned* counters = nullptr;  // [0..3] sort tiles, [4] render items, [6] refit hand-offs (8 words)
  uint2* arrivals = nullptr;     // N: climbs handed from the refit to its spanning-node pass
  int* err = nullptr;
};

int num_sms();

// build.cu
cudaError_t launch_build(const MeshBufs& m, const BuildBufs& b, cudaStream_t st);
cudaError_t launch_refit(const MeshBufs& m, const BuildBufs& b, cudaStream_t st);
// Stage-level hierarchy and refit in the reference's HNode layout (scratch:
// parent 2n - 1 words and wnodes n for the hierarchy; for the refit, flags
// n - 1 zeroed by the caller).
cudaError_t launch_stage_hierarchy(const uint32_t* codes, const uint32_t* ids, int n, int* nodes3,
                                   uint32_t* parent, WNode* wnodes, cudaStream_t st);
cudaError_t launch_stage_refit(const float* V, int nv, const int* vidx, int n, const uint32_t* ids,
                               const int* nodes3, float* boxes, int* flags, int* err, cudaStream_t st);
// Range checks of device-resident index arrays (kErrIndex in b.g->err).
cudaError_t launch_check_indices(const MeshBufs& m, const BuildBufs& b, cudaStream_t st);
cudaError_t launch_morton(const float* verts, int nv, const int* vidx, int n, const float* box6, uint32_t* codes,
                          int* err, cudaStream_t st);
// Stable LSD radix sort; scratch holds sort_scratch_bytes(n, key_bits).
size_t sort_scratch_bytes(int n, int key_bits);
// Argument check shared by crt_sort_pairs and crt_sort_pairs_noalloc (n > 0):
// every array in device memory of the current device, and no input array
// overlapping an output array, nor the two outputs each other (pass 0 of a
// multi-pass sort writes an output while later tiles still read the input).
// Returns NULL when the arguments are usable, else what is wrong.
const char* sort_args_problem(const uint32_t* kin, const uint32_t* vin, const uint32_t* kout, const uint32_t* vout,
                              int n);
cudaError_t launch_sort_pairs(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, int n,
                              int key_bits, void* scratch, int* err, cudaStream_t st);

// trace.cu
// The pixel kernels give each pixel G lanes (a power of two, at most 32 and
// at most spp rounded down to a power of two), so a warp covers 32 / G
// pixels, laid out as a tile_w(G) x tile_h(G) block (8x4, 8x2, 4x2, 2x2,
// 2x1, 1x1: the most compact, for coherent rays).
__host__ __device__ inline int lanes_per_pixel(int spp, int gmax) {
  int g = 1;
  while (2 * g <= spp && 2 * g <= gmax && g < 32) g *= 2;
  return g;
}
__host__ __device__ inline int group_tile_w(int G) { return 32 / G >= 16 ? 8 : (32 / G >= 4 ? 32 / G / 2 : 32 / G); }
__host__ __device__ inline int group_tile_h(int G) { return (32 / G) / group_tile_w(G); }
constexpr int kDefaultLanesPerPixel = 4;

// The persistent pixel kernels split the image's tiles into regions_x x
// regions_y rectangles, about one per SM: a warp takes tiles from its SM's
// rectangle (so the warps sharing an SM's L1 trace neighbouring rays), then
// helps the others (claim_tile).  One counter per rectangle and one bound;
// images of fewer than kMinTilesPerRegion tiles per SM keep one rectangle.
constexpr int kMaxTileRegions = 2048;
constexpr int kMinTilesPerRegion = 256;

struct RenderArgs {
  int W, H, spp, row0, row1;
  int group;  // lanes per pixel (lanes_per_pixel)
  int regions_x = 1, regions_y = 1;  // tile rectangles (set_tile_regions); counter holds one word per rectangle
  double angle, aspect, invW, invH, aperture, focal;
  double eye[3];
  double lpos[3], lcol[3], lradius, latt[3];
  uint8_t* rgb8;
  float* rgbf;
  int* hit_id;
  double* hit_t;
  int* shadow;
  double* rays;
  unsigned* counter;
  unsigned long long* stats;  // optional [2]: internal nodes visited, triangles tested
  double* rgbd = nullptr;     // optional: mean colour in double
  double* depth = nullptr;    // optional: mean hit t (misses count 0)
  int* shadow_id = nullptr;   // optional: occluding triangle per sample, -1 if none
  uint32_t seed_mix = 0;             // XORed into each pixel's hash input (0: parity)
  const double2* lens_cs = nullptr;  // optional lens tables (lens.cu)
  const double* lens_sqrt = nullptr;
  // adjoint (grad_rgb != NULL selects it)
  const double* grad_rgb = nullptr;
  const double* grad_depth = nullptr;
  double* grad_verts = nullptr;
  double* grad_light = nullptr;
  double* grad_albedo = nullptr;
};
cudaError_t launch_render(const DScene& S, const RenderArgs& a, cudaStream_t st);

// The tile rectangles for a tiles_x x tiles_y grid of tiles: with split and a
// large enough image about num_sms() of them, near square, else one; their
// counters and bound zeroed on st.
cudaError_t set_tile_regions(RenderArgs& a, int tiles_x, int tiles_y, bool split, cudaStream_t st);

// lens.cu: the thin-lens tables of the current device (built on first use
// when enabled and memory allows; otherwise both NULL, and the kernels
// compute the same values inline).
struct LensTables {
  const double2* cs = nullptr;
  const double* sq = nullptr;
};
LensTables lens_tables(cudaStream_t st);

// recursive.cu: traceRay with reflected and refracted rays, at most
// kMaxRecDepth levels below the primary ray.  optics[m] (device, may be
// NULL): kr and ior of material m.
constexpr int kMaxRecDepth = 8;
struct DOptics {
  double kr[3];
  double ior;
};
cudaError_t launch_render_recursive(const DScene& S, const RenderArgs& a, const DOptics* optics, int depth,
                                    cudaStream_t st);

// Device view of a batch for the batched pixel kernel.
struct BatchView {
  int M = 0, items = 0;
  const int* item_off = nullptr;  // M + 1: first work item (pixel tile) of each mesh
  const int* tri_off = nullptr;   // M + 1
  const float* verts = nullptr;
  const float* normals = nullptr;
  const int* vidx = nullptr;
  const int* nidx = nullptr;
  const int* matid = nullptr;
  const DMat* mats = nullptr;
  const WNode* wnodes = nullptr;
  const LeafTri* leaves = nullptr;
  SceneGlobals* g = nullptr;
  const RenderArgs* args = nullptr;  // M
  unsigned* counter = nullptr;
};
struct BatchTuning {
  int block = 256, lanes = kDefaultLanesPerPixel, stack = 0;  // lanes: the most lanes a pixel may take
  int launches = 2;  // 1: build and render in one launch; 2: the render in a launch of its own
};
cudaError_t launch_trace(const DScene& S, const double* rays, int64_t n, bool any, int* ids, double* t,
                         double* normals, cudaStream_t st);

}  // namespace crt

// build.cu -- the LBVH build on sm_103a.
//
// Stages (reference: Scene_d::operator= and BVH_d::setUp, src/scene.cpp:82-160,
// src/bvh.cpp:3-32):
//   k_build_init   reset the per-scene globals and sort histograms
//   k_bounds       triangle AABBs reduced to the scene box (findMinMax)
//   k_morton       30-bit Morton codes + the digit histograms of all sort passes
//   k_onesweep x3  stable LSD radix sort, 10-bit digits, decoupled look-back
//   k_hierarchy    Karras split search, one thread per internal node
//   k_refit        atomic bottom-up refit, one climber per leaf; it also
//                  writes the leaf triangles in sorted order for traversal
// Triangle boxes are never stored: each stage that needs one recomputes it
// from the three vertices (L2-resident for the sizes this targets).
#include <cstdio>

#include "crt_internal.h"

namespace crt {

namespace {

constexpr int kSpinLimit = 1 << 20;  // bounded look-back wait (x ~64 ns)

__device__ __forceinline__ void tri_box(const float* __restrict__ V, const int* __restrict__ vidx, int t,
                                        float3& a, float3& b, float3& c, float lo[3], float hi[3]) {
  const int ia = __ldg(vidx + 3 * t), ib = __ldg(vidx + 3 * t + 1), ic = __ldg(vidx + 3 * t + 2);
  a = make_float3(__ldg(V + 3 * ia), __ldg(V + 3 * ia + 1), __ldg(V + 3 * ia + 2));
  b = make_float3(__ldg(V + 3 * ib), __ldg(V + 3 * ib + 1), __ldg(V + 3 * ib + 2));
  c = make_float3(__ldg(V + 3 * ic), __ldg(V + 3 * ic + 1), __ldg(V + 3 * ic + 2));
  // computeTriangleBoundingBox (kernels/scene.cu:120-130) through
  // minimum/maximum (fminf/fmaxf): exact on float inputs.
  lo[0] = fminf(c.x, fminf(a.x, b.x)), hi[0] = fmaxf(c.x, fmaxf(a.x, b.x));
  lo[1] = fminf(c.y, fminf(a.y, b.y)), hi[1] = fmaxf(c.y, fmaxf(a.y, b.y));
  lo[2] = fminf(c.z, fminf(a.z, b.z)), hi[2] = fmaxf(c.z, fmaxf(a.z, b.z));
}

// Every coordinate finite and |x| <= 1e37 (fminf/fmaxf would hide a NaN
// inside the box, so the vertices themselves are checked).
__device__ __forceinline__ bool finite_coords(float3 a, float3 b, float3 c) {
  const float m = fmaxf(fmaxf(fmaxf(fabsf(a.x), fabsf(a.y)), fmaxf(fabsf(a.z), fabsf(b.x))),
                        fmaxf(fmaxf(fabsf(b.y), fabsf(b.z)), fmaxf(fmaxf(fabsf(c.x), fabsf(c.y)), fabsf(c.z))));
  const bool nan = (a.x != a.x) | (a.y != a.y) | (a.z != a.z) | (b.x != b.x) | (b.y != b.y) | (b.z != b.z) |
                   (c.x != c.x) | (c.y != c.y) | (c.z != c.z);
  return !nan && m <= 1e37f;
}

__global__ void k_build_init(SceneGlobals* g, uint32_t* hist, int nhist) {
  const int t = threadIdx.x;
  if (t < 3) {
    g->bmin[t] = f2ord(1e9f);  // findMinMax's initial values (kernels/scene.cu:75,80)
    g->bmax[t] = f2ord(-1e9f);
  }
  if (t == 0) {
    g->emax = f2ord(0.f);
    g->err = 0;
  }
  if (t < 4) g->tile_counter[t] = 0;
  for (int i = t; i < nhist; i += blockDim.x) hist[i] = 0;
}

// Scene bounds (kernels/scene.cu:72-85) and the largest triangle extent.
__global__ void __launch_bounds__(256) k_bounds(const float* __restrict__ V, const int* __restrict__ vidx, int n,
                                                SceneGlobals* g) {
  float lo[3] = {1e9f, 1e9f, 1e9f}, hi[3] = {-1e9f, -1e9f, -1e9f}, e = 0.f;
  bool ok = true;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    float3 a, b, c;
    float l[3], h[3];
    tri_box(V, vidx, t, a, b, c, l, h);
    ok = ok && finite_coords(a, b, c);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      lo[k] = fminf(lo[k], l[k]);
      hi[k] = fmaxf(hi[k], h[k]);
      e = fmaxf(e, h[k] - l[k]);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
    }
    e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, off));
  }
  const bool all_ok = __all_sync(0xffffffffu, ok);
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      atomicMin(&g->bmin[k], f2ord(lo[k]));
      atomicMax(&g->bmax[k], f2ord(hi[k]));
    }
    atomicMax(&g->emax, f2ord(e));
    if (!all_ok) atomicOr(&g->err, kErrNonFinite);
  }
}

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {  // ExpandBits, kernels/bvh.cu:13-21
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

// One axis of CalculateMortonCode (kernels/bvh.cu:25-27) on the normalised
// centroid p: (float)min(max(p*1024, 0), 1023) with NaN-ignoring max/min,
// truncated to unsigned.
__device__ __forceinline__ uint32_t morton_axis(double p) {
  double s = p * 1024.0;
  s = fmax(s, 0.0);
  s = fmin(s, 1023.0);
  return (uint32_t)__double2float_rn(s);
}

// computeMortonCodesKernel, kernels/bvh.cu:37-61, in double as the reference.
__device__ __forceinline__ uint32_t morton_code(const float lo[3], const float hi[3], const double mn[3],
                                                const double mx[3]) {
  uint32_t e[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double c = 0.5 * ((double)lo[k] + (double)hi[k]);
    c = (c - mn[k]) / (mx[k] - mn[k]);
    e[k] = expand_bits(morton_axis(c));
  }
  return e[0] * 4 + e[1] * 2 + e[2];
}

__device__ __forceinline__ void load_scene_box(const SceneGlobals* g, double mn[3], double mx[3]) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    mn[k] = (double)ord2f(g->bmin[k]);
    mx[k] = (double)ord2f(g->bmax[k]);
  }
}

// Morton codes + per-pass digit histograms; also clears the look-back status.
__global__ void __launch_bounds__(512) k_morton(const float* __restrict__ V, const int* __restrict__ vidx, int n,
                                                const SceneGlobals* g, uint32_t* __restrict__ keys,
                                                uint32_t* __restrict__ hist, int passes,
                                                uint32_t* __restrict__ status, int status_words) {
  __shared__ uint32_t sh[3 * kRadix];
  for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) sh[i] = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < status_words; i += gridDim.x * blockDim.x) status[i] = 0;
  double mn[3], mx[3];
  load_scene_box(g, mn, mx);
  __syncthreads();
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    float3 a, b, c;
    float lo[3], hi[3];
    tri_box(V, vidx, t, a, b, c, lo, hi);
    const uint32_t code = morton_code(lo, hi, mn, mx);
    keys[t] = code;
    for (int p = 0; p < passes; p++) atomicAdd(&sh[p * kRadix + ((code >> (p * kRadixBits)) & (kRadix - 1))], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// Standalone Morton codes against a given scene box (crt_morton).
__global__ void k_morton_only(const float* __restrict__ V, const int* __restrict__ vidx, int n,
                              const float* __restrict__ box6, uint32_t* __restrict__ keys) {
  double mn[3], mx[3];
#pragma unroll
  for (int k = 0; k < 3; k++) mn[k] = box6[k], mx[k] = box6[3 + k];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    float3 a, b, c;
    float lo[3], hi[3];
    tri_box(V, vidx, t, a, b, c, lo, hi);
    keys[t] = morton_code(lo, hi, mn, mx);
  }
}

// Digit histograms of arbitrary keys (standalone sort); clears the status.
__global__ void __launch_bounds__(512) k_key_hist(const uint32_t* __restrict__ keys, int n, uint32_t* __restrict__ hist,
                                                  int passes, uint32_t* __restrict__ status, int status_words) {
  __shared__ uint32_t sh[4 * kRadix];
  for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) sh[i] = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < status_words; i += gridDim.x * blockDim.x) status[i] = 0;
  __syncthreads();
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const uint32_t k = keys[t];
    for (int p = 0; p < passes; p++) atomicAdd(&sh[p * kRadix + ((k >> (p * kRadixBits)) & (kRadix - 1))], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

__global__ void k_zero_u32(uint32_t* p, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Exclusive scan over the block of one value per thread; returns the prefix.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* s_warp, uint32_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  uint32_t wpre = 0, tot = 0;
  for (int w = 0; w < kSortThreads / 32; w++) {
    const uint32_t s = s_warp[w];
    if (w < warp) wpre += s;
    tot += s;
  }
  __syncthreads();
  total = tot;
  return wpre + x - v;
}

constexpr uint32_t kFlagAgg = 1u << 30, kFlagInc = 2u << 30, kValMask = (1u << 30) - 1;

// One stable LSD pass over the digit at `shift` (thrust::sort_by_key's
// role, kernels/bvh.cu:267-273).  Tiles of 2048 keys are claimed in order
// from an atomic counter; within a tile, warps rank their 256 keys in input
// order with __match_any_sync, and the tile's digit offsets come from a
// decoupled look-back over the tiles before it.
__global__ void __launch_bounds__(kSortThreads) k_onesweep(const uint32_t* __restrict__ kin,
                                                           const uint32_t* __restrict__ vin,
                                                           uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           int n, int shift, const uint32_t* __restrict__ ghist,
                                                           uint32_t* __restrict__ status, unsigned* tile_counter,
                                                           int* err) {
  constexpr int W = kSortThreads / 32;
  __shared__ uint32_t s_whist[W][kRadix / 2];  // per-warp 16-bit digit counters
  __shared__ uint32_t s_tstart[kRadix];
  __shared__ uint32_t s_gbase[kRadix];
  __shared__ uint32_t s_keys[kSortTile];
  __shared__ uint32_t s_vals[kSortTile];
  __shared__ uint32_t s_warp[W];
  __shared__ int s_tile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = (int)atomicAdd(tile_counter, 1u);
  for (int i = tid; i < W * kRadix / 2; i += kSortThreads) (&s_whist[0][0])[i] = 0;
  // global start of each digit: exclusive scan of the pass histogram
  uint32_t gh[4], gsum = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) gh[j] = __ldg(ghist + 4 * tid + j), gsum += gh[j];
  uint32_t gtot;
  uint32_t gpre = block_excl_scan(gsum, s_warp, gtot);
  const int tile = s_tile;
  const int base = tile * kSortTile;
  const uint32_t mask = kRadix - 1;
  uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
  unsigned short* wh = reinterpret_cast<unsigned short*>(s_whist[warp]);
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int r = 0; r < kSortItems; r++) {
    const int idx = base + warp * (32 * kSortItems) + r * 32 + lane;
    const bool valid = idx < n;
    key[r] = valid ? __ldg(kin + idx) : 0u;
    val[r] = valid ? (vin ? __ldg(vin + idx) : (uint32_t)idx) : 0u;
    const uint32_t d = valid ? ((key[r] >> shift) & mask) : (uint32_t)kRadix;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const int leader = __ffs(peers) - 1;
    uint32_t b = 0;
    if (lane == leader && valid) {
      b = wh[d];
      wh[d] = (unsigned short)(b + __popc(peers));
    }
    b = __shfl_sync(0xffffffffu, b, leader);
    rank[r] = b + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();
  // per digit: warp offsets (exclusive, in place) and the tile count
  uint32_t cnt[4], csum = 0;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int d = 4 * tid + j;
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < W; w++) {
      unsigned short* h = reinterpret_cast<unsigned short*>(s_whist[w]) + d;
      const uint32_t x = *h;
      *h = (unsigned short)c;
      c += x;
    }
    cnt[j] = c;
    csum += c;
  }
  // publish this tile's counts, then look back for the prefix over earlier tiles
  uint32_t* my = status + (size_t)tile * kRadix;
#pragma unroll
  for (int j = 0; j < 4; j++) st_relaxed(my + 4 * tid + j, (tile == 0 ? kFlagInc : kFlagAgg) | cnt[j]);
  uint32_t pre[4] = {0, 0, 0, 0};
  if (tile > 0) {
#pragma unroll 1
    for (int j = 0; j < 4; j++) {
      const int d = 4 * tid + j;
      uint32_t acc = 0;
      for (int look = tile - 1; look >= 0; look--) {
        const uint32_t* p = status + (size_t)look * kRadix + d;
        uint32_t s = ld_relaxed(p);
        int spins = 0;
        while ((s & ~kValMask) == 0) {
          // bounded wait; once any wait has timed out, later ones give up at once
          if (++spins > kSpinLimit || ((spins & 1023) == 0 && (ld_relaxed((const uint32_t*)err) & kErrTimeout))) {
            atomicOr(err, kErrTimeout);
            s = kFlagInc;
            break;
          }
          __nanosleep(64);
          s = ld_relaxed(p);
        }
        acc += s & kValMask;
        if ((s & ~kValMask) == kFlagInc) break;
      }
      pre[j] = acc;
      st_relaxed(my + d, kFlagInc | (acc + cnt[j]));
    }
  }
  uint32_t ctot;
  uint32_t cpre = block_excl_scan(csum, s_warp, ctot);
  {
    uint32_t c = cpre, g = gpre;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int d = 4 * tid + j;
      s_tstart[d] = c;
      s_gbase[d] = g + pre[j] - c;
      c += cnt[j];
      g += gh[j];
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kSortItems; r++) {
    const int idx = base + warp * (32 * kSortItems) + r * 32 + lane;
    if (idx < n) {
      const uint32_t d = (key[r] >> shift) & mask;
      const uint32_t pos = s_tstart[d] + wh[d] + rank[r];
      s_keys[pos] = key[r];
      s_vals[pos] = val[r];
    }
  }
  __syncthreads();
  const int tile_n = min(kSortTile, n - base);
  for (int i = tid; i < tile_n; i += kSortThreads) {
    const uint32_t k = s_keys[i];
    const uint32_t pos = s_gbase[(k >> shift) & mask] + (uint32_t)i;
    kout[pos] = k;
    vout[pos] = s_vals[i];
  }
}

// delta(), kernels/bvh.cu:71-88 (i is always in range here).
__device__ __forceinline__ int kdelta(const uint32_t* __restrict__ c, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  const uint32_t a = __ldg(c + i), b = __ldg(c + j);
  return a != b ? __clz((int)(a ^ b)) : 32 + __clz(i ^ j);
}

// BuildHierarchy (kernels/bvh.cu:164-207) with FindSpan (bvh.cu:100-133) and
// FindSplit (bvh.cu:134-162): one thread per internal node writes its child
// codes, the children's parents, and clears the node's refit flag.
__global__ void __launch_bounds__(256) k_hierarchy(const uint32_t* __restrict__ codes, int n, BNode* __restrict__ nodes,
                                                   int* __restrict__ parent, int* __restrict__ flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int dd = kdelta(codes, n, i, i + 1) - kdelta(codes, n, i, i - 1);
  const int d = dd > 0 ? 1 : (dd < 0 ? -1 : 0);
  const int dmin = kdelta(codes, n, i, i - d);
  int lmax = 2;
  while (kdelta(codes, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0, t = lmax;
  do {
    t /= 2;
    if (kdelta(codes, n, i, i + (l + t) * d) > dmin) l += t;
  } while (t > 1);
  const int lo = min(i, i + l * d), hi = max(i, i + l * d);
  int left = lo, right = hi;
  const int same = kdelta(codes, n, left, right);
  do {
    const int s = (right + left) / 2;
    if (kdelta(codes, n, left, s) > same)
      left = s;
    else
      right = s;
  } while (right > left + 1);
  const int split = left;
  const int c1 = (split == lo) ? ~split : split;
  const int c2 = (split + 1 == hi) ? ~(split + 1) : split + 1;
  nodes[i].child = make_int4(c1, c2, 0, 0);
  parent[c1 < 0 ? (n - 1) + split : split] = i;
  parent[c2 < 0 ? (n - 1) + split + 1 : split + 1] = i;
  flags[i] = 0;
}

// RefitBounds (kernels/bvh.cu:209-258): one climber per leaf; at each node the
// first arrival stops and the second computes the union (bboxunion,
// bvh.cu:63-69) and climbs on.  Boxes are stored in the parent's child slot.
// Flags count arrivals; each refit adds exactly two per node, so the parity
// of the old value tells first from second without clearing between refits.
// Also writes the sorted leaf triangles and the largest triangle extent.
__global__ void __launch_bounds__(256) k_refit(const float* __restrict__ V, const int* __restrict__ vidx,
                                               const uint32_t* __restrict__ ids, int n, BNode* nodes,
                                               LeafTri* __restrict__ leaves, const int* __restrict__ parent,
                                               int* flags, SceneGlobals* g) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  float e = 0.f;
  bool ok = true;
  if (k < n) {
    const int tri = (int)__ldg(ids + k);
    float3 a, b, c;
    float lo[3], hi[3];
    tri_box(V, vidx, tri, a, b, c, lo, hi);
    ok = finite_coords(a, b, c);
    e = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    LeafTri lt;
    lt.v0 = make_float4(a.x, a.y, a.z, __int_as_float(tri));
    lt.v1 = make_float4(b.x, b.y, b.z, 0.f);
    lt.v2 = make_float4(c.x, c.y, c.z, 0.f);
    leaves[k] = lt;
    if (n == 1) {
#pragma unroll
      for (int q = 0; q < 3; q++) g->root_box[q] = lo[q], g->root_box[3 + q] = hi[q];
    } else {
      int code = ~k;
      int p = __ldg(parent + (n - 1) + k);
      // a valid tree is at most 59 levels deep (CRT_MAX_TRIANGLES); the
      // bound only guards against a corrupt parent chain
      for (int level = 0;; level++) {
        if (level >= kStackSize || p < 0 || p >= n - 1) {
          atomicOr(&g->err, kErrStack);
          break;
        }
        BNode* P = nodes + p;
        const bool is_left = (__ldcg(&P->child.x) == code);
        if (is_left) {
          __stcg(&P->xy_l, make_float4(lo[0], hi[0], lo[1], hi[1]));
          __stcg(reinterpret_cast<float2*>(&P->z_lr), make_float2(lo[2], hi[2]));
        } else {
          __stcg(&P->xy_r, make_float4(lo[0], hi[0], lo[1], hi[1]));
          __stcg(reinterpret_cast<float2*>(&P->z_lr) + 1, make_float2(lo[2], hi[2]));
        }
        __threadfence();
        const int old = atomicAdd(flags + p, 1);
        if ((old & 1) == 0) break;  // first arrival: the sibling finishes this node
        __threadfence();
        const float4 xl = __ldcg(&P->xy_l), xr = __ldcg(&P->xy_r), zz = __ldcg(&P->z_lr);
        lo[0] = fminf(xl.x, xr.x), hi[0] = fmaxf(xl.y, xr.y);
        lo[1] = fminf(xl.z, xr.z), hi[1] = fmaxf(xl.w, xr.w);
        lo[2] = fminf(zz.x, zz.z), hi[2] = fmaxf(zz.y, zz.w);
        if (p == 0) {
#pragma unroll
          for (int q = 0; q < 3; q++) g->root_box[q] = lo[q], g->root_box[3 + q] = hi[q];
          break;
        }
        code = p;
        p = __ldg(parent + p);
      }
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, off));
  const bool all_ok = __all_sync(0xffffffffu, ok);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&g->emax, f2ord(e));
    if (!all_ok) atomicOr(&g->err, kErrNonFinite);
  }
}

}  // namespace

int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

cudaError_t launch_build(const MeshBufs& m, const BuildBufs& b, cudaStream_t st) {
  const int n = m.ntri;
  if (n <= 0) return cudaSuccess;
  const int passes = 3;
  const int tiles = sort_tiles(n);
  k_build_init<<<1, 1024, 0, st>>>(b.g, b.hist, passes * kRadix);
  const int sms = num_sms();
  const int gb = min((n + 255) / 256, sms * 8);
  k_bounds<<<gb, 256, 0, st>>>(m.verts, m.vidx, n, b.g);
  const int gm = min((n + 511) / 512, sms * 2);
  k_morton<<<gm, 512, 0, st>>>(m.verts, m.vidx, n, b.g, b.keys_a, b.hist, passes, b.status, passes * tiles * kRadix);
  // pass 0: keys_a -> keys_b (values 0..n-1), pass 1: b -> a, pass 2: a -> b
  const uint32_t* kin = b.keys_a;
  const uint32_t* vin = nullptr;
  for (int p = 0; p < passes; p++) {
    uint32_t* ko = (p & 1) ? b.keys_a : b.keys_b;
    uint32_t* vo = (p & 1) ? b.vals_a : b.vals_b;
    k_onesweep<<<tiles, kSortThreads, 0, st>>>(kin, vin, ko, vo, n, p * kRadixBits, b.hist + p * kRadix,
                                                b.status + (size_t)p * tiles * kRadix, &b.g->tile_counter[p],
                                                &b.g->err);
    kin = ko;
    vin = vo;
  }
  if (n >= 2) k_hierarchy<<<(n - 1 + 255) / 256, 256, 0, st>>>(b.keys_b, n, b.nodes, b.parent, b.flags);
  k_refit<<<(n + 255) / 256, 256, 0, st>>>(m.verts, m.vidx, b.vals_b, n, b.nodes, b.leaves, b.parent, b.flags, b.g);
  return cudaGetLastError();
}

cudaError_t launch_refit(const MeshBufs& m, const BuildBufs& b, cudaStream_t st) {
  const int n = m.ntri;
  if (n <= 0) return cudaSuccess;
  cudaMemsetAsync(&b.g->emax, 0, sizeof(int), st);  // f2ord(0.f) == 0
  k_refit<<<(n + 255) / 256, 256, 0, st>>>(m.verts, m.vidx, b.vals_b, n, b.nodes, b.leaves, b.parent, b.flags, b.g);
  return cudaGetLastError();
}

cudaError_t launch_morton(const float* verts, const int* vidx, int n, const float* box6, uint32_t* codes,
                          cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int g = min((n + 255) / 256, num_sms() * 8);
  k_morton_only<<<g, 256, 0, st>>>(verts, vidx, n, box6, codes);
  return cudaGetLastError();
}

// Scratch layout: [tmp keys n][tmp vals n][hist passes*R][status passes*tiles*R][counters 4][err 1]
size_t sort_scratch_bytes(int n, int key_bits) {
  const int passes = sort_passes(key_bits);
  const size_t words = 2 * (size_t)n + (size_t)passes * kRadix + (size_t)passes * sort_tiles(n) * kRadix + 8;
  return words * sizeof(uint32_t);
}

cudaError_t launch_sort_pairs(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, int n,
                              int key_bits, void* scratch, int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int passes = sort_passes(key_bits);
  const int tiles = sort_tiles(n);
  uint32_t* w = static_cast<uint32_t*>(scratch);
  uint32_t* tk = w;
  uint32_t* tv = w + n;
  uint32_t* hist = w + 2 * (size_t)n;
  uint32_t* status = hist + passes * kRadix;
  unsigned* counters = status + (size_t)passes * tiles * kRadix;
  k_zero_u32<<<1, 256, 0, st>>>(hist, passes * kRadix);
  k_zero_u32<<<1, 32, 0, st>>>(counters, 4);
  const int gm = min((n + 511) / 512, num_sms() * 2);
  k_key_hist<<<gm, 512, 0, st>>>(kin, n, hist, passes, status, passes * tiles * kRadix);
  const uint32_t* ki = kin;
  const uint32_t* vi = vin;
  for (int p = 0; p < passes; p++) {
    const bool to_out = ((passes - 1 - p) & 1) == 0;
    uint32_t* ko = to_out ? kout : tk;
    uint32_t* vo = to_out ? vout : tv;
    k_onesweep<<<tiles, kSortThreads, 0, st>>>(ki, vi, ko, vo, n, p * kRadixBits, hist + p * kRadix,
                                                status + (size_t)p * tiles * kRadix, counters + p, err);
    ki = ko;
    vi = vo;
  }
  return cudaGetLastError();
}

}  // namespace crt

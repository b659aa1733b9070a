// build.cu -- the LBVH build on sm_103a.
//
// Stages (reference: Scene_d::operator= and BVH_d::setUp, src/scene.cpp:82-160,
// src/bvh.cpp:3-32):
//   k_build_init   reset the per-scene globals and sort histograms
//   k_bounds       triangle AABBs reduced to the scene box (findMinMax)
//   k_morton       30-bit Morton codes (+ the digit histograms of the sort
//                  passes when they run as look-back passes)
//   k_sort_coop    stable LSD radix sort, 10-bit digits, all three passes in
//                  one cooperative launch (or k_onesweep x3, decoupled
//                  look-back, when the tiles do not all fit at once)
//   k_hierarchy    Karras split search, one thread per internal node
//   k_refit        atomic bottom-up refit, one climber per leaf; it also
//                  writes the leaf triangles in sorted order for traversal
// Triangle boxes are never stored: each stage that needs one recomputes it
// from the three vertices (L2-resident for the sizes this targets).
#include <cstdio>

#include "build_device.cuh"

namespace crt {

namespace {

// Empty group boxes for k_refit's atomic min/max (order-preserving ints).
__device__ __forceinline__ void clear_group_boxes(int* gbox, int groups) {
  for (int i = threadIdx.x; i < 6 * groups; i += blockDim.x) gbox[i] = f2ord(i % 6 < 3 ? INFINITY : -INFINITY);
}

__global__ void k_build_init(SceneGlobals* g, uint32_t* hist, int nhist, int* gbox, int groups) {
  pdl_wait();
  pdl_launch_dependents();
  const int t = threadIdx.x;
  clear_group_boxes(gbox, groups);
  if (t < 3) {
    g->bmin[t] = f2ord(1e9f);  // findMinMax's initial values (kernels/scene.cu:75,80)
    g->bmax[t] = f2ord(-1e9f);
  }
  if (t == 0) {
    g->emax = f2ord(0.f);
    g->err = 0;
    g->nspan = 0u;
  }
  if (t < 4) g->tile_counter[t] = 0;
  for (int i = t; i < nhist; i += blockDim.x) hist[i] = 0;
}

// Scene bounds (kernels/scene.cu:72-85) and the largest triangle extent.
__global__ void __launch_bounds__(256) k_bounds(const float* __restrict__ V, const int* __restrict__ vidx, int n,
                                                SceneGlobals* g) {
  pdl_wait();
  pdl_launch_dependents();
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
  // block reduction, then one set of atomics per block
  __shared__ float s_red[8][7];
  __shared__ int s_bad;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_bad = 0;
  __syncthreads();
  if (!__all_sync(0xffffffffu, ok) && lane == 0) s_bad = 1;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < 3; k++) s_red[warp][k] = lo[k], s_red[warp][3 + k] = hi[k];
    s_red[warp][6] = e;
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    const int k = threadIdx.x;
    float v = s_red[0][k];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) v = (k < 3) ? fminf(v, s_red[w][k]) : fmaxf(v, s_red[w][k]);
    if (k < 3)
      atomicMin(&g->bmin[k], f2ord(v));
    else if (k < 6)
      atomicMax(&g->bmax[k - 3], f2ord(v));
    else
      atomicMax(&g->emax, f2ord(v));
  }
  if (threadIdx.x == 0 && s_bad) atomicOr(&g->err, kErrNonFinite);
}

// Morton codes; with HIST also the digit histograms of the sort passes (the
// look-back passes need them; the cooperative sort counts its digits itself)
// and the look-back status cleared.  (Counting each digit once per group of
// lanes that share it, with __match_any_sync, measured 31 us against 25 us
// for per-lane shared atomics on the 1M-triangle build.)
template <bool HIST>
__global__ void __launch_bounds__(512, 2) k_morton(const float* __restrict__ V, const int* __restrict__ vidx, int n,
                                                   const SceneGlobals* g, uint32_t* __restrict__ keys,
                                                   uint32_t* __restrict__ hist, int passes,
                                                   uint32_t* __restrict__ status, int status_words) {
  __shared__ uint32_t sh[HIST ? 3 * kRadix : 1];
  if (HIST)
    for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) sh[i] = 0;
  pdl_wait();
  pdl_launch_dependents();
  if (HIST)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < status_words; i += gridDim.x * blockDim.x) status[i] = 0;
  MortonAxis ax[3];
  load_scene_box(g, ax);
  if (HIST) __syncthreads();
  // four triangles per thread per round: their loads overlap
  const int stride = gridDim.x * blockDim.x;
  for (int t0 = blockIdx.x * blockDim.x + threadIdx.x; t0 < n; t0 += 4 * stride) {
    float lo[4][3], hi[4][3];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int t = t0 + u * stride;
      float3 a, b, c;
      if (t < n) tri_box(V, vidx, t, a, b, c, lo[u], hi[u]);
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int t = t0 + u * stride;
      if (t < n) {
        const uint32_t code = morton_code(lo[u], hi[u], ax);
        keys[t] = code;
        if (HIST)
          for (int p = 0; p < passes; p++)
            atomicAdd(&sh[p * kRadix + ((code >> (p * kRadixBits)) & (kRadix - 1))], 1u);
      }
    }
  }
  if (HIST) {
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x)
      if (sh[i]) atomicAdd(&hist[i], sh[i]);
  }
}

// Standalone Morton codes against a given scene box (crt_morton).  A
// triangle with a vertex index outside [0, nv) sets *err and gets code 0; its
// vertices are not read.
__global__ void k_morton_only(const float* __restrict__ V, int nv, const int* __restrict__ vidx, int n,
                              const float* __restrict__ box6, uint32_t* __restrict__ keys, int* err) {
  MortonAxis ax[3];
#pragma unroll
  for (int k = 0; k < 3; k++) ax[k] = morton_axis_setup(box6[k], box6[3 + k]);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    if ((unsigned)__ldg(vidx + 3 * t) >= (unsigned)nv || (unsigned)__ldg(vidx + 3 * t + 1) >= (unsigned)nv ||
        (unsigned)__ldg(vidx + 3 * t + 2) >= (unsigned)nv) {
      atomicOr(err, 1);
      keys[t] = 0u;
      continue;
    }
    float3 a, b, c;
    float lo[3], hi[3];
    tri_box(V, vidx, t, a, b, c, lo, hi);
    keys[t] = morton_code(lo, hi, ax);
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

// All passes of the build's stable LSD sort in one cooperative launch, one
// 8192-key tile per block (so at most as many tiles as blocks that fit on the
// GPU at once; launch_build falls back to k_onesweep passes beyond that).
// Within a pass every block ranks its tile as k_onesweep does, publishes its
// per-digit counts, and after a grid-wide barrier sums the counts of all
// tiles, keeping apart those of the tiles before it (up to a few hundred
// independent loads per thread instead of a chain of look-back round trips):
// the digit totals give each digit's start, so no histogram pass precedes the
// sort.  Then it scatters; a second barrier ends the pass.  Pass p reads keys_a (p even) or keys_b and writes the other
// array (values likewise; pass 0 takes values 0..n-1).  Barrier words:
// bar[0..1], zero at launch; a barrier that waits too long sets kErrTimeout
// in *err and the kernel stops.
template <int TH, int IT>
__global__ void __launch_bounds__(TH, 1) k_sort_coop(uint32_t* keys_a, uint32_t* keys_b, uint32_t* vals_a,
                                                     uint32_t* vals_b, int n, int passes, uint32_t* counts,
                                                     unsigned* bar, int* err) {
  constexpr int W = TH / 32;
  constexpr int TILE = TH * IT;
  constexpr int DPT = kRadix / TH;
  static_assert(kRadix % TH == 0 && 32 * IT < 65536, "digits per thread, 16-bit warp counters");
  __shared__ SortSmem<TH, IT> sm;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tile = blockIdx.x, ntiles = gridDim.x, base = tile * TILE;
  const uint32_t mask = kRadix - 1;
  unsigned short* wh = reinterpret_cast<unsigned short*>(sm.whist[warp]);
  const uint32_t lt = lanemask_lt();
  for (int p = 0; p < passes; p++) {
    const uint32_t* kin = (p & 1) ? keys_b : keys_a;
    const uint32_t* vin = p == 0 ? nullptr : ((p & 1) ? vals_b : vals_a);
    uint32_t* kout = (p & 1) ? keys_a : keys_b;
    uint32_t* vout = (p & 1) ? vals_a : vals_b;
    const int shift = p * kRadixBits;
    // each warp clears its own counters (no other warp reads them before the
    // block's next __syncthreads)
    for (int i = lane; i < kRadix / 2; i += 32) sm.whist[warp][i] = 0;
    __syncwarp();
    // rank the tile's keys in input order (stable), warp by warp
    uint32_t key[IT], val[IT], rank[IT];
#pragma unroll
    for (int r = 0; r < IT; r++) {  // every load issued before the ranking's warp syncs
      const int idx = base + warp * (32 * IT) + r * 32 + lane;
      const bool valid = idx < n;
      key[r] = valid ? ld_in<false>(kin + idx) : 0u;
      val[r] = valid ? (vin ? ld_in<false>(vin + idx) : (uint32_t)idx) : 0u;
    }
#pragma unroll
    for (int r = 0; r < IT; r++) {
      const int idx = base + warp * (32 * IT) + r * 32 + lane;
      const bool valid = idx < n;
      const uint32_t d = valid ? ((key[r] >> shift) & mask) : (uint32_t)kRadix;
      const uint32_t peers = digit_peers(d, valid);
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
    // per digit: warp offsets (exclusive, in place) and the tile's count
    uint32_t cnt[DPT], csum = 0;
#pragma unroll
    for (int j = 0; j < DPT; j++) {
      const int d = DPT * tid + j;
      uint32_t c = 0;
#pragma unroll
      for (int w = 0; w < W; w++) {
        unsigned short* h = reinterpret_cast<unsigned short*>(sm.whist[w]) + d;
        const uint32_t x = *h;
        *h = (unsigned short)c;
        c += x;
      }
      cnt[j] = c;
      csum += c;
    }
    uint32_t* mine = counts + ((size_t)p * ntiles + tile) * kRadix;
#pragma unroll
    for (int j = 0; j < DPT; j++) mine[DPT * tid + j] = cnt[j];
    if (!grid_barrier(bar, ntiles, err)) return;
    // each digit's count over the tiles before this one, and over all tiles
    // (every block reads every tile's counts: no longer than the last
    // block's prefix alone, which the pass waits for anyway)
    uint32_t pre[DPT], tot[DPT], gsum = 0;
#pragma unroll
    for (int j = 0; j < DPT; j++) {
      const uint32_t* col = counts + (size_t)p * ntiles * kRadix + DPT * tid + j;
      // 32 loads in flight per round (each round waits one L2 round trip)
      constexpr int U = 32;
      uint32_t acc = 0u, all = 0u;
      for (int t0 = 0; t0 < ntiles; t0 += U) {
        uint32_t x[U];
#pragma unroll
        for (int u = 0; u < U; u++) x[u] = t0 + u < ntiles ? __ldcg(col + (size_t)(t0 + u) * kRadix) : 0u;
#pragma unroll
        for (int u = 0; u < U; u++) {
          all += x[u];
          acc += t0 + u < tile ? x[u] : 0u;
        }
      }
      pre[j] = acc;
      tot[j] = all;
      gsum += all;
    }
    // digit starts (over all keys) and tile-local digit starts, in one scan
    uint32_t gpre, cpre;
    block_excl_scan2<TH>(gsum, csum, sm.warp2, gpre, cpre);
    {
      uint32_t c = cpre, g = gpre;
#pragma unroll
      for (int j = 0; j < DPT; j++) {
        const int d = DPT * tid + j;
        sm.tstart[d] = c;
        sm.gbase[d] = g + pre[j] - c;
        c += cnt[j];
        g += tot[j];
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < IT; r++) {
      const int idx = base + warp * (32 * IT) + r * 32 + lane;
      if (idx < n) {
        const uint32_t d = (key[r] >> shift) & mask;
        const uint32_t pos = sm.tstart[d] + wh[d] + rank[r];
        sm.keys[pos] = key[r];
        sm.vals[pos] = val[r];
      }
    }
    __syncthreads();
    const int tile_n = min(TILE, n - base);
    for (int i = tid; i < tile_n; i += TH) {
      const uint32_t k = sm.keys[i];
      const uint32_t pos = sm.gbase[(k >> shift) & mask] + (uint32_t)i;
      kout[pos] = k;
      vout[pos] = sm.vals[i];
    }
    if (p + 1 < passes && !grid_barrier(bar, ntiles, err)) return;
  }
}

// BuildHierarchy (kernels/bvh.cu:164-207) with FindSpan (bvh.cu:100-133) and
// FindSplit (bvh.cu:134-162): one thread per internal node writes its
// children's parent words and lists its spanning children for
// k_refit_spans (the child codes and boxes reach the wide nodes through the
// refit, which relies on the empty odd slot marked here beside a leaf
// child).  Every probe of a node
// whose span is at most kShortSpan leaves lies within kShortSpan of the node,
// so a block first stages the codes of its nodes +- kShortSpan in shared
// memory (one coalesced load) and searches there.  A node whose span turns
// out longer (the nodes near the root, whose binary searches are the longest
// chains of dependent loads) is searched by its whole warp in global memory,
// 32 candidates at a time.  Both searches look for the end of a prefix on
// which the reference's predicate holds (common prefix with the node's first
// key longer than at the span's other end), so they return the reference's
// span and split.
constexpr int kShortSpan = 512;
constexpr int kHierThreads = 256;
constexpr int kHierWindow = kHierThreads + 2 * kShortSpan + 1;

// delta() on the shared-memory window (j within it, or out of [0, n): -1).
__device__ __forceinline__ int kdelta_s(const uint32_t* s_c, int w0, int n, uint64_t ki, int j) {
  if (j < 0 || j >= n) return -1;
  const uint64_t kj = ((uint64_t)s_c[j - w0] << 32) | (uint32_t)j;
  return __clzll((long long)(ki ^ kj));
}

__global__ void __launch_bounds__(kHierThreads) k_hierarchy(const uint32_t* __restrict__ codes, int n,
                                                            uint32_t* __restrict__ parent, WNode* __restrict__ wnodes,
                                                            uint4* __restrict__ spans, unsigned* nspan) {
  __shared__ uint32_t s_c[kHierWindow];
  pdl_wait();
  pdl_launch_dependents();
  const int i0 = blockIdx.x * kHierThreads;
  const int w0 = i0 - kShortSpan;
  for (int j = threadIdx.x; j < kHierWindow; j += kHierThreads) {
    const int g = w0 + j;
    s_c[j] = (g >= 0 && g < n) ? __ldg(codes + g) : 0u;
  }
  __syncthreads();
  const int i = i0 + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool act = i < n - 1;
  int d = 1, dmin = 0, lo = 0, hi = 0, split = 0;
  bool wide = false;
  if (act) {
    const uint64_t ki = ((uint64_t)s_c[i - w0] << 32) | (uint32_t)i;
    const int dd = kdelta_s(s_c, w0, n, ki, i + 1) - kdelta_s(s_c, w0, n, ki, i - 1);
    d = dd > 0 ? 1 : (dd < 0 ? -1 : 0);
    dmin = kdelta_s(s_c, w0, n, ki, i - d);
    int lmax = 2;
    while (lmax <= kShortSpan && kdelta_s(s_c, w0, n, ki, i + lmax * d) > dmin) lmax *= 2;
    wide = lmax > kShortSpan;
    if (!wide) {
      int l = 0, t = lmax;
      do {
        t /= 2;
        if (kdelta_s(s_c, w0, n, ki, i + (l + t) * d) > dmin) l += t;
      } while (t > 1);
      lo = min(i, i + l * d), hi = max(i, i + l * d);
      int left = lo, right = hi;
      uint64_t kl = ((uint64_t)s_c[left - w0] << 32) | (uint32_t)left;
      const int same = kdelta_s(s_c, w0, n, kl, right);
      do {
        const int s = (right + left) / 2;
        if (kdelta_s(s_c, w0, n, kl, s) > same) {
          left = s;
          kl = ((uint64_t)s_c[left - w0] << 32) | (uint32_t)left;
        } else {
          right = s;
        }
      } while (right > left + 1);
      split = left;
    }
  }
  // the warp searches each wide node's span and split together
  for (unsigned todo = __ballot_sync(0xffffffffu, wide); todo; todo &= todo - 1) {
    const int L = __ffs(todo) - 1;
    const int iL = __shfl_sync(0xffffffffu, i, L), dL = __shfl_sync(0xffffffffu, d, L);
    const int dminL = __shfl_sync(0xffffffffu, dmin, L);
    const uint64_t kiL = ((uint64_t)__ldg(codes + iL) << 32) | (uint32_t)iL;
    const int l = warp_prefix_end(n, [&](int m) { return kdelta(codes, n, kiL, iL + m * dL) > dminL; });
    const int loL = min(iL, iL + l * dL), hiL = max(iL, iL + l * dL);
    const uint64_t klo = ((uint64_t)__ldg(codes + loL) << 32) | (uint32_t)loL;
    const int same = kdelta(codes, n, klo, hiL);
    const int o = warp_prefix_end(hiL - loL - 1, [&](int m) { return kdelta(codes, n, klo, loL + m) > same; });
    if (lane == L) lo = loL, hi = hiL, split = loL + o;
  }
  const int c1 = (split == lo) ? ~split : split;
  const int c2 = (split + 1 == hi) ? ~(split + 1) : split + 1;
  if (spans) {
    // the spanning children (internal nodes whose leaf range crosses a
    // kRefitBlock boundary) join the list k_refit_spans works through:
    // (node, first leaf, last leaf, parent word)
    const bool s1 = act && c1 >= 0 && lo / kRefitBlock != split / kRefitBlock;
    const bool s2 = act && c2 >= 0 && (split + 1) / kRefitBlock != hi / kRefitBlock;
    const uint32_t m1 = __ballot_sync(0xffffffffu, s1), m2 = __ballot_sync(0xffffffffu, s2);
    if (m1 | m2) {
      unsigned base = 0;
      if (lane == 0) base = atomicAdd(nspan, (unsigned)(__popc(m1) + __popc(m2)));
      base = __shfl_sync(0xffffffffu, base, 0);
      const uint32_t lt = lanemask_lt();
      const uint32_t pw = (uint32_t)i | ((lo / kRefitBlock != hi / kRefitBlock) ? kParentSpans : 0u);
      if (s1) spans[base + __popc(m1 & lt)] = make_uint4((uint32_t)c1, (uint32_t)lo, (uint32_t)split, pw | kParentLeft);
      if (s2)
        spans[base + __popc(m1) + __popc(m2 & lt)] = make_uint4((uint32_t)c2, (uint32_t)(split + 1), (uint32_t)hi, pw);
    }
  }
  if (!act) return;
  const uint32_t spanbit = (lo / kRefitBlock != hi / kRefitBlock) ? kParentSpans : 0u;
  parent[c1 < 0 ? (n - 1) + split : split] = (uint32_t)i | kParentLeft | spanbit;
  parent[c2 < 0 ? (n - 1) + split + 1 : split + 1] = (uint32_t)i | spanbit;
  // a leaf child takes one slot of this node's wide node: mark the other empty
  const float4 empty = make_float4(0.f, 0.f, 0.f, __int_as_float(kNoChild));
  if (c1 < 0) wnodes[i].s[1].lo_code = empty;
  if (c2 < 0) wnodes[i].s[3].lo_code = empty;
}

// Box helpers: six floats (lo xyz, hi xyz) at 8-byte aligned addresses,
// through L2 (written and read by different blocks).
__device__ __forceinline__ void box_union6(float b[6], const float* q) {
  const float2 x = __ldcg(reinterpret_cast<const float2*>(q)), y = __ldcg(reinterpret_cast<const float2*>(q) + 1),
               z = __ldcg(reinterpret_cast<const float2*>(q) + 2);
  b[0] = fminf(b[0], x.x), b[1] = fminf(b[1], x.y), b[2] = fminf(b[2], y.x);
  b[3] = fmaxf(b[3], y.y), b[4] = fmaxf(b[4], z.x), b[5] = fmaxf(b[5], z.y);
}
__device__ __forceinline__ void box_store6(float* q, const float b[6]) {
  float2* d = reinterpret_cast<float2*>(q);
  __stcg(d, make_float2(b[0], b[1]));
  __stcg(d + 1, make_float2(b[2], b[3]));
  __stcg(d + 2, make_float2(b[4], b[5]));
}

// The boxes of the spanning nodes (leaf ranges over several refit blocks).
// Each is the union of its leaves' boxes, and its leaf range [lo, hi] is
// known from the split search, so no climb is needed: the box is the union
// of the boxes of leaves lo..end of lo's block (suf[lo]), of the blocks in
// between (suf at a block's first leaf, or gbox for whole groups of
// kSpanGroup blocks) and of leaves start of hi's block..hi (pre[hi]), all
// written by k_refit.  (lo
// starts the leftmost maximal block-local node under the spanning node,
// which is a left child of a spanning node, and hi ends the rightmost one, a
// right child: k_refit writes suf and pre at both ends of every such node.)
// kSpanLanes lanes per listed node share the blocks and groups in between;
// the item after the list is the root.  min/max are exact, so the boxes
// equal those of the reference's climb.
constexpr int kSpanLanes = 8;

__global__ void __launch_bounds__(256) k_refit_spans(WNode* wnodes, const uint32_t* __restrict__ parent,
                                                     const uint4* __restrict__ spans, const float* suf,
                                                     const float* pre, const int* gbox, int n, SceneGlobals* g) {
  pdl_wait();
  pdl_launch_dependents();
  const unsigned count = *(volatile unsigned*)&g->nspan;
  const int sub = threadIdx.x & (kSpanLanes - 1);
  const unsigned groups = (gridDim.x * blockDim.x) / kSpanLanes;
  const unsigned first = (blockIdx.x * blockDim.x + threadIdx.x) / kSpanLanes;
  // every lane of a warp runs the same number of rounds (the shuffles below)
  const unsigned rounds = (count + 1 + groups - 1) / groups;
  for (unsigned rnd = 0; rnd < rounds; rnd++) {
    const unsigned item = first + rnd * groups;
    const bool live = item <= count;
    const bool root = item == count;
    uint4 e = make_uint4(0u, 0u, (uint32_t)(n - 1), 0u);
    if (live && !root) e = __ldg(spans + item);
    const int lo = (int)e.y, hi = (int)e.z;
    bool ok = live;
    if (live && !root && ((unsigned)lo >= (unsigned)n || (unsigned)hi >= (unsigned)n ||
                          lo / kRefitBlock >= hi / kRefitBlock)) {
      if (sub == 0) atomicOr(&g->err, kErrStack);  // only a corrupt list gets here
      ok = false;
    }
    // blocks strictly between the ends (the root: all): [b0, h) and [t, b1)
    // one by one, the whole groups in [h, t) from gbox
    const int b0 = root ? 0 : lo / kRefitBlock + 1;
    int b1 = root ? (n - 1) / kRefitBlock + 1 : hi / kRefitBlock;
    int h = min(b1, (b0 + kSpanGroup - 1) / kSpanGroup * kSpanGroup);
    int t = max(h, b1 / kSpanGroup * kSpanGroup);
    if (!ok) h = t = b1 = b0;
    const int nh = h - b0, ng = (t - h) / kSpanGroup, nt = b1 - t, total = nh + ng + nt;
    float b[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int j = sub; j < total; j += kSpanLanes) {
      if (j >= nh && j < nh + ng) {
        const int* q = gbox + 6 * (size_t)(h / kSpanGroup + j - nh);
#pragma unroll
        for (int c = 0; c < 3; c++)
          b[c] = fminf(b[c], ord2f(__ldcg(q + c))), b[3 + c] = fmaxf(b[3 + c], ord2f(__ldcg(q + 3 + c)));
      } else {
        box_union6(b, suf + 6 * (size_t)kRefitBlock * (size_t)(j < nh ? b0 + j : t + j - nh - ng));
      }
    }
    if (__any_sync(0xffffffffu, total > 0)) {
#pragma unroll
      for (int o = kSpanLanes / 2; o > 0; o >>= 1) {
#pragma unroll
        for (int q = 0; q < 3; q++) {
          b[q] = fminf(b[q], __shfl_xor_sync(0xffffffffu, b[q], o));
          b[3 + q] = fmaxf(b[3 + q], __shfl_xor_sync(0xffffffffu, b[3 + q], o));
        }
      }
    }
    if (!ok || sub != 0) continue;
    if (root) {
#pragma unroll
      for (int q = 0; q < 6; q++) g->root_box[q] = b[q];
      continue;
    }
    box_union6(b, suf + 6 * (size_t)lo);
    box_union6(b, pre + 6 * (size_t)hi);
    const int x = (int)e.x, p = (int)(e.w & kParentMask);
    const uint32_t wn = (p == 0) ? 0u : __ldg(parent + p);
    const int gp = (p == 0) ? n - 1 : (int)(wn & kParentMask);
    if (x <= 0 || x >= n - 1 || p >= n - 1 || (p != 0 && gp >= n - 1)) {  // only a corrupt tree gets here
      atomicOr(&g->err, kErrStack);
      continue;
    }
    const float lo3[3] = {b[0], b[1], b[2]}, hi3[3] = {b[3], b[4], b[5]};
    put_wide(wnodes, x, (e.w & kParentLeft) != 0, p, gp, (p == 0) || (wn & kParentLeft) != 0, lo3, hi3);
  }
}

__global__ void __launch_bounds__(kRefitBlock, 4) k_refit(const float* __restrict__ V, const int* __restrict__ vidx,
                                                       const uint32_t* __restrict__ ids, int n,
                                                       WNode* wnodes, LeafTri* __restrict__ leaves,
                                                       const uint32_t* __restrict__ parent, float* __restrict__ suf,
                                                       float* __restrict__ pre, int* __restrict__ gbox,
                                                       SceneGlobals* g) {
  // children's boxes at each block-local node (lo, hi); lo.w: the leaf-range
  // end the first arrival brings (its first leaf if it is the left child,
  // else its last)
  __shared__ float4 s_box[kRefitBlock][2][2];
  __shared__ int s_flag[kRefitBlock];
  // the block's maximal block-local nodes (their parents span): box, and
  // first / last leaf in lo.w / hi.w
  __shared__ float4 s_top[kRefitBlock][2];
  __shared__ int s_ntop;
  s_flag[threadIdx.x] = 0;
  if (threadIdx.x == 0) s_ntop = 0;
  pdl_wait();
  pdl_launch_dependents();
  __syncthreads();
  const int k0 = blockIdx.x * kRefitBlock;
  const int k = k0 + threadIdx.x;
  float e = 0.f;
  bool ok = true;
  int top = -1;  // this thread's entry in s_top
  int l = k, r = k;  // leaf range of the climbing node
  float lo[3], hi[3];
  bool live = false;
  if (k < n) {
    const int tri = (int)__ldg(ids + k);
    if ((unsigned)tri >= (unsigned)n) {  // only a corrupt sort gets here
      atomicOr(&g->err, kErrStack);
    } else {
      float3 a, b, c;
      tri_box(V, vidx, tri, a, b, c, lo, hi);
      ok = finite_coords(a, b, c);
      e = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
      LeafTri lt;
      lt.v0 = make_float4(a.x, a.y, a.z, __int_as_float(tri));
      lt.v1 = make_float4(b.x, b.y, b.z, 0.f);
      lt.v2 = make_float4(c.x, c.y, c.z, 0.f);
      leaves[k] = lt;
      live = true;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, off));
  const bool all_ok = __all_sync(0xffffffffu, ok);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&g->emax, f2ord(e));
    if (!all_ok) atomicOr(&g->err, kErrNonFinite);
  }
  if (live) {
    if (n == 1) {
#pragma unroll
      for (int q = 0; q < 3; q++) g->root_box[q] = lo[q], g->root_box[3 + q] = hi[q];
    } else {
      uint32_t w = __ldg(parent + (n - 1) + k);
      int xc = ~k;  // code of the node that climbs (a leaf, then internal nodes)
      for (;;) {
        const int p = (int)(w & kParentMask);
        if (p >= n - 1) {  // only a corrupt tree gets here
          atomicOr(&g->err, kErrStack);
          break;
        }
        const uint32_t wn = (p == 0) ? 0u : __ldg(parent + p);  // next step's word, issued early
        const bool is_left = (w & kParentLeft) != 0;
        const int gp = (p == 0) ? n - 1 : (int)(wn & kParentMask);
        const bool p_left = (p == 0) || (wn & kParentLeft) != 0;
        if (gp >= n - 1 && p != 0) {  // only a corrupt tree gets here
          atomicOr(&g->err, kErrStack);
          break;
        }
        put_wide(wnodes, xc, is_left, p, gp, p_left, lo, hi);
        if (!(w & kParentSpans)) {  // both arrivals are threads of this block
          const int sl = p - k0;
          if ((unsigned)sl >= (unsigned)kRefitBlock) {  // only a corrupt tree gets here
            atomicOr(&g->err, kErrStack);
            break;
          }
          float4* mine = s_box[sl][is_left ? 0 : 1];
          mine[0] = make_float4(lo[0], lo[1], lo[2], __int_as_float(is_left ? l : r));
          mine[1] = make_float4(hi[0], hi[1], hi[2], 0.f);
          __threadfence_block();
          // the first arrival stops; only the second climbs on (so a corrupt
          // tree cannot make a climb loop: each slot lets one climber through)
          const int arrived = atomicAdd(&s_flag[sl], 1);
          if (arrived != 1) {
            if (arrived != 0) atomicOr(&g->err, kErrStack);
            break;
          }
          __threadfence_block();
          const float4* o = s_box[sl][is_left ? 1 : 0];
          const float4 ol = o[0], oh = o[1];
          lo[0] = fminf(lo[0], ol.x), lo[1] = fminf(lo[1], ol.y), lo[2] = fminf(lo[2], ol.z);
          hi[0] = fmaxf(hi[0], oh.x), hi[1] = fmaxf(hi[1], oh.y), hi[2] = fmaxf(hi[2], oh.z);
          if (is_left)
            r = __float_as_int(ol.w);
          else
            l = __float_as_int(ol.w);
        } else {
          // the parent spans: k_refit_spans finds its box from the block boxes
          // and the edge boxes written below
          top = atomicAdd(&s_ntop, 1);
          s_top[top][0] = make_float4(lo[0], lo[1], lo[2], __int_as_float(l));
          s_top[top][1] = make_float4(hi[0], hi[1], hi[2], __int_as_float(r));
          break;
        }
        if (p == 0) {
#pragma unroll
          for (int q = 0; q < 3; q++) g->root_box[q] = lo[q], g->root_box[3 + q] = hi[q];
          break;
        }
        xc = p;
        w = wn;
      }
    }
  }
  // The maximal block-local nodes tile the block's leaves.  Each writes the
  // union of its own and the later ones' boxes at its first leaf (suf) and of
  // the earlier ones' and its own at its last leaf (pre).
  __syncthreads();
  const int ntop = s_ntop;
  if (top >= 0) {
    const int l = __float_as_int(s_top[top][0].w), r = __float_as_int(s_top[top][1].w);
    // one pass per edge box keeps the live registers down
    for (int side = 0; side < 2; side++) {
      float u[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
      for (int t = 0; t < ntop; t++) {
        const float4 a = s_top[t][0], b = s_top[t][1];
        if (side == 0 ? __float_as_int(a.w) >= l : __float_as_int(b.w) <= r) {
          u[0] = fminf(u[0], a.x), u[1] = fminf(u[1], a.y), u[2] = fminf(u[2], a.z);
          u[3] = fmaxf(u[3], b.x), u[4] = fmaxf(u[4], b.y), u[5] = fmaxf(u[5], b.z);
        }
      }
      box_store6(side == 0 ? suf + 6 * (size_t)l : pre + 6 * (size_t)r, u);
      if (side == 0 && l == k0) {
        // suf at the block's first leaf is the block's box; it also joins
        // the box of the block's group of kSpanGroup blocks, by exact atomic
        // min/max on order-preserving integers (reset before every refit)
        int* q = gbox + 6 * (blockIdx.x / kSpanGroup);
#pragma unroll
        for (int c = 0; c < 3; c++) atomicMin(q + c, f2ord(u[c])), atomicMax(q + 3 + c, f2ord(u[3 + c]));
      }
    }
  }
}

}  // namespace

namespace {
__global__ void k_refit_init(SceneGlobals* g, int* gbox, int groups) {
  if (threadIdx.x == 0) g->emax = f2ord(0.f);
  clear_group_boxes(gbox, groups);
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

// Launches kernel k on st with `grid` blocks of `block` threads, as a
// programmatic dependent of the kernel launched on st before it (dep) or the
// ordinary way.
template <typename... P, typename... A>
static void launch_k(bool dep, void (*k)(P...), int grid, int block, cudaStream_t st, A... args) {
  if (!dep) {
    k<<<grid, block, 0, st>>>(args...);
    return;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, args...);
}

// One sort pass in the shape sort_large(n) picks; `status` holds the
// pass's sort_tiles(n) * kRadix words (enough for either shape).
static void onesweep_pass(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, int n, int shift,
                          const uint32_t* ghist, uint32_t* status, unsigned* counter, int* err, cudaStream_t st,
                          bool dep = false) {
  if (sort_large(n))
    launch_k(dep, k_onesweep<kSortThreadsL, kSortItems>, sort_tiles_used(n), kSortThreadsL, st, kin, vin, kout, vout,
             n, shift, ghist, status, counter, err);
  else
    launch_k(dep, k_onesweep<kSortThreads, kSortItems>, sort_tiles_used(n), kSortThreads, st, kin, vin, kout, vout, n,
             shift, ghist, status, counter, err);
}

// The refit and its spanning-node pass, as programmatic dependents of the
// kernel before them.
static void refit(const MeshBufs& m, const BuildBufs& b, cudaStream_t st) {
  const int n = m.ntri;
  launch_k(true, k_refit, (n + kRefitBlock - 1) / kRefitBlock, kRefitBlock, st, (const float*)m.verts,
           (const int*)m.vidx, (const uint32_t*)b.vals_b, n, b.wnodes, b.leaves, (const uint32_t*)b.parent, b.suf,
           b.pre, b.gbox, b.g);
  if (n > kRefitBlock)
    launch_k(true, k_refit_spans, num_sms() * 8, 256, st, b.wnodes, (const uint32_t*)b.parent,
             (const uint4*)b.spans, (const float*)b.suf, (const float*)b.pre, (const int*)b.gbox, n, b.g);
}

// Whether the build's sort runs as one cooperative launch (k_sort_coop): its
// 8192-key tiles must all be resident at once.
static bool coop_sort_fits(int n) {
  static int capacity = -1;
  if (capacity < 0) {
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_sort_coop<kSortThreadsL, kSortItems>, kSortThreadsL, 0) !=
        cudaSuccess) {
      cudaGetLastError();
      bps = 0;
    }
    capacity = bps * num_sms();
  }
  return n >= 2 * kSortTileL && (n + kSortTileL - 1) / kSortTileL <= capacity;
}

cudaError_t launch_build(const MeshBufs& m, const BuildBufs& b, cudaStream_t st) {
  const int n = m.ntri;
  if (n <= 0) return cudaSuccess;
  const int passes = 3;
  const int tiles = sort_tiles(n);
  const bool coop = coop_sort_fits(n);
  k_build_init<<<1, 1024, 0, st>>>(b.g, b.hist, passes * kRadix, b.gbox, (int)span_groups(n));
  const int sms = num_sms();
  const int gb = min((n + 255) / 256, sms * 8);
  launch_k(true, k_bounds, gb, 256, st, (const float*)m.verts, (const int*)m.vidx, n, b.g);
  const int gm = min((n + 511) / 512, sms * 2);
  // (the look-back status is cleared only for the passes that use it)
  if (coop)
    launch_k(true, k_morton<false>, gm, 512, st, (const float*)m.verts, (const int*)m.vidx, n,
             (const SceneGlobals*)b.g, b.keys_a, b.hist, passes, b.status, 0);
  else
    launch_k(true, k_morton<true>, gm, 512, st, (const float*)m.verts, (const int*)m.vidx, n,
             (const SceneGlobals*)b.g, b.keys_a, b.hist, passes, b.status, passes * tiles * kRadix);
  // pass 0: keys_a -> keys_b (values 0..n-1), pass 1: b -> a, pass 2: a -> b
  if (coop) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)((n + kSortTileL - 1) / kSortTileL));
    cfg.blockDim = dim3(kSortThreadsL);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    // barrier words: tile_counter[0..1], zeroed by k_build_init
    cudaLaunchKernelEx(&cfg, k_sort_coop<kSortThreadsL, kSortItems>, b.keys_a, b.keys_b, b.vals_a, b.vals_b, n,
                       passes, b.status, &b.g->tile_counter[0], &b.g->err);
  } else {
    const uint32_t* kin = b.keys_a;
    const uint32_t* vin = nullptr;
    for (int p = 0; p < passes; p++) {
      uint32_t* ko = (p & 1) ? b.keys_a : b.keys_b;
      uint32_t* vo = (p & 1) ? b.vals_a : b.vals_b;
      onesweep_pass(kin, vin, ko, vo, n, p * kRadixBits, b.hist + p * kRadix, b.status + (size_t)p * tiles * kRadix,
                    &b.g->tile_counter[p], &b.g->err, st, true);
      kin = ko;
      vin = vo;
    }
  }
  if (n >= 2)
    launch_k(true, k_hierarchy, (n - 1 + kHierThreads - 1) / kHierThreads, kHierThreads, st,
             (const uint32_t*)b.keys_b, n, b.parent, b.wnodes, b.spans, &b.g->nspan);
  refit(m, b, st);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- stages
// crt_hierarchy: the parent words of k_hierarchy turned into the reference's
// HNode triplets (parent, left, right; a leaf holds its triangle id twice).
__global__ void __launch_bounds__(256) k_nodes3(const uint32_t* __restrict__ parent,
                                                const uint32_t* __restrict__ ids, int n,
                                                int* __restrict__ nodes3) {
  const int nn = 2 * n - 1;
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < nn; x += gridDim.x * blockDim.x) {
    if (x == 0) {
      nodes3[0] = -1;  // the root
    } else {
      const uint32_t w = __ldg(parent + x);
      const int p = (int)(w & kParentMask);
      nodes3[3 * x] = p;
      nodes3[3 * p + ((w & kParentLeft) ? 1 : 2)] = x;
    }
    if (x >= n - 1) {
      const int id = (int)__ldg(ids + (x - (n - 1)));
      nodes3[3 * x + 1] = id, nodes3[3 * x + 2] = id;
    }
  }
}

cudaError_t launch_stage_hierarchy(const uint32_t* codes, const uint32_t* ids, int n, int* nodes3,
                                   uint32_t* parent, WNode* wnodes, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (n >= 2)
    k_hierarchy<<<(n - 1 + kHierThreads - 1) / kHierThreads, kHierThreads, 0, st>>>(codes, n, parent, wnodes,
                                                                                     nullptr, nullptr);
  k_nodes3<<<(2 * n - 1 + 255) / 256, 256, 0, st>>>(parent, ids, n, nodes3);
  return cudaGetLastError();
}

// crt_refit: RefitBounds (kernels/bvh.cu:209-258) on a caller's HNode
// triplets: one climber per leaf, the second arrival at a node takes the
// union of its children's boxes (bboxunion, bvh.cu:63-69) and climbs on.
// Every index is range-checked (kErrIndex in *err) before it is followed.
__global__ void __launch_bounds__(256) k_refit_nodes(const float* __restrict__ V, int nv,
                                                     const int* __restrict__ vidx, int n,
                                                     const uint32_t* __restrict__ ids,
                                                     const int* __restrict__ nodes3, float* boxes, int* flags,
                                                     int* err) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int tri = (int)__ldg(ids + k);
  if ((unsigned)tri >= (unsigned)n) {
    atomicOr(err, kErrIndex);
    return;
  }
  for (int j = 0; j < 3; j++)
    if ((unsigned)__ldg(vidx + 3 * tri + j) >= (unsigned)nv) {
      atomicOr(err, kErrIndex);
      return;
    }
  float3 a, b, c;
  float lo[3], hi[3];
  tri_box(V, vidx, tri, a, b, c, lo, hi);
  int x = (n - 1) + k;
  for (int q = 0; q < 3; q++) __stcg(boxes + 6 * x + q, lo[q]), __stcg(boxes + 6 * x + 3 + q, hi[q]);
  for (int level = 0; level < 2 * n; level++) {
    const int p = __ldg(nodes3 + 3 * x);
    if (p < 0) return;  // the root
    if (p >= n - 1) {
      atomicOr(err, kErrIndex);
      return;
    }
    __threadfence();
    if (atomicAdd(flags + p, 1) == 0) return;  // first arrival: the sibling climbs on
    __threadfence();
    const int l = __ldg(nodes3 + 3 * p + 1), r = __ldg(nodes3 + 3 * p + 2);
    if ((unsigned)l >= (unsigned)(2 * n - 1) || (unsigned)r >= (unsigned)(2 * n - 1)) {
      atomicOr(err, kErrIndex);
      return;
    }
    const int o = (l == x) ? r : l;
    for (int q = 0; q < 3; q++) {
      lo[q] = fminf(lo[q], __ldcg(boxes + 6 * o + q));
      hi[q] = fmaxf(hi[q], __ldcg(boxes + 6 * o + 3 + q));
    }
    x = p;
    for (int q = 0; q < 3; q++) __stcg(boxes + 6 * x + q, lo[q]), __stcg(boxes + 6 * x + 3 + q, hi[q]);
  }
  atomicOr(err, kErrIndex);  // a cycle: only corrupt triplets get here
}

cudaError_t launch_stage_refit(const float* V, int nv, const int* vidx, int n, const uint32_t* ids,
                               const int* nodes3, float* boxes, int* flags, int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_refit_nodes<<<(n + 255) / 256, 256, 0, st>>>(V, nv, vidx, n, ids, nodes3, boxes, flags, err);
  return cudaGetLastError();
}

// Index arrays that came from device memory (the host checks the others):
// every vertex, normal and material index in range, or kErrIndex.  Reads
// only the index arrays, so a bad index is reported before any kernel uses
// it to address the vertices.
__global__ void __launch_bounds__(256) k_check_indices(const int* __restrict__ vidx, const int* __restrict__ nidx,
                                                       const int* __restrict__ matid, int n, int nv, int nn, int nm,
                                                       SceneGlobals* g) {
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 3 * (int64_t)n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int v = __ldg(vidx + i), k = __ldg(nidx + i);
    bad = bad || (unsigned)v >= (unsigned)nv || (unsigned)k >= (unsigned)nn;
    if (i < n) bad = bad || (unsigned)__ldg(matid + i) >= (unsigned)nm;
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&g->err, kErrIndex);
}

cudaError_t launch_check_indices(const MeshBufs& m, const BuildBufs& b, cudaStream_t st) {
  if (m.ntri <= 0) return cudaSuccess;
  const int64_t need = (3 * (int64_t)m.ntri + 255) / 256;
  const int grid = (int)(need < (int64_t)num_sms() * 8 ? need : (int64_t)num_sms() * 8);
  k_check_indices<<<grid, 256, 0, st>>>(m.vidx, m.nidx, m.matid, m.ntri, m.nv, m.nn, m.nmat, b.g);
  return cudaGetLastError();
}

cudaError_t launch_refit(const MeshBufs& m, const BuildBufs& b, cudaStream_t st) {
  const int n = m.ntri;
  if (n <= 0) return cudaSuccess;
  k_refit_init<<<1, 256, 0, st>>>(b.g, b.gbox, (int)span_groups(n));
  refit(m, b, st);
  return cudaGetLastError();
}

cudaError_t launch_morton(const float* verts, int nv, const int* vidx, int n, const float* box6, uint32_t* codes,
                          int* err, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int g = min((n + 255) / 256, num_sms() * 8);
  k_morton_only<<<g, 256, 0, st>>>(verts, nv, vidx, n, box6, codes, err);
  return cudaGetLastError();
}

namespace {
bool on_current_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev;
}
bool overlap(const void* a, const void* b, size_t bytes) {
  const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
  return x < y + bytes && y < x + bytes;
}
}  // namespace

const char* sort_args_problem(const uint32_t* kin, const uint32_t* vin, const uint32_t* kout, const uint32_t* vout,
                              int n) {
  if (!kin || !kout || !vout) return "null array";
  const size_t bytes = sizeof(uint32_t) * (size_t)n;
  if (overlap(kin, kout, bytes) || overlap(kin, vout, bytes) || overlap(kout, vout, bytes) ||
      (vin && (overlap(vin, kout, bytes) || overlap(vin, vout, bytes))))
    return "the sort's input and output arrays overlap (it does not sort in place)";
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return "no current CUDA device";
  }
  if (!(on_current_device(kin, dev) && on_current_device(kout, dev) && on_current_device(vout, dev) &&
        (!vin || on_current_device(vin, dev))))
    return "the sort takes device pointers on the current device";
  return nullptr;
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
    onesweep_pass(ki, vi, ko, vo, n, p * kRadixBits, hist + p * kRadix, status + (size_t)p * tiles * kRadix,
                  counters + p, err, st);
    ki = ko;
    vi = vo;
  }
  return cudaGetLastError();
}

}  // namespace crt

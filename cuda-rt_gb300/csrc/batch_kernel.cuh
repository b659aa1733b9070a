// batch_kernel.cuh -- the batched form's persistent kernels: every mesh's
// LBVH build and every mesh's render.
//
// All meshes live in concatenated arrays (mesh m owns triangles
// [tri_off[m], tri_off[m+1]) and internal nodes [tri_off[m] - m,
// tri_off[m+1] - m - 1)).  Child codes in the wide nodes are local to the
// mesh, so each mesh's node and leaf ranges are a self-contained tree for the
// traversal; parent words hold global internal indices; mesh m's virtual
// wide node (its root's children) is NI + m.
//
// k_batch runs the phases below one after another, every block taking part
// in every phase, with a grid-wide barrier between them (the launch is
// cooperative, so all blocks are resident; every barrier wait is bounded and
// reports CRT_TIMEOUT through the batch's error word instead of hanging):
//   init       per-mesh globals, the mesh-id histogram (the mesh sizes),
//              counters
//   bounds     per-mesh scene boxes and largest triangle extents
//   morton     codes against each mesh's own box (kept in codes0 as well),
//              the digit histograms of the three code passes, look-back
//              status cleared
//   sort 0..2  stable LSD passes over the 10-bit code digits (tiles claimed
//              in order, decoupled look-back)
//   mesh keys  each sorted triangle's mesh id
//   sort mesh  one stable pass on the mesh id: triangles grouped by mesh,
//              each mesh's code order unchanged
//   gather     each mesh's sorted codes
//   hierarchy  Karras split search per internal node, on the mesh's codes
//   refit      block-local subtrees of 512 sorted leaves meet in shared
//              memory; climbs that reach a node spanning several chunks are
//              handed on
//   refit top  the handed-on climbs meet at gpu scope
//   render     persistent warps claim (mesh, pixel tile) work items
// The render phase runs either inside k_batch (one launch for everything)
// or alone in k_batch_render after k_batch has run the others (two
// launches); crt_batch_tuning.launches selects the form.
//
// Arrays written in an earlier phase of the launch are read with ordinary
// (coherent) loads, with one exception: the render reads the wide nodes and
// leaf triangles through the read-only path, which is sound because no stale
// copy of them can be in any SM's L1 -- L1 starts empty at each launch, and
// the build phases write them with st.global.cg and read them back only with
// ld.global.cg, both of which bypass L1 -- so the first read of each line
// after the grid barrier fetches it from L2.
#pragma once
#include "build_device.cuh"
#include "pixel.cuh"

namespace crt {

namespace {

enum BatchPhase : int {
  kPhInit = 0,
  kPhBounds,
  kPhMorton,
  kPhSort0,
  kPhSort1,
  kPhSort2,
  kPhMeshKeys,
  kPhSortMesh,
  kPhGather,
  kPhHierarchy,
  kPhRefit,
  kPhRefitTop,
  kPhRender,
  kPhCount
};

// Everything one launch needs (the host fills it; the kernels take its
// fields as separate parameters).
struct BatchLaunch {
  BatchBufs b;
  BatchView v;
  int gmax;         // the most lanes a pixel may take (lanes per pixel option)
  int sort_tiles;   // tiles of one sort pass
  unsigned* bar;    // grid barrier: [0] arrivals, [1] generation (both 0 at launch)
  int first, last;  // the phases to run
};

__device__ __noinline__ void ph_init(const BatchBufs b) {
  const int M = b.M;
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 3; k++) b.g[m].bmin[k] = f2ord(1e9f), b.g[m].bmax[k] = f2ord(-1e9f);
    b.g[m].emax = f2ord(0.f);
    b.g[m].err = 0;
  }
  // passes 0-2: code digits (counted in the morton phase); pass 3: the mesh
  // id, whose histogram is the mesh sizes
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * kRadix; i += gridDim.x * blockDim.x) {
    const int p = i / kRadix, d = i % kRadix;
    b.hist[i] = (p == 3 && d < M) ? (uint32_t)(__ldg(b.tri_off + d + 1) - __ldg(b.tri_off + d)) : 0u;
  }
  // [0..3] sort tiles, [4] render items, [6] refit hand-offs; the error word
  if (blockIdx.x == 0 && threadIdx.x < 8) b.counters[threadIdx.x] = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) *b.err = 0;
}

// Per-mesh scene bounds and largest triangle extent; warps whose lanes share
// a mesh (nearly all) reduce before their atomics.
__device__ __noinline__ void ph_bounds(const BatchBufs b) {
  const int N = b.N;
  const int stride = gridDim.x * blockDim.x;
  for (int t0 = blockIdx.x * blockDim.x; t0 < N; t0 += stride) {
    const int t = t0 + threadIdx.x;
    float lo[3] = {1e9f, 1e9f, 1e9f}, hi[3] = {-1e9f, -1e9f, -1e9f}, e = 0.f;
    bool ok = true;
    int m = -1;
    if (t < N) {
      float3 a, bb, c;
      tri_box(b.verts, b.vidx, t, a, bb, c, lo, hi);
      ok = finite_coords(a, bb, c);
      e = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
      m = __ldg(b.mesh_of + t);
    }
    const unsigned peers = __match_any_sync(0xffffffffu, m);
    if (peers == 0xffffffffu) {  // one mesh in the whole warp
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
          hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
        e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, o));
      }
      ok = __all_sync(0xffffffffu, ok);
      if ((threadIdx.x & 31) != 0) m = -1;
    }
    if (m >= 0) {
#pragma unroll
      for (int k = 0; k < 3; k++) {
        atomicMin(&b.g[m].bmin[k], f2ord(lo[k]));
        atomicMax(&b.g[m].bmax[k], f2ord(hi[k]));
      }
      atomicMax(&b.g[m].emax, f2ord(e));
      if (!ok) atomicOr(&b.g[m].err, kErrNonFinite);
    }
  }
}

// Morton codes against each triangle's own mesh box, a copy of the codes,
// the digit histograms of the three code passes; clears the look-back status.
__device__ __noinline__ void ph_morton(const BatchBufs b, int sort_tiles, uint32_t* sh) {
  const int N = b.N;
  const int status_words = 4 * sort_tiles * kRadix;
  for (int i = threadIdx.x; i < 3 * kRadix; i += blockDim.x) sh[i] = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < status_words; i += gridDim.x * blockDim.x)
    b.status[i] = 0;
  __syncthreads();
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
    float3 a, bb, c;
    float lo[3], hi[3];
    MortonAxis ax[3];
    tri_box(b.verts, b.vidx, t, a, bb, c, lo, hi);
    load_scene_box(b.g + __ldg(b.mesh_of + t), ax);
    const uint32_t code = morton_code(lo, hi, ax);
    b.keys_a[t] = code;
    b.codes0[t] = code;
    for (int p = 0; p < 3; p++) atomicAdd(&sh[p * kRadix + ((code >> (p * kRadixBits)) & (kRadix - 1))], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 3 * kRadix; i += blockDim.x)
    if (sh[i]) atomicAdd(&b.hist[i], sh[i]);
}

// One sort pass: the blocks claim 2048-key tiles in order until none is left
// (each key written straight to its place: with 1024 digits a tile's digit
// runs are two keys long on average, so staging the tile buys little).
template <int TH>
using BatchSortSmem = SortSmem<TH, kSortTile / TH, false>;

template <int TH>
__device__ __noinline__ void ph_sort(const BatchBufs b, int sort_tiles, BatchSortSmem<TH>& sm, int pass,
                                     const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                                     int shift) {
  while (true) {
    if (threadIdx.x == 0) sm.tile = (int)atomicAdd(b.counters + pass, 1u);
    __syncthreads();
    const int tile = sm.tile;
    if (tile >= sort_tiles) break;
    onesweep_tile<TH, kSortTile / TH, false, false>(sm, tile, kin, vin, kout, vout, b.N, shift,
                                                    b.hist + pass * kRadix,
                                                    b.status + (size_t)pass * sort_tiles * kRadix, b.err);
    __syncthreads();
  }
}

__device__ __forceinline__ int mesh_of_internal(const int* __restrict__ tri_off, int M, int gi) {
  // last m with int_off[m] = tri_off[m] - m <= gi
  int lo = 0, hi = M - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(tri_off + mid) - mid <= gi)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// BuildHierarchy per mesh (FindSpan/FindSplit, kernels/bvh.cu:100-207, on
// the mesh's sorted codes), one internal node per thread.
__device__ __noinline__ void ph_hierarchy(const BatchBufs b) {
  const int M = b.M, NI = b.NI;
  for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < NI; gi += gridDim.x * blockDim.x) {
    int m = mesh_of_internal(b.tri_off, M, gi);
    // meshes with one triangle own no internal node: skip to the owner
    while (m + 1 < M && __ldg(b.tri_off + m + 1) - (m + 1) <= gi) m++;
    const int t0 = __ldg(b.tri_off + m);
    const int n = __ldg(b.tri_off + m + 1) - t0;
    const int i = gi - (t0 - m);
    const uint32_t* codes = b.keys_b + t0;
    const uint64_t ki = ((uint64_t)ld_in<false>(codes + i) << 32) | (uint32_t)i;
    const int dd = kdelta<false>(codes, n, ki, i + 1) - kdelta<false>(codes, n, ki, i - 1);
    const int d = dd > 0 ? 1 : (dd < 0 ? -1 : 0);
    const int dmin = kdelta<false>(codes, n, ki, i - d);
    int lmax = 2;
    while (kdelta<false>(codes, n, ki, i + lmax * d) > dmin) lmax *= 2;
    int l = 0, t = lmax;
    do {
      t /= 2;
      if (kdelta<false>(codes, n, ki, i + (l + t) * d) > dmin) l += t;
    } while (t > 1);
    const int lo = min(i, i + l * d), hi = max(i, i + l * d);
    int left = lo, right = hi;
    uint64_t kl = ((uint64_t)ld_in<false>(codes + left) << 32) | (uint32_t)left;
    const int same = kdelta<false>(codes, n, kl, right);
    do {
      const int s = (right + left) / 2;
      if (kdelta<false>(codes, n, kl, s) > same) {
        left = s;
        kl = ((uint64_t)ld_in<false>(codes + left) << 32) | (uint32_t)left;
      } else {
        right = s;
      }
    } while (right > left + 1);
    const int split = left;
    const int c1 = (split == lo) ? ~split : split;
    const int c2 = (split + 1 == hi) ? ~(split + 1) : split + 1;
    const int ib = t0 - m;  // this mesh's first internal node
    const uint32_t spans = ((t0 + lo) / kRefitBlock != (t0 + hi) / kRefitBlock) ? kParentSpans : 0u;
    b.parent[c1 < 0 ? NI + t0 + split : ib + split] = (uint32_t)gi | kParentLeft | spans;
    b.parent[c2 < 0 ? NI + t0 + split + 1 : ib + split + 1] = (uint32_t)gi | spans;
    b.flags[gi] = 0;
    const float4 empty = make_float4(0.f, 0.f, 0.f, __int_as_float(kNoChild));
    if (c1 < 0) __stcg(&b.wnodes[gi].s[1].lo_code, empty);
    if (c2 < 0) __stcg(&b.wnodes[gi].s[3].lo_code, empty);
  }
}

// Shared memory of the refit phase: the children's boxes at each block-local
// node of the chunk (lo xyz, hi xyz) and the nodes' arrival counts.
struct RefitSmem {
  float box[kRefitBlock][2][6];
  int flag[kRefitBlock];
};

// The climb of one leaf (global sorted position k) through the block-local
// nodes of its chunk of kRefitBlock leaves (RefitBounds, kernels/bvh.cu:
// 209-258): the second arrival at a node takes the union; a climb that
// reaches a node spanning several chunks is handed on.
__device__ __forceinline__ void refit_leaf(const BatchBufs& b, RefitSmem& sm, int k0, int k) {
  const int N = b.N, NI = b.NI;
  const int tri = (int)ld_in<false>(b.vals_a + k);
  if ((unsigned)tri >= (unsigned)N) {  // only a corrupt sort gets here
    atomicOr(&b.g[0].err, kErrStack);
    return;
  }
  const int m = __ldg(b.mesh_of + tri);
  const int t0 = __ldg(b.tri_off + m);
  const int n = __ldg(b.tri_off + m + 1) - t0;
  float3 a, bb, c;
  float lo[3], hi[3];
  tri_box(b.verts, b.vidx, tri, a, bb, c, lo, hi);
  float4* lt = reinterpret_cast<float4*>(b.leaves + k);  // st.global.cg: see the note on the render's loads
  __stcg(lt, make_float4(a.x, a.y, a.z, __int_as_float(tri)));
  __stcg(lt + 1, make_float4(bb.x, bb.y, bb.z, 0.f));
  __stcg(lt + 2, make_float4(c.x, c.y, c.z, 0.f));
  if (n == 1) {
#pragma unroll
    for (int q = 0; q < 3; q++) b.g[m].root_box[q] = lo[q], b.g[m].root_box[3 + q] = hi[q];
    return;
  }
  const int root = t0 - m;
  uint32_t w = ld_in<false>(b.parent + NI + k);
  int xc = ~(k - t0);  // codes are local to the mesh
  for (int level = 0;; level++) {
    const int p = (int)(w & kParentMask);
    if (level >= kStackSize || p < root || p >= root + n - 1) {  // only a corrupt tree gets here
      atomicOr(&b.g[m].err, kErrStack);
      return;
    }
    const uint32_t wn = (p == root) ? 0u : ld_in<false>(b.parent + p);
    const bool is_left = (w & kParentLeft) != 0;
    const int gp = (p == root) ? NI + m : (int)(wn & kParentMask);
    const bool p_left = (p == root) || (wn & kParentLeft) != 0;
    if (p != root && (gp < root || gp >= root + n - 1)) {  // only a corrupt tree gets here
      atomicOr(&b.g[m].err, kErrStack);
      return;
    }
    put_wide(b.wnodes, xc, is_left, p, gp, p_left, lo, hi);
    if (!(w & kParentSpans)) {
      const int sl = p + m - k0;  // global leaf position of the node's index, within this chunk
      float* mine = sm.box[sl][is_left ? 0 : 1];
#pragma unroll
      for (int q = 0; q < 3; q++) mine[q] = lo[q], mine[3 + q] = hi[q];
      __threadfence_block();
      if (atomicAdd(&sm.flag[sl], 1) == 0) return;  // first arrival
      __threadfence_block();
      const float* o = sm.box[sl][is_left ? 1 : 0];
#pragma unroll
      for (int q = 0; q < 3; q++) lo[q] = fminf(lo[q], o[q]), hi[q] = fmaxf(hi[q], o[3 + q]);
    } else {  // spanning node: the climb continues in the refit-top phase
      b.arrivals[atomicAdd(b.counters + 6, 1u)] = make_uint2(w, (uint32_t)m);
      return;
    }
    if (p == root) {
#pragma unroll
      for (int q = 0; q < 3; q++) b.g[m].root_box[q] = lo[q], b.g[m].root_box[3 + q] = hi[q];
      return;
    }
    xc = p - root;
    w = wn;
  }
}

// The block takes chunks of kRefitBlock sorted leaves in turn; each thread
// climbs from kRefitBlock / blockDim.x leaves of the chunk, one after
// another (a climb never waits: the first arrival at a node stops).
__device__ __noinline__ void ph_refit(const BatchBufs b, RefitSmem& sm) {
  const int N = b.N;
  const int chunks = (N + kRefitBlock - 1) / kRefitBlock;
  for (int ch = blockIdx.x; ch < chunks; ch += gridDim.x) {
    for (int i = threadIdx.x; i < kRefitBlock; i += blockDim.x) sm.flag[i] = 0;
    __syncthreads();
    const int k0 = ch * kRefitBlock;
    for (int i = threadIdx.x; i < kRefitBlock; i += blockDim.x)
      if (k0 + i < N) refit_leaf(b, sm, k0, k0 + i);
    __syncthreads();
  }
}

// The handed-on climbs through the spanning nodes: each arrival meets its
// sibling at gpu scope (a release/acquire add on the node's flag, whose
// parity tells the second arrival), which takes the union and climbs on.
__device__ __noinline__ void ph_refit_top(const BatchBufs b) {
  const int M = b.M, NI = b.NI;
  const unsigned count = ld_in<false>(b.counters + 6);
  WNode* wnodes = b.wnodes;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const uint2 arr = b.arrivals[i];
    const int m = (int)arr.y;
    if (m < 0 || m >= M) continue;  // only a corrupt arrival gets here
    const int t0 = __ldg(b.tri_off + m), n = __ldg(b.tri_off + m + 1) - t0, root = t0 - m;
    uint32_t w = arr.x;
    int p = (int)(w & kParentMask);
    if (p < root || p >= root + n - 1) {
      atomicOr(&b.g[m].err, kErrStack);
      continue;
    }
    uint32_t wn = (p == root) ? 0u : ld_in<false>(b.parent + p);
    bool is_left = (w & kParentLeft) != 0;
    int gp = (p == root) ? NI + m : (int)(wn & kParentMask);
    bool p_left = (p == root) || (wn & kParentLeft) != 0;
    if (p != root && (gp < root || gp >= root + n - 1)) {
      atomicOr(&b.g[m].err, kErrStack);
      continue;
    }
    float lo[3], hi[3];
    {
      const WSlot* q = wnodes[gp].s + (p_left ? 0 : 2) + (is_left ? 0 : 1);
      const float4 a = __ldcg(&q->lo_code), bb = __ldcg(&q->hi);
      lo[0] = a.x, lo[1] = a.y, lo[2] = a.z, hi[0] = bb.x, hi[1] = bb.y, hi[2] = bb.z;
    }
    for (int level = 0;; level++) {
      const uint32_t wn_next = (p == root) ? 0u : __ldcg(b.parent + gp);
      if ((atomic_add_acq_rel(b.flags + p, 1) & 1) == 0) break;  // first arrival
      sibling_box(wnodes, gp, p_left, is_left, lo, hi);
      if (p == root) {
#pragma unroll
        for (int q = 0; q < 3; q++) b.g[m].root_box[q] = lo[q], b.g[m].root_box[3 + q] = hi[q];
        break;
      }
      const int xc = p - root;
      w = wn;
      p = (int)(w & kParentMask);
      if (level >= kStackSize || p < root || p >= root + n - 1) {
        atomicOr(&b.g[m].err, kErrStack);
        break;
      }
      wn = wn_next;
      is_left = (w & kParentLeft) != 0;
      gp = (p == root) ? NI + m : (int)(wn & kParentMask);
      p_left = (p == root) || (wn & kParentLeft) != 0;
      if (p != root && (gp < root || gp >= root + n - 1)) {
        atomicOr(&b.g[m].err, kErrStack);
        break;
      }
      put_wide(wnodes, xc, is_left, p, gp, p_left, lo, hi);
    }
  }
}

// The render: warps claim work items (mesh, pixel tile) from a counter, with
// per-mesh tile prefix sums item_off[M + 1]; mesh m's pixels take
// lanes_per_pixel(spp, gmax) lanes each; SHORT is the shared-memory part of
// the traversal stack (0: all local).
template <int SHORT>
__device__ __forceinline__ void ph_render(const BatchView& V, int gmax, int2* ring) {
  TravStats ts;
  D3 glight = d3(0, 0, 0);
  const int lane = threadIdx.x & 31;
  int cur = -1;
  DScene S;
  const RenderArgs* Ap = V.args;  // the mesh's arguments, read through L1 rather than held in registers
  float rb[6], B = 0.f, D = 0.f;
  unsigned pred = 0xffffffffu;
  int G = 1, tw = 8, th = 4;
  while (true) {
    int item = 0;
    if (lane == 0) item = (int)atomicAdd(V.counter, 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= V.items) break;
    // mesh of this item: last m with item_off[m] <= item
    int lo = 0, hi = V.M - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(V.item_off + mid) <= item)
        lo = mid;
      else
        hi = mid - 1;
    }
    const int m = lo;
    if (m != cur) {
      cur = m;
      const int t0 = __ldg(V.tri_off + m), n = __ldg(V.tri_off + m + 1) - t0;
      S.ntri = n;
      S.root = n >= 2 ? 0 : ~0;
      S.verts = V.verts, S.normals = V.normals, S.vidx = V.vidx, S.nidx = V.nidx, S.matid = V.matid, S.mats = V.mats;
      S.wnodes = V.wnodes + (t0 - m);
      S.leaves = V.leaves + t0;
      S.g = V.g + m;
      Ap = V.args + m;
      scene_consts(S, rb, B, D);
      G = lanes_per_pixel(Ap->spp, gmax), tw = group_tile_w(G), th = group_tile_h(G);
    }
    const int tile = item - __ldg(V.item_off + m);
    const int W = Ap->W, H = Ap->H;
    const int tiles_x = (W + tw - 1) / tw;
    const int p = lane / G;
    const int px = (tile % tiles_x) * tw + (p % tw);
    const int py = (tile / tiles_x) * th + (p / tw);
    pixel<kRender, SHORT, true>(S, *Ap, px, py, px < W && py < H, G, pred, rb, B, D, ts, glight, ring);
  }
}

// Shared memory of one block: the phases run one at a time, so they share
// one buffer sized for the largest of those launched (the sort tile's, the
// refit's, or the render's traversal-stack ring).
template <int TH>
constexpr size_t batch_smem_bytes(int stack, bool build_phases) {
  constexpr size_t sort = sizeof(BatchSortSmem<TH>);
  constexpr size_t refit = sizeof(RefitSmem);
  constexpr size_t morton = 3 * kRadix * sizeof(uint32_t);
  constexpr size_t a = sort > refit ? sort : refit;
  const size_t build = build_phases ? (a > morton ? a : morton) : 0;
  const size_t ring = (size_t)stack * TH * sizeof(int2);
  return build > ring ? build : ring;
}

// Phases [first, last] of the list above.  The render reads its view
// straight from the kernel's parameters; the build phases get copies of
// theirs.
template <int TH, int SHORT>
__global__ void __launch_bounds__(TH, 1024 / TH) k_batch(const BatchBufs b, const BatchView V, int gmax, int sort_tiles,
                                                        unsigned* bar, int first, int last) {
  extern __shared__ __align__(16) unsigned char smem[];
  BatchSortSmem<TH>& sort_sm = *reinterpret_cast<BatchSortSmem<TH>*>(smem);
  RefitSmem& refit_sm = *reinterpret_cast<RefitSmem*>(smem);
  uint32_t* morton_sm = reinterpret_cast<uint32_t*>(smem);
  int2* ring = SHORT > 0 ? reinterpret_cast<int2*>(smem) + threadIdx.x : nullptr;
  for (int ph = first; ph <= last; ph++) {
    if (ph > first && !grid_barrier(bar, gridDim.x, b.err)) return;
    switch (ph) {
      case kPhInit:
        ph_init(b);
        break;
      case kPhBounds:
        ph_bounds(b);
        break;
      case kPhMorton:
        ph_morton(b, sort_tiles, morton_sm);
        break;
      case kPhSort0:  // keys_a -> keys_b (values 0..N-1)
        ph_sort<TH>(b, sort_tiles, sort_sm, 0, b.keys_a, nullptr, b.keys_b, b.vals_b, 0);
        break;
      case kPhSort1:  // b -> a
        ph_sort<TH>(b, sort_tiles, sort_sm, 1, b.keys_b, b.vals_b, b.keys_a, b.vals_a, kRadixBits);
        break;
      case kPhSort2:  // a -> b
        ph_sort<TH>(b, sort_tiles, sort_sm, 2, b.keys_a, b.vals_a, b.keys_b, b.vals_b, 2 * kRadixBits);
        break;
      case kPhMeshKeys:
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < b.N; j += gridDim.x * blockDim.x)
          b.keys_a[j] = (uint32_t)__ldg(b.mesh_of + ld_in<false>(b.vals_b + j));
        break;
      case kPhSortMesh:  // stable on the mesh id: ids grouped by mesh, by code within
        ph_sort<TH>(b, sort_tiles, sort_sm, 3, b.keys_a, b.vals_b, b.keys_b, b.vals_a, 0);
        break;
      case kPhGather:
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < b.N; j += gridDim.x * blockDim.x)
          b.keys_b[j] = ld_in<false>(b.codes0 + ld_in<false>(b.vals_a + j));
        break;
      case kPhHierarchy:
        ph_hierarchy(b);
        break;
      case kPhRefit:
        ph_refit(b, refit_sm);
        break;
      case kPhRefitTop:
        ph_refit_top(b);
        break;
      case kPhRender:
        ph_render<SHORT>(V, gmax, ring);
        break;
      default:
        break;
    }
  }
}

// The render phase as a kernel of its own, for the two-launch form (k_batch
// runs the build phases, then this): compiled alone, the traversal loop
// keeps more of its state in registers (inside k_batch it spills about a
// quarter more, and the render measured 25% slower on the 256-mesh batch).
template <int TH, int SHORT>
__global__ void __launch_bounds__(TH, 1024 / TH) k_batch_render(const BatchView V, int gmax) {
  extern __shared__ __align__(16) unsigned char smem[];
  int2* ring = SHORT > 0 ? reinterpret_cast<int2*>(smem) + threadIdx.x : nullptr;
  ph_render<SHORT>(V, gmax, ring);
}

}  // namespace

}  // namespace crt

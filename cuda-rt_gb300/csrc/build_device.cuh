// build_device.cuh -- device routines of the LBVH build shared by the plain
// build's kernels (build.cu) and the batched form's persistent kernel
// (batch_kernel.cuh): triangle boxes, Morton codes, the radix-sort tile, the
// augmented-key delta and the wide-node writes of the refit.
#pragma once
#include "crt_internal.h"

namespace crt {

namespace {

constexpr int kSpinLimit = 1 << 20;  // bounded look-back wait (x ~64 ns)

// Programmatic dependent launch.  The plain build launches its kernels as
// programmatic dependents of the kernel before them (launch_dep): a
// dependent's blocks may be scheduled once every block of the kernel before
// it has started, and pdl_wait() holds them until that kernel has completed
// and its writes are visible.  Every build kernel calls pdl_wait() before it
// touches global memory and then lets its own dependents be scheduled, so a
// stage boundary no longer costs a launch.  Launched the ordinary way, both
// instructions are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;"); }

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

// Loads of arrays the build reads.  NC = true: through the read-only cache
// (the array is not written while the kernel runs); NC = false: ordinary
// (coherent) global loads, for a persistent kernel that wrote the array in
// an earlier phase.
template <bool NC>
__device__ __forceinline__ uint32_t ld_in(const uint32_t* p) {
  if (NC) return __ldg(p);
  return __ldca(p);
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

// computeMortonCodesKernel, kernels/bvh.cu:37-61, in double as the reference:
// c = 0.5*(lo+hi), q = (c-mn)/(mx-mn), cell = trunc(RN32(clamp(1024 q))).
static __device__ __noinline__ uint32_t morton_axis_exact(float lo, float hi, double mn, double mx) {
  double c = 0.5 * ((double)lo + (double)hi);
  c = (c - mn) / (mx - mn);
  return morton_axis(c);
}

// Exact sum a + b as an unevaluated pair (s, e): s = RN(a + b), e the error.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Per-axis constants of morton_cell for a scene box [mn, mx]: the extent
// mx - mn as an exact float-float pair (dh, dl), and 1/dh rounded to nearest
// and upwards.  `fast` is false when dh is not positive or lies outside
// [2^-125, 2^125] (the reciprocals are then not normal floats): every cell of
// that axis comes from the double path.
struct MortonAxis {
  float mn, mx, dh, dl, rcp, rcp_up;
  bool fast;
};
__device__ __forceinline__ MortonAxis morton_axis_setup(float mn, float mx) {
  MortonAxis a;
  a.mn = mn;
  a.mx = mx;
  two_sum(mx, -mn, a.dh, a.dl);
  a.fast = a.dh >= 2.3509887e-38f && a.dh <= 4.2535296e37f;  // 2^-125, 2^125
  a.rcp = __frcp_rn(a.dh);
  a.rcp_up = __frcp_ru(a.dh);
  return a;
}

// The same cell without double arithmetic whenever that is provably right.
// y = 1024 (c - mn) / (mx - mn) is formed in float-float: c = (lo + hi)/2,
// c - mn and mx - mn by exact two-sums, then a quotient q1 = nh * RN(1/dh)
// and one correction term from the exact residual (q1*dh split by an FMA).
// q1 is within 2^-23 of nh/dh (relative), the computed residual within
// ~2^-45 |nh|, so y_hi + y_lo is within ~2^-34 |nh| / dh of the exact
// quotient -- far inside E = 2^-30 (|y| + 1024 (|c| + |mn|)/dh), the bound
// the checks below use (|nh| <= |c| + |mn|).  E is evaluated with upward
// rounding and the upward reciprocal, so it never falls below that value.
// The cell is floor(y) unless y sits within half a float ulp (<= 2^-15 below
// 1024) of the next integer, or the bound does not separate y from an
// integer: then the double path decides.  Any overflow or NaN fails every
// check and also goes to the double path.
__device__ __forceinline__ uint32_t morton_cell(float lo, float hi, const MortonAxis& ax) {
  if (ax.fast) {
    const float mn = ax.mn, dh = ax.dh, dl = ax.dl;
    float sh, sl;
    two_sum(lo, hi, sh, sl);
    const float ch = 0.5f * sh, cl = 0.5f * sl;  // exact halving
    float nh, nl;
    two_sum(ch, -mn, nh, nl);
    nl = __fadd_rn(nl, cl);
    const float q1 = __fmul_rn(nh, ax.rcp);
    // r = (nh + nl) - q1 (dh + dl), with q1*dh split exactly by an FMA
    const float ph = __fmul_rn(q1, dh);
    const float pl = __fmaf_rn(q1, dh, -ph);
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(nh, ph), pl), __fsub_rn(nl, __fmul_rn(q1, dl)));
    const float q2 = __fmul_rn(r, ax.rcp);
    const float yh = 1024.f * q1, yl = 1024.f * q2;  // exact scaling
    const float E = __fmul_ru(9.3132257e-10f, __fadd_ru(fabsf(yh), __fmul_ru(1024.f, __fmul_ru(__fadd_ru(fabsf(ch),
                                                                                                   fabsf(mn)), ax.rcp_up))));
    if (__fadd_ru(__fadd_ru(yh, yl), E) < 0.f) return 0u;
    if (__fsub_rd(__fsub_rd(yh, -yl), E) > 1023.f) return 1023u;
    const float fl = floorf(yh);
    if (fl >= 0.f && fl <= 1023.f) {
      const float fr = __fsub_rn(yh, fl);  // exact: fl <= yh < fl + 1
      // need fr + yl in [E, 1 - 2^-14 - E)
      if (__fsub_rd(__fadd_rd(fr, yl), E) >= 0.f && __fadd_ru(__fadd_ru(fr, yl), E) < 0.99993896484375f)
        return (uint32_t)fl;
    }
  }
  return morton_axis_exact(lo, hi, (double)ax.mn, (double)ax.mx);
}

__device__ __forceinline__ uint32_t morton_code(const float lo[3], const float hi[3], const MortonAxis ax[3]) {
  const uint32_t ex = expand_bits(morton_cell(lo[0], hi[0], ax[0]));
  const uint32_t ey = expand_bits(morton_cell(lo[1], hi[1], ax[1]));
  const uint32_t ez = expand_bits(morton_cell(lo[2], hi[2], ax[2]));
  return ex * 4 + ey * 2 + ez;
}

__device__ __forceinline__ void load_scene_box(const SceneGlobals* g, MortonAxis ax[3]) {
#pragma unroll
  for (int k = 0; k < 3; k++) ax[k] = morton_axis_setup(ord2f(g->bmin[k]), ord2f(g->bmax[k]));
}

__device__ __forceinline__ int atomic_add_acq_rel(int* p, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
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
template <int TH>
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
  for (int w = 0; w < TH / 32; w++) {
    const uint32_t s = s_warp[w];
    if (w < warp) wpre += s;
    tot += s;
  }
  __syncthreads();
  total = tot;
  return wpre + x - v;
}

// The same for two values per thread at once (a, b < 2^32 in total over the
// block): returns both exclusive prefixes.
template <int TH>
__device__ __forceinline__ void block_excl_scan2(uint32_t a, uint32_t b, unsigned long long* s_warp, uint32_t& pa,
                                                 uint32_t& pb) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned long long v = ((unsigned long long)a << 32) | b;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  unsigned long long wpre = 0;
  for (int w = 0; w < warp; w++) wpre += s_warp[w];
  __syncthreads();
  const unsigned long long r = wpre + x - v;
  pa = (uint32_t)(r >> 32);
  pb = (uint32_t)r;
}

constexpr uint32_t kFlagAgg = 1u << 30, kFlagInc = 2u << 30, kValMask = (1u << 30) - 1;

constexpr int kBarrierSpinLimit = 1 << 22;  // bounded barrier wait (x ~100 ns)

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// Grid-wide barrier over all `nblocks` blocks: every write made before it by
// any thread of the grid is visible to every thread after it.  Returns false
// (and sets kErrTimeout) when the wait gave up; the caller then stops.
__device__ __noinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, int* err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    const unsigned gen = ld_acquire_u32(bar + 1);
    if (atom_add_acq_rel_u32(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      st_release_u32(bar + 1, gen + 1);
    } else {
      int spins = 0;
      while (ld_acquire_u32(bar + 1) == gen) {
        if (++spins > kBarrierSpinLimit ||
            ((spins & 1023) == 0 && (ld_relaxed(reinterpret_cast<const uint32_t*>(err)) & kErrTimeout))) {
          atomicOr(err, kErrTimeout);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The lanes of the warp whose key has digit d (a 10-bit digit; lanes with
// valid false take part in the votes and match no one): one ballot per digit
// bit, each lane keeping the lanes that agree with it on every bit.  (This
// replaces __match_any_sync, whose issue cost made it the sort's bottleneck.)
__device__ __forceinline__ uint32_t digit_peers(uint32_t d, bool valid) {
  uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
  for (int b = 0; b < kRadixBits; b++) {
    const bool bit = (d >> b) & 1u;
    const uint32_t vote = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? vote : ~vote;
  }
  return peers;
}

// One stable LSD pass over the digit at `shift` (thrust::sort_by_key's
// role, kernels/bvh.cu:267-273).  Tiles of TH * IT keys are claimed in order
// from an atomic counter; within a tile, warps rank their 32 * IT keys in
// input order (digit_peers), and the tile's digit offsets come from a
// decoupled look-back over the tiles before it.  Two shapes (sort_large):
// 2048-key tiles of 256 threads for small inputs, 8192-key tiles of 1024
// threads from 2^19 keys on (a quarter of the tiles, so a quarter of the
// look-back chain; 45 us less per 1M-key build, 20 us more at 100k).
// STAGE: the tile's keys and values are reordered in shared memory and
// written out in order (coalesced runs); otherwise each key goes straight
// to its global position (no staging buffers: for small tiles, whose digit
// runs are short anyway).
template <int TH, int IT, bool STAGE = true>
struct SortSmem {
  uint32_t whist[TH / 32][kRadix / 2];  // per-warp 16-bit digit counters
  uint32_t tstart[kRadix];
  uint32_t gbase[kRadix];
  uint32_t keys[STAGE ? TH * IT : 1];
  uint32_t vals[STAGE ? TH * IT : 1];
  uint32_t warp[TH / 32];
  unsigned long long warp2[TH / 32];
  int tile;
};

// One tile of the pass; all TH threads of the block call it.  NC: the input
// arrays are read through the read-only cache (they are not written while
// the kernel runs); otherwise with ordinary loads.
template <int TH, int IT, bool NC = true, bool STAGE = true>
__device__ __forceinline__ void onesweep_tile(SortSmem<TH, IT, STAGE>& sm, int tile, const uint32_t* __restrict__ kin,
                                              const uint32_t* __restrict__ vin, uint32_t* __restrict__ kout,
                                              uint32_t* __restrict__ vout, int n, int shift,
                                              const uint32_t* __restrict__ ghist, uint32_t* __restrict__ status,
                                              int* err) {
  constexpr int W = TH / 32;
  constexpr int TILE = TH * IT;
  constexpr int DPT = kRadix / TH;  // digits per thread
  static_assert(kRadix % TH == 0 && 32 * IT < 65536, "digits per thread, 16-bit warp counters");
  auto& s_whist = sm.whist;
  auto& s_tstart = sm.tstart;
  auto& s_gbase = sm.gbase;
  auto& s_keys = sm.keys;
  auto& s_vals = sm.vals;
  auto& s_warp = sm.warp;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < W * kRadix / 2; i += TH) (&s_whist[0][0])[i] = 0;
  // global start of each digit: exclusive scan of the pass histogram
  uint32_t gh[DPT], gsum = 0;
#pragma unroll
  for (int j = 0; j < DPT; j++) gh[j] = ld_in<NC>(ghist + DPT * tid + j), gsum += gh[j];
  uint32_t gtot;
  uint32_t gpre = block_excl_scan<TH>(gsum, s_warp, gtot);
  const int base = tile * TILE;
  const uint32_t mask = kRadix - 1;
  uint32_t key[IT], val[IT], rank[IT];
  unsigned short* wh = reinterpret_cast<unsigned short*>(s_whist[warp]);
  const uint32_t lt = lanemask_lt();
#pragma unroll
  for (int r = 0; r < IT; r++) {  // every load issued before the ranking's warp syncs
    const int idx = base + warp * (32 * IT) + r * 32 + lane;
    const bool valid = idx < n;
    key[r] = valid ? ld_in<NC>(kin + idx) : 0u;
    val[r] = valid ? (vin ? ld_in<NC>(vin + idx) : (uint32_t)idx) : 0u;
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
  // per digit: warp offsets (exclusive, in place) and the tile count
  uint32_t cnt[DPT], csum = 0;
#pragma unroll
  for (int j = 0; j < DPT; j++) {
    const int d = DPT * tid + j;
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
  for (int j = 0; j < DPT; j++) st_relaxed(my + DPT * tid + j, (tile == 0 ? kFlagInc : kFlagAgg) | cnt[j]);
  uint32_t pre[DPT];
#pragma unroll
  for (int j = 0; j < DPT; j++) pre[j] = 0;
  if (tile > 0) {
    // The thread's DPT digits walk back together: DPT independent loads
    // per L2 round trip.  A walk stops at the first inclusive prefix.
    int look[DPT];
#pragma unroll
    for (int j = 0; j < DPT; j++) look[j] = tile - 1;
    int spins = 0;
    uint32_t live = (1u << DPT) - 1u;
    while (live) {
      uint32_t sv[DPT];
#pragma unroll
      for (int j = 0; j < DPT; j++)
        sv[j] = (live >> j) & 1 ? ld_relaxed(status + (size_t)look[j] * kRadix + DPT * tid + j) : 0u;
      bool waiting = false;
#pragma unroll
      for (int j = 0; j < DPT; j++) {
        if (!((live >> j) & 1)) continue;
        const uint32_t f = sv[j] & ~kValMask;
        if (f == 0) {
          waiting = true;
          continue;
        }
        pre[j] += sv[j] & kValMask;
        if (f == kFlagInc || look[j] == 0) {
          live &= ~(1u << j);
          st_relaxed(my + DPT * tid + j, kFlagInc | (pre[j] + cnt[j]));
        } else {
          look[j]--;
        }
      }
      if (waiting) {
        // bounded wait; once any wait has timed out, later ones give up at once
        if (++spins > kSpinLimit || ((spins & 1023) == 0 && (ld_relaxed((const uint32_t*)err) & kErrTimeout))) {
          atomicOr(err, kErrTimeout);
#pragma unroll
          for (int j = 0; j < DPT; j++)
            if ((live >> j) & 1) st_relaxed(my + DPT * tid + j, kFlagInc | (pre[j] + cnt[j]));
          break;
        }
        __nanosleep(32);
      }
    }
  }
  uint32_t ctot;
  uint32_t cpre = block_excl_scan<TH>(csum, s_warp, ctot);
  {
    uint32_t c = cpre, g = gpre;
#pragma unroll
    for (int j = 0; j < DPT; j++) {
      const int d = DPT * tid + j;
      s_tstart[d] = c;
      s_gbase[d] = g + pre[j] - c;
      c += cnt[j];
      g += gh[j];
    }
  }
  __syncthreads();
  if constexpr (!STAGE) {
#pragma unroll
    for (int r = 0; r < IT; r++) {
      const int idx = base + warp * (32 * IT) + r * 32 + lane;
      if (idx < n) {
        const uint32_t d = (key[r] >> shift) & mask;
        const uint32_t pos = s_gbase[d] + s_tstart[d] + wh[d] + rank[r];
        kout[pos] = key[r];
        vout[pos] = val[r];
      }
    }
  } else {
#pragma unroll
    for (int r = 0; r < IT; r++) {
      const int idx = base + warp * (32 * IT) + r * 32 + lane;
      if (idx < n) {
        const uint32_t d = (key[r] >> shift) & mask;
        const uint32_t pos = s_tstart[d] + wh[d] + rank[r];
        s_keys[pos] = key[r];
        s_vals[pos] = val[r];
      }
    }
    __syncthreads();
    const int tile_n = min(TILE, n - base);
    for (int i = tid; i < tile_n; i += TH) {
      const uint32_t k = s_keys[i];
      const uint32_t pos = s_gbase[(k >> shift) & mask] + (uint32_t)i;
      kout[pos] = k;
      vout[pos] = s_vals[i];
    }
  }
}

// One pass as a kernel: each block claims the next tile.
template <int TH, int IT>
__global__ void __launch_bounds__(TH) k_onesweep(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                 uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, int n,
                                                 int shift, const uint32_t* __restrict__ ghist,
                                                 uint32_t* __restrict__ status, unsigned* tile_counter, int* err) {
  __shared__ SortSmem<TH, IT> sm;
  pdl_wait();
  pdl_launch_dependents();
  if (threadIdx.x == 0) sm.tile = (int)atomicAdd(tile_counter, 1u);
  __syncthreads();
  onesweep_tile<TH, IT>(sm, sm.tile, kin, vin, kout, vout, n, shift, ghist, status, err);
}

// delta(), kernels/bvh.cu:71-88: with the augmented key (code << 32 | index)
// the common-prefix length is one 64-bit clz -- clz(ci ^ cj) when the codes
// differ, 32 + clz(i ^ j) when they are equal, exactly the reference's two
// cases; -1 out of range.
template <bool NC = true>
__device__ __forceinline__ int kdelta(const uint32_t* __restrict__ c, int n, uint64_t ki, int j) {
  if (j < 0 || j >= n) return -1;
  const uint64_t kj = ((uint64_t)ld_in<NC>(c + j) << 32) | (uint32_t)j;
  return __clzll((long long)(ki ^ kj));
}

// The parent word of a node: parent index | bit 31 when the node is its
// parent's left child | bit 30 when the parent's leaf range crosses a
// kRefitBlock boundary (a spanning node: its box does not come from the
// block-local climbs).
constexpr uint32_t kParentLeft = 1u << 31, kParentSpans = 1u << 30, kParentMask = (1u << 30) - 1;

// The largest m in [0, limit] with pred(m), for a predicate true on a prefix
// of [0, limit] (pred(0) holds): the warp evaluates 32 candidates per round,
// log32 rounds instead of log2 dependent steps.  All 32 lanes call it with
// the same arguments.
template <typename Pred>
__device__ __forceinline__ int warp_prefix_end(int limit, Pred pred) {
  const int lane = threadIdx.x & 31;
  int top = 1;
  while ((int64_t)top * 32 < (int64_t)limit + 1) top *= 32;
  int m = 0;
  for (int stride = top; stride >= 1; stride /= 32) {
    const int64_t cand = (int64_t)m + (int64_t)(lane + 1) * stride;
    const bool ok = cand <= limit && pred((int)cand);
    m += __popc(__ballot_sync(0xffffffffu, ok)) * stride;
  }
  return m;
}

// RefitBounds (kernels/bvh.cu:209-258): one climber per leaf; at each node the
// first arrival stops and the second computes the union (bboxunion,
// bvh.cu:63-69) and climbs on.  min/max are exact, so every schedule gives the
// reference's boxes.  Every box goes to the wide nodes (WNode): child x (code
// xc) of binary node p fills slot 2*side(p) + side(x) of the wide node of p's
// parent gp (for the root, the virtual node past the last internal one), and
// a leaf child also fills its own slot of p's wide node (the hierarchy marks
// the odd slot empty).  Codes are rewritten with the boxes, so a refit alone keeps
// the wide nodes complete, and the children of every node can be read back
// from its parent's wide node (the export does).
//
// A block owns kRefitBlock consecutive sorted leaves.  A node whose leaf
// range lies inside that span has both children's climbers in the block, so
// its two arrivals meet in shared memory with block-scope ordering (most
// nodes).  The single-scene build (k_refit_spans) then takes each node
// spanning several blocks as the union of block and block-edge boxes; the
// batched build meets there too, through a global flag with release/acquire
// at gpu scope, reading the other child's box from the wide node (global
// flags count arrivals; each refit adds exactly two per spanning node, so the
// parity of the old value tells first from second without clearing between
// refits).  Each climb step needs one dependent load: the parent word (index,
// side, spanning bit).
__device__ __forceinline__ void put_wide(WNode* W, int xc, bool x_left, int p, int gp, bool p_left,
                                         const float lo[3], const float hi[3]) {
  const float4 a = make_float4(lo[0], lo[1], lo[2], __int_as_float(xc));
  const float4 b = make_float4(hi[0], hi[1], hi[2], 0.f);
  if (xc < 0) {  // (the hierarchy marked the odd slot empty)
    WSlot* q = W[p].s + (x_left ? 0 : 2);
    __stcg(&q[0].lo_code, a);
    __stcg(&q[0].hi, b);
  }
  WSlot* q = W[gp].s + (p_left ? 0 : 2) + (x_left ? 0 : 1);
  __stcg(&q->lo_code, a);
  __stcg(&q->hi, b);
}

// The box of the other child of p, from the wide node of p's parent.
__device__ __forceinline__ void sibling_box(const WNode* W, int gp, bool p_left, bool x_left, float lo[3],
                                            float hi[3]) {
  const WSlot* q = W[gp].s + (p_left ? 0 : 2) + (x_left ? 1 : 0);
  const float4 a = __ldcg(&q->lo_code), b = __ldcg(&q->hi);
  lo[0] = fminf(lo[0], a.x), lo[1] = fminf(lo[1], a.y), lo[2] = fminf(lo[2], a.z);
  hi[0] = fmaxf(hi[0], b.x), hi[1] = fmaxf(hi[1], b.y), hi[2] = fmaxf(hi[2], b.z);
}

}  // namespace

}  // namespace crt

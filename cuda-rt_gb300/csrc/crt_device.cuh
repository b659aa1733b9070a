// crt_device.cuh -- device data layout and the per-ray arithmetic shared by
// the build, traversal and render kernels.
//
// Exactness: the reference computes in double (inc/vec.h).  Every routine
// named *_exact below performs the reference's double operations in the
// reference's order.  The library is compiled with -fmad=false so no
// multiply-add is contracted into an FMA; together with IEEE division and
// square root (nvcc's defaults) this reproduces the reference's results bit
// for bit.  Routines named cons_* are FP32 filters that may accept more than
// the exact test but never less; every decision that reaches an output is
// taken by an *_exact routine.
#pragma once
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

namespace crt {

constexpr double kRayEps = 0.00000001;  // RAY_EPSILON, inc/common.h:2
constexpr int kStackSize = 64;          // STACK_SIZE, kernels/bvh.cu:379
// The four-wide traversal pushes up to three entries per wide level: trees of
// height < 60 (see CRT_MAX_TRIANGLES) need at most 3 * 30 entries.
constexpr int kWideStack = 96;

// Material (inc/material.h:8-24): the fields shade() and the shadow test read.
struct DMat {
  double ka[3], kd[3], ks[3], kt[3], ke[3];
  double shininess;
};

// Four-wide traversal node (128 bytes, one aligned 8 x 16-byte fetch): the
// binary radix tree with every other level folded in.  Wide node i holds the
// children of binary node i's children, in left-first order: slots 0-1 come
// from the left child, 2-3 from the right; a leaf child takes its even slot
// itself and leaves the odd one empty (code kNoChild).  Per slot: box lo in
// xyz and the child's code (int bits) in w, box hi in xyz.  Child code >= 0:
// internal node index in the reference's numbering (it names both the binary
// node and its wide node); child code < 0: leaf at sorted position ~code.
// The array has one entry more than there are internal nodes: that last,
// virtual node holds the root's two children in slots 0 and 1 (the root
// counts as its left child), so every node's children sit in the wide node
// of its parent.
constexpr int kNoChild = (int)0x80000000;
struct __align__(16) WSlot {
  float4 lo_code;
  float4 hi;
};
struct __align__(128) WNode {
  WSlot s[4];
};

// The triangle of the leaf at sorted position k: its three vertices, the
// triangle id in v0.w (as int bits).
struct __align__(16) LeafTri {
  float4 v0, v1, v2;
};

// Per-scene device globals written by the build kernels.
struct SceneGlobals {
  int bmin[3], bmax[3];  // scene bounds, order-preserving int encoding of floats
  int emax;              // largest per-axis extent of a triangle box (encoded)
  int err;               // CRT_ERR_* bits
  unsigned tile_counter[4];
  unsigned nspan;        // spanning internal nodes listed by the split search
  float root_box[6];     // box of the root (lo xyz, hi xyz)
};

enum : int {
  kErrNonFinite = 1,
  kErrTimeout = 2,
  kErrStack = 4,
  kErrIndex = 8,  // a vertex, normal or material index out of range
};

// Everything a traversal needs, passed by value.
struct DScene {
  int ntri;
  int root;  // 0 (internal) when ntri >= 2, ~0 (leaf 0) when ntri == 1
  const float* verts;
  const float* normals;
  const int* vidx;
  const int* nidx;
  const int* matid;
  const DMat* mats;
  const WNode* wnodes;
  const LeafTri* leaves;
  SceneGlobals* g;
};

// Order-preserving float <-> int encoding for atomicMin/atomicMax.
__device__ __forceinline__ int f2ord(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

// ---------------------------------------------------------------- vectors
struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return d3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// normalize(), inc/vec.h:117-122: the squared length is rounded to float for sqrtf.
__device__ __forceinline__ D3 normalize_exact(D3 a) {
  double s = 1.0 / (double)sqrtf(__double2float_rn(a.x * a.x + a.y * a.y + a.z * a.z));
  return d3(a.x * s, a.y * s, a.z * s);
}
// norm(), inc/vec.h:136-140.
__device__ __forceinline__ double norm_exact(D3 a) {
  return (double)sqrtf(__double2float_rn(a.x * a.x + a.y * a.y + a.z * a.z));
}

// ---------------------------------------------------------------- rays
// Per-ray constants: the double ray for the exact tests, and an FP32 form
// whose rounding is bounded, for filters that decide most tests without
// any double arithmetic.
struct RayC {
  double ox, oy, oz, dx, dy, dz;
  float fox, foy, foz, fdx, fdy, fdz;  // origin, direction rounded to float
  float omax;            // max |origin| component (float, rounded up)
  float ax, ay, az;      // 1/d in float; 0 on a "free" axis
  float lx, ly, lz;      // RD(c - m), c = RN(-o_f * a_f)
  float hx, hy, hz;      // RU(c + m)
  float dprune;          // widening of the entry bound for pruning
  float tau;             // slack on t for pruning
  int sx, sy, sz;        // 1 when 1/d < 0: the box's hi plane is the near one
};

// Slab filter constants.  For a box coordinate b (a float) the exact test
// uses t = (b - o) * a in double, a = 1.0/d.  Here, in float,
//   a_f = RN(1/RN(d)), c = RN(-RN(o) * a_f),
//   |b a_f + c - t| <= 4.1 u |a| (|b| + |o|)      (u = 2^-24),
// and the margin is m = 8 u |a_f| (B + |o_f|), B >= |b| over the scene.  So
//   RD(b a_f + RD(c - m)) <= t <= RU(b a_f + RU(c + m))
// for every slab value the exact test can produce.  An axis whose constants
// do not fit comfortably in float ("free") never decides anything.
//
// Pruning (closest hit only): a triangle the exact test accepts may put its
// plane crossing up to eps outside the triangle (alpha/beta rounding) and its
// t up to tau away from that crossing; eps and tau bound first-order rounding
// of Moller-Trumbore with |det| >= 1e-8 for triangles of diameter <= D, with
// a factor 2^23 of headroom.  A subtree whose entry bound, lowered by
// dprune = eps * max|a|, exceeds best + tau cannot hold a t <= best.
__device__ __forceinline__ void ray_setup(RayC& r, double ox, double oy, double oz, double dx, double dy, double dz,
                                          float B, float D) {
  r.ox = ox, r.oy = oy, r.oz = oz, r.dx = dx, r.dy = dy, r.dz = dz;
  const float fo[3] = {__double2float_rn(ox), __double2float_rn(oy), __double2float_rn(oz)};
  const float fd[3] = {__double2float_rn(dx), __double2float_rn(dy), __double2float_rn(dz)};
  r.fox = fo[0], r.foy = fo[1], r.foz = fo[2];
  r.fdx = fd[0], r.fdy = fd[1], r.fdz = fd[2];
  // |o| rounded up: float rounding of o is at most a relative 2^-24
  const float omax = __fmul_ru(fmaxf(fmaxf(fabsf(fo[0]), fabsf(fo[1])), fabsf(fo[2])), 1.0000002f);
  r.omax = omax;
  const float reach = __fmul_ru(1.7320509f, __fadd_ru(omax, B));
  const float D2 = __fmul_ru(D, D);
  // 2^-29 / 1e-8 and 2^-30 / 1e-8, rounded up
  const float eps = __fmul_ru(__fmul_ru(0.18626452f, D2), __fadd_ru(reach, D));
  r.tau = __fmul_ru(__fmul_ru(0.093132258f, D2), __fadd_ru(__fmul_ru(4.f, reach), D));
  float af[3], lo[3], hi[3], amax = 0.f;
  int sg[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float a = __frcp_rn(fd[k]);  // +-inf for a zero component
    const float aa = fabsf(a);
    const float m = __fmul_ru(__fmul_ru(4.7683724e-07f, aa), __fadd_ru(B, __fmul_ru(fabsf(fo[k]), 1.0000002f)));
    const float c = __fmul_rn(-fo[k], a);
    sg[k] = fd[k] < 0.f ? 1 : 0;  // a zero component makes the axis free
    if (aa <= 1e30f && m <= 1e30f && fabsf(c) <= 1e30f) {
      af[k] = a;
      lo[k] = __fsub_rd(c, m);
      hi[k] = __fadd_ru(c, m);
      amax = fmaxf(amax, aa);
    } else {  // free axis
      af[k] = 0.f;
      lo[k] = __int_as_float(0xff800000);
      hi[k] = __int_as_float(0x7f800000);
    }
  }
  r.ax = af[0], r.ay = af[1], r.az = af[2];
  r.lx = lo[0], r.ly = lo[1], r.lz = lo[2];
  r.hx = hi[0], r.hy = hi[1], r.hz = hi[2];
  r.sx = sg[0], r.sy = sg[1], r.sz = sg[2];
  r.dprune = __fmul_ru(eps, __fmul_ru(amax, 1.0000002f));
}

// The conservative filter: true whenever box_exact is true.  tprune (out):
// a lower bound on the entry t of the box dilated by eps, for pruning.
__device__ __forceinline__ bool box_cons(const RayC& r, float lox, float hix, float loy, float hiy, float loz,
                                         float hiz, float& tprune) {
  const float nx = r.sx ? hix : lox, fx = r.sx ? lox : hix;
  const float ny = r.sy ? hiy : loy, fy = r.sy ? loy : hiy;
  const float nz = r.sz ? hiz : loz, fz = r.sz ? loz : hiz;
  const float L = fmaxf(fmaxf(__fmaf_rd(nx, r.ax, r.lx), __fmaf_rd(ny, r.ay, r.ly)), __fmaf_rd(nz, r.az, r.lz));
  const float U = fminf(fminf(__fmaf_ru(fx, r.ax, r.hx), __fmaf_ru(fy, r.ay, r.hy)), __fmaf_ru(fz, r.az, r.hz));
  tprune = __fsub_rd(L, r.dprune);
  return L <= U;
}

// Certain acceptance: true only when box_exact is certainly true (every
// exact entry value <= every exact exit value).
__device__ __forceinline__ bool box_sure(const RayC& r, float lox, float hix, float loy, float hiy, float loz,
                                         float hiz) {
  const float nx = r.sx ? hix : lox, fx = r.sx ? lox : hix;
  const float ny = r.sy ? hiy : loy, fy = r.sy ? loy : hiy;
  const float nz = r.sz ? hiz : loz, fz = r.sz ? loz : hiz;
  const float L = fmaxf(fmaxf(__fmaf_ru(nx, r.ax, r.hx), __fmaf_ru(ny, r.ay, r.hy)), __fmaf_ru(nz, r.az, r.hz));
  const float U = fminf(fminf(__fmaf_rd(fx, r.ax, r.lx), __fmaf_rd(fy, r.ay, r.ly)), __fmaf_rd(fz, r.az, r.lz));
  return L <= U;
}

// BoundingBox::intersect(const ray&), inc/bbox.h:82-102, in double.  Kept
// out of line: it runs only when the filters are not certain.
static __device__ __noinline__ bool box_exact(double ox, double oy, double oz, double dx, double dy, double dz, float lox,
                                       float hix, float loy, float hiy, float loz, float hiz) {
  const double ix = 1.0 / dx, iy = 1.0 / dy, iz = 1.0 / dz;
  double tminx, tmaxx, tminy, tmaxy, tminz, tmaxz;
  if (ix >= 0) {
    tminx = ((double)lox - ox) * ix;
    tmaxx = ((double)hix - ox) * ix;
  } else {
    tmaxx = ((double)lox - ox) * ix;
    tminx = ((double)hix - ox) * ix;
  }
  if (iy >= 0) {
    tminy = ((double)loy - oy) * iy;
    tmaxy = ((double)hiy - oy) * iy;
  } else {
    tmaxy = ((double)loy - oy) * iy;
    tminy = ((double)hiy - oy) * iy;
  }
  if (iz >= 0) {
    tminz = ((double)loz - oz) * iz;
    tmaxz = ((double)hiz - oz) * iz;
  } else {
    tmaxz = ((double)loz - oz) * iz;
    tminz = ((double)hiz - oz) * iz;
  }
  const double tMin = fmax(fmax(tminx, tminy), tminz);
  const double tMax = fmin(fmin(tmaxx, tmaxy), tmaxz);
  return tMin <= tMax;
}

// Certain rejection for the triangle test (tri_exact): true only when the
// double Moller-Trumbore test certainly rejects.  The FP32 determinant and
// numerators differ from the exact values by at most
//   E_det = K |AB| |d| |AC|,  E_a = K |d| |AC| (|o| + |T|),
//   E_b = K |d| |AB| (|o| + |T|)            (max-norms, K = 2^-16),
// a factor of about 2^2 over a first-order rounding analysis with u = 2^-24
// (the double computation's own error is far smaller).
__device__ __forceinline__ bool tri_reject_sure(const RayC& r, float4 a, float4 b, float4 c) {
  const float ABx = b.x - a.x, ABy = b.y - a.y, ABz = b.z - a.z;
  const float ACx = c.x - a.x, ACy = c.y - a.y, ACz = c.z - a.z;
  const float Px = r.fdy * ACz - r.fdz * ACy;
  const float Py = r.fdz * ACx - r.fdx * ACz;
  const float Pz = r.fdx * ACy - r.fdy * ACx;
  const float det = ABx * Px + ABy * Py + ABz * Pz;
  const float Tx = r.fox - a.x, Ty = r.foy - a.y, Tz = r.foz - a.z;
  const float an = Tx * Px + Ty * Py + Tz * Pz;
  const float Qx = Ty * ABz - Tz * ABy;
  const float Qy = Tz * ABx - Tx * ABz;
  const float Qz = Tx * ABy - Ty * ABx;
  const float bn = r.fdx * Qx + r.fdy * Qy + r.fdz * Qz;
  const float nAB = fmaxf(fmaxf(fabsf(ABx), fabsf(ABy)), fabsf(ABz));
  const float nAC = fmaxf(fmaxf(fabsf(ACx), fabsf(ACy)), fabsf(ACz));
  const float nT = fmaxf(fmaxf(fabsf(Tx), fabsf(Ty)), fabsf(Tz));
  const float nd = fmaxf(fmaxf(fabsf(r.fdx), fabsf(r.fdy)), fabsf(r.fdz));
  const float K = 1.52587890625e-05f;  // 2^-16
  const float ot = __fadd_ru(r.omax, nT);
  const float Ed = __fmul_ru(__fmul_ru(__fmul_ru(K, nAB), nd), nAC);
  const float Ea = __fmul_ru(__fmul_ru(__fmul_ru(K, nd), nAC), ot);
  const float Eb = __fmul_ru(__fmul_ru(__fmul_ru(K, nd), nAB), ot);
  const float ad = fabsf(det);
  if (__fadd_ru(ad, Ed) < 0.99e-8f) return true;  // |det| < 1e-8 for certain
  if (!(ad > Ed)) return false;                  // sign of det not certain
  const float A = det > 0.f ? an : -an, Bv = det > 0.f ? bn : -bn;
  const float Dhi = __fmul_ru(__fadd_ru(ad, Ed), 1.0000001f);
  if (__fadd_ru(A, Ea) < 0.f) return true;                  // alpha < 0
  if (__fsub_rd(A, Ea) > Dhi) return true;                  // alpha > 1
  if (__fadd_ru(Bv, Eb) < 0.f) return true;                 // beta < 0
  if (__fsub_rd(__fsub_rd(__fadd_rd(A, Bv), Ea), Eb) > __fadd_ru(Dhi, __fmul_ru(1e-7f, __fadd_ru(fabsf(A), fabsf(Bv)))))
    return true;                                            // alpha + beta > 1
  return false;
}

struct TriHit {
  double t, alpha, beta;
  bool hit;
};

// BVH_d::intersectTriangle, kernels/bvh.cu:297-371: Moller-Trumbore in
// double without culling; |det| and |t| are compared after rounding to float
// (fabsf on a double); inclusive edges; negative t accepted.  Out of line:
// tri_reject_sure settles most tests first.
static __device__ __noinline__ TriHit tri_exact(double ox, double oy, double oz, double dx, double dy, double dz, float4 a,
                                         float4 b, float4 c) {
  TriHit h;
  h.hit = false;
  const double ax = a.x, ay = a.y, az = a.z;
  const double ABx = (double)b.x - ax, ABy = (double)b.y - ay, ABz = (double)b.z - az;
  const double ACx = (double)c.x - ax, ACy = (double)c.y - ay, ACz = (double)c.z - az;
  const double Px = dy * ACz - dz * ACy;
  const double Py = dz * ACx - dx * ACz;
  const double Pz = dx * ACy - dy * ACx;
  const double det = ABx * Px + ABy * Py + ABz * Pz;
  if ((double)fabsf(__double2float_rn(det)) < kRayEps) return h;
  const double inv = 1 / det;
  const double Tx = ox - ax, Ty = oy - ay, Tz = oz - az;
  const double al = (Tx * Px + Ty * Py + Tz * Pz) * inv;
  if (al < 0 || al > 1) return h;
  const double Qx = Ty * ABz - Tz * ABy;
  const double Qy = Tz * ABx - Tx * ABz;
  const double Qz = Tx * ABy - Ty * ABx;
  const double be = (dx * Qx + dy * Qy + dz * Qz) * inv;
  if (be < 0 || al + be > 1) return h;
  const double tt = (ACx * Qx + ACy * Qy + ACz * Qz) * inv;
  if ((double)fabsf(__double2float_rn(tt)) < kRayEps) return h;
  h.t = tt;
  h.alpha = al;
  h.beta = be;
  h.hit = true;
  return h;
}

struct HitRec {
  double t, alpha, beta;
  int id;
  int pos;  // sorted position of the leaf (its rank in left-first DFS order)
};

// The pruning bound for the current best t, rounded up to float: best +
// tau + 2^-40 |best|.  A subtree with tprune > this bound cannot hold a
// candidate with t <= best, so it can neither win nor tie; skipping it leaves
// the closest hit and its left-first tie-break unchanged.
__device__ __forceinline__ float prune_bound(double best, float tau) {
  return __double2float_ru(best + (double)tau + 9.094947017729282e-13 * fabs(best));
}

// BVH_d::intersect (ANY = false: closest hit, ties to the first hit in
// left-first DFS order) and BVH_d::intersectAny (ANY = true: the first hit
// in that order), kernels/bvh.cu:382-449.  The candidate set is the same as
// the reference's: internal boxes pass a conservative filter (a superset of
// the exact test that is monotone in the box, so a grandchild passing implies
// its parent passes, and a leaf's box passes exactly only if all its
// ancestors pass exactly), and each leaf's box and triangle are tested
// exactly.  Leaves are sorted in left-first DFS order, so the reference's
// closest hit is the candidate with the least (t, sorted position); the
// closest-hit walk visits children nearest first and prunes, the any-hit walk
// keeps the reference's left-first order.  Returns 1 hit, 0 miss, -1 stack
// overflow (impossible for trees of height < 60, see CRT_MAX_TRIANGLES).
// STATS counts visited wide nodes and tested triangles (the traffic model of
// the roofline figure); it changes nothing else.
struct TravStats {
  uint32_t nodes = 0, tris = 0;
};
// The traversal stack: entries live in local memory, or (SHORT > 0) the top
// SHORT entries in a per-thread shared-memory ring (slot i of thread t at
// ring[i * blockDim.x], int2 slots) with older entries spilled to local
// memory.  E is int2 (node, pruning bound) for closest hits and int (node)
// for any hits.
__device__ __forceinline__ int2 to_slot(int2 e) { return e; }
__device__ __forceinline__ int2 to_slot(int e) { return make_int2(e, 0); }
__device__ __forceinline__ void from_slot(int2 s, int2& e) { e = s; }
__device__ __forceinline__ void from_slot(int2 s, int& e) { e = s.x; }
template <int SHORT, typename E>
struct TravStack {
  E local[kWideStack];
  int2* ring;
  int sp = 0;
  __device__ __forceinline__ void push(E e) {
    if (SHORT == 0) {
      local[sp++] = e;
      return;
    }
    const int slot = (sp & (SHORT - 1)) * (int)blockDim.x;
    if (sp >= SHORT) from_slot(ring[slot], local[sp - SHORT]);
    ring[slot] = to_slot(e);
    sp++;
  }
  __device__ __forceinline__ E pop() {
    --sp;
    if (SHORT == 0) return local[sp];
    const int slot = (sp & (SHORT - 1)) * (int)blockDim.x;
    E e;
    from_slot(ring[slot], e);
    if (sp >= SHORT) ring[slot] = to_slot(local[sp - SHORT]);
    return e;
  }
};

__device__ __forceinline__ int2 stack_entry(int node, float t, int2*) { return make_int2(node, __float_as_int(t)); }
__device__ __forceinline__ int stack_entry(int node, float, int*) { return node; }
__device__ __forceinline__ int entry_node(int2 e) { return e.x; }
__device__ __forceinline__ int entry_node(int e) { return e; }
__device__ __forceinline__ float entry_bound(int2 e) { return __int_as_float(e.y); }
__device__ __forceinline__ float entry_bound(int) { return 0.f; }

// Leaf codes carry a flag: bit 30 of ~code set = the leaf's box passed the
// conservative filter but not the certain one, so its exact box test is
// still due (set when the leaf is visited and its triangle is a candidate).  kPop marks "take the next node from the stack".
constexpr int kLeafBoxDue = 1 << 30;
constexpr int kLeafIndex = kLeafBoxDue - 1;
constexpr int kPop = kNoChild;

__device__ __forceinline__ void cswap(float& ta, int& ca, float& tb, int& cb) {
  if (tb < ta) {
    const float t = ta;
    ta = tb, tb = t;
    const int c = ca;
    ca = cb, cb = c;
  }
}

// Warp-synchronous traversal: all 32 lanes of the warp call it together
// (`live` false: the lane has no ray and only takes part in the votes).
// Each round, every lane walks its own stack in FP32 until it reaches its
// next candidate leaf (box filter passed, triangle not certainly rejected)
// or runs out of nodes; then the lanes holding a candidate run the exact
// double tests together.  The double arithmetic is thus issued once per
// round for the whole warp instead of once per lane.  A lane waits at its
// candidate until it is tested, so the pruning bound is current when it
// walks on.
// NC = true reads the nodes and leaf triangles through the read-only cache;
// NC = false uses ordinary (coherent) global loads, cached in L1 as well.
template <bool NC>
__device__ __forceinline__ float4 ld_node(const float4* p) {
  if (NC) return __ldg(p);
  return __ldca(p);
}

template <bool ANY, bool STATS = false, int SHORT = 0, bool NC = true>
__device__ __forceinline__ int traverse(const DScene& S, const RayC& r, const float rb[6], HitRec& h, bool live,
                                        TravStats* ts = nullptr, int2* ring = nullptr) {
  bool run = live && S.ntri > 0;
  bool have = false, err = false;
  float tp;
  if (run && !box_cons(r, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], tp)) run = false;
  int node = S.root;
  float pb = __int_as_float(0x7f800000);  // prune bound; +inf until a hit
  using E = typename std::conditional<ANY, int, int2>::type;
  TravStack<SHORT, E> stk;
  stk.ring = ring;
  int cand = 0;  // the pending candidate's leaf code (with its box flag)
  bool pending = false;
  // a valid tree visits each node at most once per ray; the bound and the
  // index checks only guard against a corrupt tree
  const int max_steps = 2 * S.ntri + 64;  // < 2^31 below CRT_MAX_TRIANGLES
  int steps = 0;
  while (true) {
    // FP32 phase: this lane's next candidate
    while (run && !pending) {
      if (node == kPop) {
        bool next = false;
        while (stk.sp > 0) {
          const E e = stk.pop();
          if (!ANY && entry_bound(e) > pb) continue;
          node = entry_node(e);
          next = true;
          break;
        }
        if (!next) {
          run = false;
          break;
        }
      }
      if (++steps > max_steps || node >= S.ntri - 1 || (node < 0 && (~node & kLeafIndex) >= S.ntri)) {
        err = true;
        run = false;
        break;
      }
      if (node >= 0) {
        if (STATS) ts->nodes++;
        const float4* np = reinterpret_cast<const float4*>(S.wnodes + node);
        float4 q[8];
#pragma unroll
        for (int j = 0; j < 8; j++) q[j] = ld_node<NC>(np + j);
        int c[4];
        float t[4];
        int nhit = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const float4 lo = q[2 * k], hi = q[2 * k + 1];
          c[k] = __float_as_int(lo.w);
          bool hk = c[k] != kNoChild && box_cons(r, lo.x, hi.x, lo.y, hi.y, lo.z, hi.z, t[k]);
          if (!ANY) hk = hk && !(t[k] > pb);
          if (!hk) c[k] = kNoChild;
          if (ANY) t[k] = 0.f;  // pruning bounds are not used
          else if (!hk) t[k] = __int_as_float(0x7f800000);
          nhit += hk ? 1 : 0;
        }
        if (!ANY) {  // nearest first; misses (+inf) sort last
          cswap(t[0], c[0], t[1], c[1]);
          cswap(t[2], c[2], t[3], c[3]);
          cswap(t[0], c[0], t[2], c[2]);
          cswap(t[1], c[1], t[3], c[3]);
          cswap(t[1], c[1], t[2], c[2]);
        }
        if (stk.sp + nhit > kWideStack) {
          err = true;
          run = false;
          break;
        }
        // take the first hit slot now, stack the others so they pop in order
        int next = kPop;
        float tnext = 0.f;
#pragma unroll
        for (int k = 3; k >= 0; k--) {
          if (c[k] != kNoChild) {
            if (next != kPop) stk.push(stack_entry(next, tnext, (E*)nullptr));
            next = c[k];
            tnext = t[k];
          }
        }
        node = next;
      } else {
        if (STATS) ts->tris++;
        const float4* lp = reinterpret_cast<const float4*>(S.leaves + (~node & kLeafIndex));
        const float4 a = ld_node<NC>(lp), b = ld_node<NC>(lp + 1), c = ld_node<NC>(lp + 2);
        if (!tri_reject_sure(r, a, b, c)) {
          cand = node, pending = true;
          // the leaf's box (as the refit computes it from the same vertices)
          // is tested here rather than when the leaf is pushed: one copy of
          // the test in the walk's code, and none for leaves never reached
          if (!box_sure(r, fminf(c.x, fminf(a.x, b.x)), fmaxf(c.x, fmaxf(a.x, b.x)), fminf(c.y, fminf(a.y, b.y)),
                        fmaxf(c.y, fmaxf(a.y, b.y)), fminf(c.z, fminf(a.z, b.z)), fmaxf(c.z, fmaxf(a.z, b.z))))
            cand = ~(~cand | kLeafBoxDue);
        }
        node = kPop;
      }
    }
    // double phase: the lanes holding a candidate, together
    if (__ballot_sync(0xffffffffu, pending) == 0u) break;
    if (pending) {
      const int pos = ~cand & kLeafIndex;
      const float4* lp = reinterpret_cast<const float4*>(S.leaves + pos);
      const float4 a = ld_node<NC>(lp), b = ld_node<NC>(lp + 1), c = ld_node<NC>(lp + 2);
      bool in_box = true;
      if (~cand & kLeafBoxDue) {  // the leaf's box, as the refit computes it from the same vertices
        in_box = box_exact(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, fminf(c.x, fminf(a.x, b.x)),
                           fmaxf(c.x, fmaxf(a.x, b.x)), fminf(c.y, fminf(a.y, b.y)), fmaxf(c.y, fmaxf(a.y, b.y)),
                           fminf(c.z, fminf(a.z, b.z)), fmaxf(c.z, fmaxf(a.z, b.z)));
      }
      pending = false;
      if (in_box) {
        const TriHit th = tri_exact(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, a, b, c);
        if (th.hit && (ANY || !have || th.t < h.t || (th.t == h.t && pos < h.pos))) {
          h.t = th.t, h.alpha = th.alpha, h.beta = th.beta, h.id = __float_as_int(a.w), h.pos = pos;
          have = true;
          if (ANY) run = false;
          else pb = prune_bound(th.t, r.tau);
        }
      }
    }
  }
  return err ? -1 : (have ? 1 : 0);
}

// The scene constants the ray setup needs: B = max |coordinate| of the root
// box, D = sqrt(3) * largest triangle-box extent (a triangle-diameter bound).
__device__ __forceinline__ void scene_consts(const DScene& S, float rb[6], float& B, float& D) {
  const float* p = S.g->root_box;
#pragma unroll
  for (int k = 0; k < 6; k++) rb[k] = p[k];
  B = 0.f;
#pragma unroll
  for (int k = 0; k < 6; k++) B = fmaxf(B, fabsf(rb[k]));
  D = __fmul_ru(1.7320509f, ord2f(S.g->emax));
}

// True when shade()'s Phong term cannot change the colour (material.cu:30-
// 36), so it need not be evaluated: ks = 0 and 0 <= shininess <= 1e6 make
// the term ks * powf(max(0, R.V), shininess) a signed zero (R and V are unit
// vectors, so the base is at most 1 + 2^-21 and the power is finite), and
// d + (+-0) is d unless d is itself a zero; a zero d gives a zero product
// att * d * lcol (or NaN whatever the sign), and I + (+-0) is I unless I is
// -0.  So the colour is the same bit for bit unless some I component is -0.
__device__ __forceinline__ bool phong_vanishes(const DMat& m, const D3& I) {
  const long long neg0 = (long long)0x8000000000000000ull;
  return m.ks[0] == 0.0 && m.ks[1] == 0.0 && m.ks[2] == 0.0 && m.shininess >= 0.0 && m.shininess <= 1e6 &&
         __double_as_longlong(I.x) != neg0 && __double_as_longlong(I.y) != neg0 && __double_as_longlong(I.z) != neg0;
}

// Material::shade's Phong term ks * powf(max(0, R.V), shininess)
// (material.cu:17-20, 30-35) at q with unit light direction L and normal N;
// V is the direction from the eye to q.  Out of line: Lambert materials skip
// it (phong_vanishes), and its powf would sit in the hot loop's code.
static __device__ __noinline__ D3 phong_term(const DMat* __restrict__ m, D3 L, D3 N, D3 q, D3 eye) {
  D3 V = eye - q;
  V = normalize_exact(d3(-V.x, -V.y, -V.z));
  D3 R = (-2.0 * dot(L, N)) * N + L;
  R = normalize_exact(R);
  double sp = dot(R, V);
  sp = (double)powf(__double2float_rn(fmax(0.0, sp)), __double2float_rn(m->shininess));
  return d3(m->ks[0] * sp, m->ks[1] * sp, m->ks[2] * sp);
}

// Smooth normal of a hit, bvh.cu:357-364.
__device__ __forceinline__ D3 hit_normal(const DScene& S, const HitRec& h) {
  const int na = S.nidx[3 * h.id], nb = S.nidx[3 * h.id + 1], nc = S.nidx[3 * h.id + 2];
  const D3 A = d3(S.normals[3 * na], S.normals[3 * na + 1], S.normals[3 * na + 2]);
  const D3 Bn = d3(S.normals[3 * nb], S.normals[3 * nb + 1], S.normals[3 * nb + 2]);
  const D3 Cn = d3(S.normals[3 * nc], S.normals[3 * nc + 1], S.normals[3 * nc + 2]);
  const D3 N = (1.0 - (h.alpha + h.beta)) * A + h.alpha * Bn + h.beta * Cn;
  return normalize_exact(N);
}

// ---------------------------------------------------------------- pixel tiles
// The next tile for the calling warp (one lane calls it), or -1 when every
// tile is taken.  The warp starts in its SM's rectangle r (home set); once
// that is exhausted it helps the lowest-numbered rectangle that may still
// have tiles: counters[R] holds a bound below which every rectangle is
// exhausted, raised by the warps that find one so, so that a warp looking
// for work skips what others have found empty.  Tiles inside a rectangle go
// row by row; each is handed out exactly once.
__device__ __forceinline__ int claim_tile(unsigned* counters, int tiles_x, int tiles_y, int RX, int RY, int& r,
                                          bool& home) {
  const int R = RX * RY;
  unsigned* bound = counters + R;
  while (r < R) {
    const int rx = r % RX, ry = r / RX;
    const int x0 = (int)((int64_t)rx * tiles_x / RX), x1 = (int)((int64_t)(rx + 1) * tiles_x / RX);
    const int y0 = (int)((int64_t)ry * tiles_y / RY), y1 = (int)((int64_t)(ry + 1) * tiles_y / RY);
    const int w = x1 - x0, cnt = w * (y1 - y0);
    if (cnt > 0) {
      const int t = (int)atomicAdd(counters + r, 1u);
      if (t < cnt) return (y0 + t / w) * tiles_x + x0 + t % w;
    }
    if (home) {  // the home rectangle is done: on to the lowest one that may not be
      home = false;
      r = (int)*(volatile unsigned*)bound;
      continue;
    }
    atomicMax(bound, (unsigned)(r + 1));
    r = max(r + 1, (int)*(volatile unsigned*)bound);
  }
  return -1;
}
__device__ __forceinline__ int home_region(int RX, int RY) {
  unsigned smid;
  asm("mov.u32 %0, %%smid;" : "=r"(smid));
  return (int)(smid % (unsigned)(RX * RY));
}

// ---------------------------------------------------------------- mrand
// kernels/mrand.cu:3-41.
__device__ __forceinline__ uint32_t xorshift32(uint32_t& s) {
  s ^= (s << 13);
  s ^= (s >> 17);
  s ^= (s << 5);
  return s;
}
__device__ __forceinline__ uint32_t wang_hash(uint32_t seed) {
  seed = (seed ^ 61) ^ (seed >> 16);
  seed *= 9;
  seed = seed ^ (seed >> 4);
  seed *= 0x27d4eb2d;
  seed = seed ^ (seed >> 15);
  return seed;
}
// randDouble: the 32-bit draw is rounded to float, then scaled by 2^-32.
__device__ __forceinline__ double draw_value(float f) { return (double)f * 2.3283064365386963e-10; }
__device__ __forceinline__ double rand_double(uint32_t& s) {
  const uint32_t v = xorshift32(s);
  return draw_value(__uint2float_rn(v));
}

// ---------------------------------------------------------------- lens
// A draw is (double)(float)v * 2^-32, so it takes one of kLensValues values:
// the floats that are integers in [0, 2^32], 2^24 below 2^24 and 2^23 in each
// of the eight binades above.  lens_index numbers them densely.
constexpr uint32_t kLensValues = 83886081u;
__device__ __forceinline__ uint32_t lens_index(float f) {
  return f < 16777216.f ? (uint32_t)f : 16777216u + (__float_as_uint(f) - 0x4B800000u);
}
__device__ __forceinline__ float lens_value(uint32_t i) {
  return i < 16777216u ? (float)i : __uint_as_float(0x4B800000u + (i - 16777216u));
}
// cos and sin of the lens angle 2*pi*u and sqrt(u) of the lens radius draw
// u, as runRayTracerKernelRec computes them (raytracer.cu:141-142).  Out of
// line: with the lens tables the pixel kernels never call them, and code
// inside the hot loop costs instruction-cache misses even when skipped.
static __device__ __noinline__ void lens_angle(double u, double& ca, double& sa) {
  sincos(2 * 3.14159265358979323846 * u, &sa, &ca);
}
static __device__ __noinline__ double lens_root(double u) { return sqrt(u); }

// Table loads that neither allocate in L1 nor keep their lines in L2 ahead
// of other data (an evict-first L2 policy): the lens tables are read at
// random, once per sample, and would otherwise push BVH nodes and the
// threads' local memory out of L2.
__device__ __forceinline__ uint64_t evict_first_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ double2 ld_stream(const double2* p) {
  double2 v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
               : "=d"(v.x), "=d"(v.y)
               : "l"(p), "l"(evict_first_policy()));
  return v;
}
__device__ __forceinline__ double ld_stream(const double* p) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(evict_first_policy()));
  return v;
}

// The thin-lens origin of one sample (raytracer.cu:141-144): two draws, the
// angle's and the radius's, and (dofRadius cos, dofRadius sin, 0).  With
// tables (cs[i] = cos/sin and sq[i] = sqrt at draw value i, built from the
// same expressions) the double sincos and sqrt become two loads; the result
// is the same either way.  A zero radius gives +-0 components, which no later
// operation can tell apart from 0.
__device__ __forceinline__ void lens_origin(const double2* cs, const double* sq, double aperture, uint32_t& st,
                                            double& ox, double& oy) {
  const float f1 = __uint2float_rn(xorshift32(st)), f2 = __uint2float_rn(xorshift32(st));
  const double root = sq ? ld_stream(sq + lens_index(f2)) : lens_root(draw_value(f2));
  const double dofRadius = aperture * root / 2.0;
  ox = 0.0, oy = 0.0;
  if (dofRadius != 0.0) {
    double ca, sa;
    if (cs) {
      const double2 c = ld_stream(cs + lens_index(f1));
      ca = c.x, sa = c.y;
    } else {
      lens_angle(draw_value(f1), ca, sa);
    }
    ox = dofRadius * ca, oy = dofRadius * sa;
  }
}

}  // namespace crt

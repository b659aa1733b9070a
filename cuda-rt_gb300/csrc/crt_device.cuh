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
#include <cuda_runtime.h>

namespace crt {

constexpr double kRayEps = 0.00000001;  // RAY_EPSILON, inc/common.h:2
constexpr int kStackSize = 64;          // STACK_SIZE, kernels/bvh.cu:379

// Material (inc/material.h:8-24): the fields shade() and the shadow test read.
struct DMat {
  double ka[3], kd[3], ks[3], kt[3], ke[3];
  double shininess;
};

// Traversal node: the boxes of both children plus their codes (64 bytes, one
// aligned 4 x 16-byte fetch).  Child code >= 0: internal node index in the
// reference's numbering; child code < 0: leaf at sorted position ~code.
struct __align__(16) BNode {
  float4 xy_l;  // left  child lo.x, hi.x, lo.y, hi.y
  float4 xy_r;  // right child lo.x, hi.x, lo.y, hi.y
  float4 z_lr;  // left lo.z, hi.z, right lo.z, hi.z
  int4 child;   // left code, right code, -, -
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
  float root_box[6];     // box of the root (lo xyz, hi xyz)
};

enum : int {
  kErrNonFinite = 1,
  kErrTimeout = 2,
  kErrStack = 4,
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
  const BNode* nodes;
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
// Per-ray constants: the double ray for the exact tests, and an FP32 copy
// with error margins for the conservative box filter.
struct RayC {
  double ox, oy, oz, dx, dy, dz;
  double ix, iy, iz;     // 1.0/d, as bbox.h:88 computes it
  float fox, foy, foz;   // origin rounded to float
  float fix, fiy, fiz;   // 1/d rounded to float; 0 on a "free" axis
  float mx, my, mz;      // accept margins (t units); +inf on a free axis
  float px, py, pz;      // prune margins: accept margin + box dilation
  float tau;             // slack on t for pruning
};

// Conservative-filter bounds (derivation in the design notes):
//  |t_f32 - t_f64| <= 4.01 u |a| (|b| + |e|), u = 2^-24, for a slab value
//  t = (b - e) * a; the margin uses 8u (a factor 2 of headroom) and B >= |b|.
//  Pruning a subtree is safe when its dilated-box entry bound exceeds the
//  best t by tau; eps bounds how far a double Moller-Trumbore hit can fall
//  outside its triangle (alpha/beta rounding) and tau how far its t can be
//  off (see prune_ok).  Both carry a 2^23 factor of headroom over a
//  first-order rounding analysis with |det| >= 1e-8.
__device__ __forceinline__ void ray_setup(RayC& r, double ox, double oy, double oz, double dx, double dy, double dz,
                                          float B, float D) {
  r.ox = ox, r.oy = oy, r.oz = oz, r.dx = dx, r.dy = dy, r.dz = dz;
  r.ix = 1.0 / dx, r.iy = 1.0 / dy, r.iz = 1.0 / dz;
  const double omax = fmax(fmax(fabs(ox), fabs(oy)), fabs(oz));
  const double Dd = (double)D;
  const double reach = 1.7320508075688772 * (omax + (double)B);
  const double eps = 1.862645149230957e-09 * Dd * Dd * (reach + Dd) / 1e-8;          // 2^-29
  const double tau = 9.313225746154785e-10 * Dd * Dd * (4.0 * reach + Dd) / 1e-8;    // 2^-30
  r.tau = __double2float_ru(tau);
  double o[3] = {ox, oy, oz}, a[3] = {r.ix, r.iy, r.iz};
  float fo[3], fi[3], m[3], p[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double aa = fabs(a[k]);
    const double md = 4.76837158203125e-07 * aa * ((double)B + fabs(o[k])) + 1e-30;  // 8 * 2^-24
    const double pd = md + eps * aa;
    fo[k] = __double2float_rn(o[k]);
    if (aa <= 1e30 && md <= 1e30 && pd <= 1e30) {
      fi[k] = __double2float_rn(a[k]);
      m[k] = __double2float_ru(md);
      p[k] = __double2float_ru(pd);
    } else {  // free axis: this slab never rejects in the filter
      fi[k] = 0.f;
      m[k] = __int_as_float(0x7f800000);
      p[k] = __int_as_float(0x7f800000);
    }
  }
  r.fox = fo[0], r.foy = fo[1], r.foz = fo[2];
  r.fix = fi[0], r.fiy = fi[1], r.fiz = fi[2];
  r.mx = m[0], r.my = m[1], r.mz = m[2];
  r.px = p[0], r.py = p[1], r.pz = p[2];
}

// Conservative slab filter: true whenever the exact double test
// (box_exact) is true.  tprune: a lower bound on the entry t of the dilated
// box, for pruning.
__device__ __forceinline__ bool box_cons(const RayC& r, float lox, float hix, float loy, float hiy, float loz,
                                         float hiz, float& tprune) {
  const float x1 = __fmul_rn(__fsub_rn(lox, r.fox), r.fix), x2 = __fmul_rn(__fsub_rn(hix, r.fox), r.fix);
  const float y1 = __fmul_rn(__fsub_rn(loy, r.foy), r.fiy), y2 = __fmul_rn(__fsub_rn(hiy, r.foy), r.fiy);
  const float z1 = __fmul_rn(__fsub_rn(loz, r.foz), r.fiz), z2 = __fmul_rn(__fsub_rn(hiz, r.foz), r.fiz);
  const float ax = fminf(x1, x2), bx = fmaxf(x1, x2);
  const float ay = fminf(y1, y2), by = fmaxf(y1, y2);
  const float az = fminf(z1, z2), bz = fmaxf(z1, z2);
  const float L = fmaxf(fmaxf(__fsub_rd(ax, r.mx), __fsub_rd(ay, r.my)), __fsub_rd(az, r.mz));
  const float U = fminf(fminf(__fadd_ru(bx, r.mx), __fadd_ru(by, r.my)), __fadd_ru(bz, r.mz));
  tprune = fmaxf(fmaxf(__fsub_rd(ax, r.px), __fsub_rd(ay, r.py)), __fsub_rd(az, r.pz));
  return L <= U;
}

// BoundingBox::intersect(const ray&), inc/bbox.h:82-102, in double.
__device__ __forceinline__ bool box_exact(const RayC& r, float lox, float hix, float loy, float hiy, float loz,
                                          float hiz) {
  double tminx, tmaxx, tminy, tmaxy, tminz, tmaxz;
  if (r.ix >= 0) {
    tminx = ((double)lox - r.ox) * r.ix;
    tmaxx = ((double)hix - r.ox) * r.ix;
  } else {
    tmaxx = ((double)lox - r.ox) * r.ix;
    tminx = ((double)hix - r.ox) * r.ix;
  }
  if (r.iy >= 0) {
    tminy = ((double)loy - r.oy) * r.iy;
    tmaxy = ((double)hiy - r.oy) * r.iy;
  } else {
    tmaxy = ((double)loy - r.oy) * r.iy;
    tminy = ((double)hiy - r.oy) * r.iy;
  }
  if (r.iz >= 0) {
    tminz = ((double)loz - r.oz) * r.iz;
    tmaxz = ((double)hiz - r.oz) * r.iz;
  } else {
    tmaxz = ((double)loz - r.oz) * r.iz;
    tminz = ((double)hiz - r.oz) * r.iz;
  }
  const double tMin = fmax(fmax(tminx, tminy), tminz);
  const double tMax = fmin(fmin(tmaxx, tmaxy), tmaxz);
  return tMin <= tMax;
}

// BVH_d::intersectTriangle, kernels/bvh.cu:297-371: Moller-Trumbore in
// double without culling; |det| and |t| are compared after rounding to float
// (fabsf on a double); inclusive edges; negative t accepted.
__device__ __forceinline__ bool tri_exact(const RayC& r, float4 a, float4 b, float4 c, double& t, double& alpha,
                                          double& beta) {
  const double ax = a.x, ay = a.y, az = a.z;
  const double ABx = (double)b.x - ax, ABy = (double)b.y - ay, ABz = (double)b.z - az;
  const double ACx = (double)c.x - ax, ACy = (double)c.y - ay, ACz = (double)c.z - az;
  const double Px = r.dy * ACz - r.dz * ACy;
  const double Py = r.dz * ACx - r.dx * ACz;
  const double Pz = r.dx * ACy - r.dy * ACx;
  const double det = ABx * Px + ABy * Py + ABz * Pz;
  if ((double)fabsf(__double2float_rn(det)) < kRayEps) return false;
  const double inv = 1 / det;
  const double Tx = r.ox - ax, Ty = r.oy - ay, Tz = r.oz - az;
  const double al = (Tx * Px + Ty * Py + Tz * Pz) * inv;
  if (al < 0 || al > 1) return false;
  const double Qx = Ty * ABz - Tz * ABy;
  const double Qy = Tz * ABx - Tx * ABz;
  const double Qz = Tx * ABy - Ty * ABx;
  const double be = (r.dx * Qx + r.dy * Qy + r.dz * Qz) * inv;
  if (be < 0 || al + be > 1) return false;
  const double tt = (ACx * Qx + ACy * Qy + ACz * Qz) * inv;
  if ((double)fabsf(__double2float_rn(tt)) < kRayEps) return false;
  t = tt;
  alpha = al;
  beta = be;
  return true;
}

struct HitRec {
  double t, alpha, beta;
  int id;
};

// The pruning rule: a subtree whose dilated-box entry bound exceeds the
// best t by more than tau (plus 2^-40 |best| for the rounding of the double
// slab values themselves) cannot hold a candidate with t <= best, so it can
// neither win nor tie; skipping it leaves the closest hit and its left-first
// tie-break unchanged.
__device__ __forceinline__ bool prune_ok(float tprune, float tau, double best) {
  return (double)tprune > best + (double)tau + 9.094947017729282e-13 * fabs(best);
}

// BVH_d::intersect (ANY = false: closest hit, ties to the first hit in
// left-first DFS order) and BVH_d::intersectAny (ANY = true: the first hit
// in that order), kernels/bvh.cu:382-449.  The candidate set is the same as
// the reference's: internal boxes pass a conservative filter (a superset of
// the exact test, and a leaf's box passes exactly only if all its ancestors
// pass exactly), each leaf's box and triangle are tested exactly, and leaves
// are visited in the reference's order.  Returns 1 hit, 0 miss, -1 stack
// overflow (impossible for trees of height < 64, see CRT_MAX_TRIANGLES).
// STATS counts visited internal nodes and tested triangles (the traffic
// model of the roofline figure); it changes nothing else.
struct TravStats {
  uint32_t nodes = 0, tris = 0;
};
template <bool ANY, bool STATS = false>
__device__ __forceinline__ int traverse(const DScene& S, const RayC& r, float rb[6], HitRec& h,
                                        TravStats* ts = nullptr) {
  if (S.ntri <= 0) return 0;
  float tp;
  if (!box_cons(r, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5], tp)) return 0;
  int node = S.root;
  if (node < 0 && !box_exact(r, rb[0], rb[3], rb[1], rb[4], rb[2], rb[5])) return 0;
  bool have = false;
  int2 stack[kStackSize];
  int sp = 0;
  // a valid tree visits each node at most once per ray; the bound and the
  // index checks only guard against a corrupt tree
  const int64_t max_steps = 2 * (int64_t)S.ntri + 64;
  for (int64_t steps = 0;; steps++) {
    if (steps > max_steps || node >= S.ntri - 1 || ~node >= S.ntri) return -1;
    if (node >= 0) {
      if (STATS) ts->nodes++;
      const float4* np = reinterpret_cast<const float4*>(S.nodes + node);
      const float4 xl = __ldg(np + 0), xr = __ldg(np + 1), zz = __ldg(np + 2);
      const int4 ch = __ldg(reinterpret_cast<const int4*>(np + 3));
      float tl, tr;
      bool hl = box_cons(r, xl.x, xl.y, xl.z, xl.w, zz.x, zz.y, tl);
      bool hr = box_cons(r, xr.x, xr.y, xr.z, xr.w, zz.z, zz.w, tr);
      if (hl && ch.x < 0) hl = box_exact(r, xl.x, xl.y, xl.z, xl.w, zz.x, zz.y);
      if (hr && ch.y < 0) hr = box_exact(r, xr.x, xr.y, xr.z, xr.w, zz.z, zz.w);
      if (!ANY && have) {
        if (hl && prune_ok(tl, r.tau, h.t)) hl = false;
        if (hr && prune_ok(tr, r.tau, h.t)) hr = false;
      }
      if (hl) {
        if (hr) {
          if (sp >= kStackSize) return -1;
          stack[sp++] = make_int2(ch.y, __float_as_int(tr));
        }
        node = ch.x;
        continue;
      }
      if (hr) {
        node = ch.y;
        continue;
      }
    } else {
      if (STATS) ts->tris++;
      const float4* lp = reinterpret_cast<const float4*>(S.leaves + (~node));
      const float4 a = __ldg(lp), b = __ldg(lp + 1), c = __ldg(lp + 2);
      double t, al, be;
      if (tri_exact(r, a, b, c, t, al, be)) {
        if (ANY) {
          h.t = t, h.alpha = al, h.beta = be, h.id = __float_as_int(a.w);
          return 1;
        }
        if (!have || t < h.t) {
          h.t = t, h.alpha = al, h.beta = be, h.id = __float_as_int(a.w);
          have = true;
        }
      }
    }
    // pop
    bool next = false;
    while (sp > 0) {
      const int2 e = stack[--sp];
      if (!ANY && have && prune_ok(__int_as_float(e.y), r.tau, h.t)) continue;
      node = e.x;
      next = true;
      break;
    }
    if (!next) break;
  }
  return have ? 1 : 0;
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

// Smooth normal of a hit, bvh.cu:357-364.
__device__ __forceinline__ D3 hit_normal(const DScene& S, const HitRec& h) {
  const int na = S.nidx[3 * h.id], nb = S.nidx[3 * h.id + 1], nc = S.nidx[3 * h.id + 2];
  const D3 A = d3(S.normals[3 * na], S.normals[3 * na + 1], S.normals[3 * na + 2]);
  const D3 Bn = d3(S.normals[3 * nb], S.normals[3 * nb + 1], S.normals[3 * nb + 2]);
  const D3 Cn = d3(S.normals[3 * nc], S.normals[3 * nc + 1], S.normals[3 * nc + 2]);
  const D3 N = (1.0 - (h.alpha + h.beta)) * A + h.alpha * Bn + h.beta * Cn;
  return normalize_exact(N);
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
__device__ __forceinline__ double rand_double(uint32_t& s) {
  const uint32_t v = xorshift32(s);
  return (double)__uint2float_rn(v) * 2.3283064365386963e-10;
}

}  // namespace crt

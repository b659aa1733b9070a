// crt_oracle.cpp -- CPU restatement of cuda-rt's ray-tracing hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the tests, the
// smoke check and the CPU-baseline leg of bench.py load it to check (or to
// time beside) the CUDA product.  The product library never links, loads or
// calls it, and nothing in the product falls back to it.
//
// Every routine restates one piece of the reference (mbartling/cuda-rt) in
// plain C++ double arithmetic, keeping the reference's order of operations
// and its float roundings, so that results are bit-identical to the
// reference's semantics under IEEE-754 round-to-nearest with no FMA
// contraction (build with -ffp-contract=off).  Citations are path:line in the
// reference project.
//
// Data model: the reference keeps vertices as double (Vec3d); the synthetic
// inputs here are FP32 and are widened exactly to double on load.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// RAY_EPSILON, inc/common.h:2
constexpr double kRayEps = 0.00000001;

struct V3 {
  double x, y, z;
};
// Vec3d arithmetic, inc/vec.h:55-115 (component order and association kept).
inline V3 v3(double x, double y, double z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(double s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 mulc(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }  // operator%
inline V3 cross(V3 a, V3 b) {                                                 // operator^
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// normalize(): 1.0/sqrtf(sum of squares) -- the sum is rounded to float
// before the square root (inc/vec.h:117-122).
inline V3 normalize(V3 a) {
  double s = 1.0 / (double)sqrtf((float)(a.x * a.x + a.y * a.y + a.z * a.z));
  return v3(a.x * s, a.y * s, a.z * s);
}
// norm(): sqrtf of the float-rounded squared length (inc/vec.h:136-140).
inline double norm(V3 a) { return (double)sqrtf((float)(a.x * a.x + a.y * a.y + a.z * a.z)); }
// minimum()/maximum() apply fminf/fmaxf, rounding each double to float
// (inc/vec.h:157-165).
inline V3 vmin(V3 a, V3 b) {
  return v3(fminf((float)a.x, (float)b.x), fminf((float)a.y, (float)b.y), fminf((float)a.z, (float)b.z));
}
inline V3 vmax(V3 a, V3 b) {
  return v3(fmaxf((float)a.x, (float)b.x), fmaxf((float)a.y, (float)b.y), fmaxf((float)a.z, (float)b.z));
}
inline double comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }

struct Box {
  V3 lo, hi;
};

// BoundingBox::intersect(const ray&), inc/bbox.h:82-102 (Kay/Kajiya slabs;
// accepts iff tMin <= tMax, with no test against t >= 0).
inline bool box_hit(const Box& b, V3 e, V3 d) {
  double a[3] = {1.0 / d.x, 1.0 / d.y, 1.0 / d.z};
  double tmin[3], tmax[3];
  for (int i = 0; i < 3; i++) {
    double ei = comp(e, i);
    if (a[i] >= 0) {
      tmin[i] = (comp(b.lo, i) - ei) * a[i];
      tmax[i] = (comp(b.hi, i) - ei) * a[i];
    } else {
      tmax[i] = (comp(b.lo, i) - ei) * a[i];
      tmin[i] = (comp(b.hi, i) - ei) * a[i];
    }
  }
  double tMin = fmax(fmax(tmin[0], tmin[1]), tmin[2]);
  double tMax = fmin(fmin(tmax[0], tmax[1]), tmax[2]);
  return tMin <= tMax;
}

// ExpandBits, kernels/bvh.cu:13-21.
inline uint32_t expand_bits(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}
// One axis of CalculateMortonCode, kernels/bvh.cu:25-27:
// (float)min(max(p*1024.0f, 0.0f), 1023.0f) with the double max/min
// ignoring NaN, then truncation to unsigned.
inline uint32_t morton_axis(double p) {
  double s = p * 1024.0;
  s = fmax(s, 0.0);
  s = fmin(s, 1023.0);
  return (uint32_t)(float)s;
}

struct Material {
  double ka[3], kd[3], ks[3], kt[3], ke[3];
  double shininess;
};

struct Scene {
  int nv = 0, nn = 0, ntri = 0, nmat = 0;
  std::vector<V3> verts, normals;
  std::vector<int> vidx, nidx, matid;
  std::vector<Material> mats;
  // build products (reference layout: internal nodes 0..N-2, leaves N-1..2N-2)
  V3 smin{}, smax{};
  std::vector<Box> tri_box;          // Scene_d::BBoxs
  std::vector<int> codes_unsorted;   // mortonCodes before the sort
  std::vector<int> codes;            // mortonCodes after the sort
  std::vector<uint32_t> ids;         // object_ids after the sort
  std::vector<int> parent, left, right;
  std::vector<Box> nbox;             // sortedBBoxs
};

inline V3 vert(const Scene& s, int tri, int k) { return s.verts[s.vidx[3 * tri + k]]; }

// computeTriangleBoundingBox, kernels/scene.cu:120-130.
Box tri_bounds(const Scene& s, int tri) {
  V3 a = vert(s, tri, 0), b = vert(s, tri, 1), c = vert(s, tri, 2);
  Box bb;
  bb.hi = vmax(a, b);
  bb.lo = vmin(a, b);
  bb.hi = vmax(c, bb.hi);
  bb.lo = vmin(c, bb.lo);
  return bb;
}

// delta(), kernels/bvh.cu:71-88: common-prefix length of the codes, with the
// index as a tie-breaker for equal codes and -1 out of range.
inline int delta(const int* codes, int n, int i1, int i2) {
  int l = std::min(i1, i2), r = std::max(i1, i2);
  if (l < 0 || r >= n) return -1;
  int lc = codes[l], rc = codes[r];
  auto clz = [](uint32_t x) { return x ? __builtin_clz(x) : 32; };
  return lc != rc ? clz((uint32_t)(lc ^ rc)) : 32 + clz((uint32_t)(l ^ r));
}

// sign(), kernels/bvh.cu:92-99.
inline int fsign(float x) {
  if (x > 0) return 1;
  if (x < 0) return -1;
  return 0;
}

// FindSpan, kernels/bvh.cu:100-133.
void find_span(const int* c, int n, int idx, int* lo, int* hi) {
  int d = fsign((float)(delta(c, n, idx, idx + 1) - delta(c, n, idx, idx - 1)));
  int dmin = delta(c, n, idx, idx - d);
  int lmax = 2;
  while (delta(c, n, idx, idx + lmax * d) > dmin) lmax *= 2;
  int l = 0, t = lmax;
  do {
    t /= 2;
    if (delta(c, n, idx, idx + (l + t) * d) > dmin) l = l + t;
  } while (t > 1);
  *lo = std::min(idx, idx + l * d);
  *hi = std::max(idx, idx + l * d);
}

// FindSplit, kernels/bvh.cu:134-162.
int find_split(const int* c, int n, int left, int right) {
  int same = delta(c, n, left, right);
  do {
    int s = (right + left) / 2;
    if (delta(c, n, left, s) > same)
      left = s;
    else
      right = s;
  } while (right > left + 1);
  return left;
}

void build(Scene& s) {
  const int n = s.ntri;
  s.tri_box.resize(n);
  // computeBoundingBoxes_kernel, kernels/scene.cu:88-108
  for (int i = 0; i < n; i++) s.tri_box[i] = tri_bounds(s, i);
  // Scene_d::findMinMax, kernels/scene.cu:72-85: fold of minimum/maximum from
  // (+1e9) / (-1e9).  min and max are exact, so the fold order is immaterial.
  V3 mn = v3(1e9, 1e9, 1e9), mx = v3(-1e9, -1e9, -1e9);
  for (int i = 0; i < n; i++) {
    mn = vmin(mn, s.tri_box[i].lo);
    mx = vmax(mx, s.tri_box[i].hi);
  }
  s.smin = mn;
  s.smax = mx;
  // computeMortonCodesKernel, kernels/bvh.cu:37-61
  s.codes_unsorted.resize(n);
  for (int i = 0; i < n; i++) {
    const Box& b = s.tri_box[i];
    V3 c = 0.5 * (b.lo + b.hi);
    c.x = (c.x - mn.x) / (mx.x - mn.x);
    c.y = (c.y - mn.y) / (mx.y - mn.y);
    c.z = (c.z - mn.z) / (mx.z - mn.z);
    uint32_t xx = expand_bits(morton_axis(c.x));
    uint32_t yy = expand_bits(morton_axis(c.y));
    uint32_t zz = expand_bits(morton_axis(c.z));
    s.codes_unsorted[i] = (int)(xx * 4 + yy * 2 + zz);
  }
  // BVH_d::sortMortonCodes, kernels/bvh.cu:267-273: thrust::sort_by_key on
  // (int code, uint id) with ids = 0..N-1, a stable ascending sort.
  std::vector<uint32_t> perm(n);
  for (int i = 0; i < n; i++) perm[i] = (uint32_t)i;
  std::stable_sort(perm.begin(), perm.end(),
                   [&](uint32_t a, uint32_t b) { return s.codes_unsorted[a] < s.codes_unsorted[b]; });
  s.codes.resize(n);
  s.ids = perm;
  for (int i = 0; i < n; i++) s.codes[i] = s.codes_unsorted[perm[i]];
  // BuildHierarchy, kernels/bvh.cu:164-207.  The root's parent is never
  // written by the reference; it is reported here as -1.
  const int nn = n > 0 ? 2 * n - 1 : 0;
  s.parent.assign(nn, -1);
  s.left.assign(nn, 0);
  s.right.assign(nn, 0);
  s.nbox.assign(nn, Box{});
  const int* c = s.codes.data();
  for (int g = 0; g < n; g++) {
    int leaf = (n - 1) + g;
    s.left[leaf] = s.right[leaf] = (int)s.ids[g];
    s.nbox[leaf] = s.tri_box[s.ids[g]];
  }
  for (int g = 0; g < n - 1; g++) {
    int lo, hi;
    find_span(c, n, g, &lo, &hi);
    int split = find_split(c, n, lo, hi);
    int c1 = (split == lo) ? (n - 1) + split : split;
    int c2 = (split + 1 == hi) ? (n - 1) + split + 1 : split + 1;
    s.left[g] = c1;
    s.right[g] = c2;
    s.parent[c1] = g;
    s.parent[c2] = g;
  }
  // RefitBounds, kernels/bvh.cu:209-258: one climber per leaf, the second
  // arrival at a node unions its children (bboxunion, bvh.cu:63-69).  A
  // sequential schedule is one valid interleaving; min/max make every
  // interleaving give the same boxes.  With one triangle there is nothing to
  // refit (the reference would read the root's unwritten parent).
  if (n >= 2) {
    std::vector<int> flags(n - 1, 0);
    for (int g = 0; g < n; g++) {
      int idx = (n - 1) + g;
      do {
        idx = s.parent[idx];
        if (flags[idx]) {
          Box b;
          b.lo = vmin(s.nbox[s.left[idx]].lo, s.nbox[s.right[idx]].lo);
          b.hi = vmax(s.nbox[s.left[idx]].hi, s.nbox[s.right[idx]].hi);
          s.nbox[idx] = b;
        } else {
          flags[idx] = 1;
          break;
        }
      } while (idx != 0);
    }
  }
}

// Refit on fixed topology: new vertex positions, same nodes.  This is
// RefitBounds (kernels/bvh.cu:209-258) run on the existing hierarchy after
// the leaf boxes are recomputed (computeTriangleBoundingBox, scene.cu:120).
void refit(Scene& s) {
  const int n = s.ntri;
  for (int i = 0; i < n; i++) s.tri_box[i] = tri_bounds(s, i);
  for (int g = 0; g < n; g++) s.nbox[(n - 1) + g] = s.tri_box[s.ids[g]];
  if (n >= 2) {
    std::vector<int> flags(n - 1, 0);
    for (int g = 0; g < n; g++) {
      int idx = (n - 1) + g;
      do {
        idx = s.parent[idx];
        if (flags[idx]) {
          Box b;
          b.lo = vmin(s.nbox[s.left[idx]].lo, s.nbox[s.right[idx]].lo);
          b.hi = vmax(s.nbox[s.left[idx]].hi, s.nbox[s.right[idx]].hi);
          s.nbox[idx] = b;
        } else {
          flags[idx] = 1;
          break;
        }
      } while (idx != 0);
    }
  }
}

struct Hit {
  double t;
  V3 N;
  int id;
  double alpha, beta;
};

// BVH_d::intersectTriangle, kernels/bvh.cu:297-371 (Moller-Trumbore in
// double, no culling: |det| and |t| are compared after rounding to float by
// fabsf; negative t is accepted).
bool tri_hit(const Scene& s, V3 p, V3 d, int tri, Hit* h) {
  V3 a = vert(s, tri, 0), b = vert(s, tri, 1), c = vert(s, tri, 2);
  V3 AB = b - a;
  V3 AC = c - a;
  V3 P = cross(d, AC);
  double det = dot(AB, P);
  if (fabsf((float)det) < kRayEps) return false;
  double inv = 1 / det;
  V3 T = p - a;
  double alpha = dot(T, P) * inv;
  if (alpha < 0 || alpha > 1) return false;
  V3 Q = cross(T, AB);
  double beta = dot(d, Q) * inv;
  if (beta < 0 || alpha + beta > 1) return false;
  double t = dot(AC, Q) * inv;
  if (fabsf((float)t) < kRayEps) return false;
  h->t = t;
  h->id = tri;
  h->alpha = alpha;
  h->beta = beta;
  return true;
}

// The smooth normal of a hit (bvh.cu:357-364): barycentric blend of the
// vertex normals, then normalize().
V3 hit_normal(const Scene& s, const Hit& h) {
  int tri = h.id;
  V3 na = s.normals[s.nidx[3 * tri + 0]];
  V3 nb = s.normals[s.nidx[3 * tri + 1]];
  V3 nc = s.normals[s.nidx[3 * tri + 2]];
  V3 N = (1.0 - (h.alpha + h.beta)) * na + h.alpha * nb + h.beta * nc;
  return normalize(N);
}

constexpr int kStack = 64;  // STACK_SIZE, kernels/bvh.cu:379

// BVH_d::intersect (closest hit), kernels/bvh.cu:382-414, and
// BVH_d::intersectAny (first hit in DFS order), bvh.cu:416-449.
// Returns 1 hit, 0 miss, -1 stack overflow (the reference returns false).
int traverse(const Scene& s, V3 p, V3 d, bool any, Hit* out) {
  if (s.ntri == 0) return 0;
  int stack[kStack];
  int top = kStack;
  stack[--top] = 0;
  bool have = false;
  Hit cur;
  while (top != kStack) {
    int node = stack[top++];
    if (!box_hit(s.nbox[node], p, d)) continue;
    if (s.left[node] == s.right[node]) {  // LEAFNODE, inc/bvh.cuh:25
      if (tri_hit(s, p, d, s.left[node], &cur)) {
        if (!have || cur.t < out->t) {
          *out = cur;
          have = true;
          if (any) return 1;
        }
      }
    } else {
      if (top - 2 < 0) return -1;
      stack[--top] = s.right[node];
      stack[--top] = s.left[node];
    }
  }
  return have ? 1 : 0;
}

// mrand stream, kernels/mrand.cu:3-41.
inline uint32_t xorshift(uint32_t& st) {
  st ^= (st << 13);
  st ^= (st >> 17);
  st ^= (st << 5);
  return st;
}
inline uint32_t wang_hash(uint32_t seed) {
  seed = (seed ^ 61) ^ (seed >> 16);
  seed *= 9;
  seed = seed ^ (seed >> 4);
  seed *= 0x27d4eb2d;
  seed = seed ^ (seed >> 15);
  return seed;
}
// randDouble: the uint is rounded to float, then scaled by 2^-32 in double.
inline double rand_double(uint32_t& st) {
  uint32_t v = xorshift(st);
  return (double)((float)v * 1.0 / 4294967296.0);
}

// randVec3d (kernels/mrand.cu:33-35) is Vec3d(randDouble(), randDouble(),
// randDouble()): the order in which a compiler evaluates the three
// constructor arguments decides which draw lands in which component.
// g_light_order[i] is the component that the i-th draw goes to ({0, 1, 2}:
// left to right).
int g_light_order[3] = {0, 1, 2};
inline void light_draws(uint32_t& st, double r[3]) {
  for (int i = 0; i < 3; i++) r[g_light_order[i]] = rand_double(st);
}

}  // namespace

extern "C" {

// Which component each of randVec3d's three draws goes to (a permutation of
// 0, 1, 2); returns -1 and changes nothing for anything else.
int orc_set_light_draw_order(int first, int second, int third) {
  const int o[3] = {first, second, third};
  int seen = 0;
  for (int i = 0; i < 3; i++) {
    if (o[i] < 0 || o[i] > 2) return -1;
    seen |= 1 << o[i];
  }
  if (seen != 7) return -1;
  for (int i = 0; i < 3; i++) g_light_order[i] = o[i];
  return 0;
}

struct orc_material {  // one reference Material (inc/material.h:8-24), the fields shade() reads
  double ka[3], kd[3], ks[3], kt[3], ke[3];
  double shininess;
};

struct orc_camera {  // the Camera getters the pixel kernel reads (inc/camera.h)
  double fov;         // degrees, vertical
  double focal_point; // getFocalPoint()
  double fstop;       // getAperature() = 1/fstop
  double eye[3];      // getEye() (Camera() sets the origin)
};

struct orc_light {  // Light_h, inc/Light.h:7-29 (positional light)
  double color[3];
  double position[3];
  double radius;
  double constant_term, linear_term, quadratic_term;
};

// Material::shade (kernels/material.cu:6-40) at the closest hit hh of the ray
// (org, dir), N its smooth normal, with the positional Light: getDirection
// takes three draws from st (Light.cu:71-80), distanceAttenuation
// (Light.cu:56-68), shadowAttenuation from q = r.at(t) with no offset
// (Light.cu:5-37).  *sh: 1 occluded, 0 lit; *shid: the occluder or -1;
// *overflow counts stack overflows of the shadow ray.
static V3 shade_hit(const Scene& s, const orc_camera* cam, const orc_light* light, V3 org, V3 dir, const Hit& hh,
                    V3 N, uint32_t& st, int* sh, int* shid, int* overflow) {
  const V3 lpos = v3(light->position[0], light->position[1], light->position[2]);
  const V3 lcol = v3(light->color[0], light->color[1], light->color[2]);
  const V3 eye = v3(cam->eye[0], cam->eye[1], cam->eye[2]);
  V3 q = org + (hh.t * dir);
  const Material& m = s.mats[s.matid[hh.id]];
  V3 I = v3(m.ke[0] + m.ka[0] * 0.0, m.ke[1] + m.ka[1] * 0.0, m.ke[2] + m.ka[2] * 0.0);
  V3 Vv = eye - q;
  Vv = v3(-Vv.x, -Vv.y, -Vv.z);
  Vv = normalize(Vv);
  double r[3];
  light_draws(st, r);
  V3 off = v3(r[0], r[1], r[2]) * light->radius;
  off = v3(off.x - 0.5, off.y - 0.5, off.z - 0.5);
  V3 L = normalize(lpos + off - q);
  double dist = norm(lpos - q);
  double fall = light->constant_term + (light->linear_term + light->quadratic_term * dist) * dist;
  fall = (fabs(fall) < kRayEps) ? 1.0 : 1.0 / fall;
  double datt = fmin(1.0, fall);
  V3 satt = v3(1, 1, 1);
  Hit sh_hit;
  int sres = traverse(s, q, L, true, &sh_hit);
  if (sres < 0) (*overflow)++;
  *sh = 0;
  *shid = -1;
  if (sres > 0 && sh_hit.t < norm(lpos - q)) {
    const Material& om = s.mats[s.matid[sh_hit.id]];
    if (sh_hit.t < kRayEps) {
      satt = v3(1, 1, 1);
    } else {
      *sh = 1;
      *shid = sh_hit.id;
      // Trans() is isZero(kt) (inc/material.h:31), so an opaque
      // occluder (kt = 0) passes kd % (1 - kt).
      bool trans = om.kt[0] == 0 && om.kt[1] == 0 && om.kt[2] == 0;
      if (trans)
        satt = v3(om.kd[0] * (1 - om.kt[0]), om.kd[1] * (1 - om.kt[1]), om.kd[2] * (1 - om.kt[2]));
      else
        satt = v3(0, 0, 0);
    }
  }
  V3 att = datt * satt;
  double lam = dot(N, L);
  if (lam < 0) lam = 0;
  V3 diffuse = v3(m.kd[0] * lam, m.kd[1] * lam, m.kd[2] * lam);
  V3 R = (-2.0 * dot(L, N)) * N + L;
  R = normalize(R);
  double sp = dot(R, Vv);
  sp = (double)powf((float)fmax(0.0, sp), (float)m.shininess);
  V3 spec = v3(m.ks[0] * sp, m.ks[1] * sp, m.ks[2] * sp);
  return I + mulc(mulc(att, diffuse + spec), lcol);
}

// traceRay (kernels/raytracer.cu:169-249) with the reflection and refraction
// block of raytracer.cu:196-237 (commented out in the reference) taking
// part: after shade(), while depth > 0, a reflective material (kr != 0)
// adds kr % traceRay(reflected ray, depth - 1), then a transmissive one
// (kt != 0) adds kt % traceRay(refracted ray, depth - 1) unless the ray is
// totally internally reflected.  The block tests Refl()/Trans(), which
// setBools() defines as isZero(kr)/isZero(kt) (inc/material.h:27-31), so
// as written it would trace the rays of materials that cannot reflect and
// add nothing; this restatement takes the evident intent (trace when the
// coefficient is non-zero).  Secondary rays start at q = r.at(t) with no
// offset and use the same closest-hit search as primary rays (negative t
// accepted, |t| < RAY_EPSILON rejected).  optics[4*m]: kr xyz, ior of
// material m.  Draws from st in the recursion's order (depth first).
static V3 trace_rec(const Scene& s, const orc_camera* cam, const orc_light* light, const double* optics, V3 org,
                    V3 dir, int depth, uint32_t& st, int* overflow, Hit* first, int* first_res, int64_t* counts) {
  Hit hh;
  int res = traverse(s, org, dir, false, &hh);
  if (res < 0) (*overflow)++;
  if (first) *first = hh, *first_res = res;
  counts[0]++;
  if (res <= 0) return v3(0.9, 0.9, 0.9);
  counts[1]++;
  const V3 N = hit_normal(s, hh);
  int sh, shid;
  V3 c = shade_hit(s, cam, light, org, dir, hh, N, st, &sh, &shid, overflow);
  if (depth <= 0) return c;
  const V3 q = org + (hh.t * dir);
  const int mid = s.matid[hh.id];
  const Material& m = s.mats[mid];
  const double* o = optics + 4 * (size_t)mid;
  if (!(o[0] == 0 && o[1] == 0 && o[2] == 0)) {
    V3 Rdir = (-2.0 * dot(dir, N)) * N + dir;
    Rdir = normalize(Rdir);
    V3 v = trace_rec(s, cam, light, optics, q, Rdir, depth - 1, st, overflow, nullptr, nullptr, counts);
    c = c + mulc(v3(o[0], o[1], o[2]), v);
  }
  if (!(m.kt[0] == 0 && m.kt[1] == 0 && m.kt[2] == 0)) {
    V3 n = N;
    const V3 rd = dir;
    const V3 mrd = v3(-rd.x, -rd.y, -rd.z);
    const V3 rcos = n * dot(mrd, n);
    const V3 rsin = rcos + rd;
    const double etai = 1.0, etat = o[3];
    double eta;
    if (dot(rd, n) < 0) {
      eta = etai / etat;
      n = v3(-n.x, -n.y, -n.z);
    } else {
      eta = etat / etai;
    }
    const V3 tsin = eta * rsin;
    const double TIR = 1 - dot(tsin, tsin);
    if (TIR >= 0) {
      const V3 tcos = n * sqrt(TIR);
      V3 Tdir = tcos + tsin;
      Tdir = normalize(Tdir);
      V3 v = trace_rec(s, cam, light, optics, q, Tdir, depth - 1, st, overflow, nullptr, nullptr, counts);
      c = c + mulc(v3(m.kt[0], m.kt[1], m.kt[2]), v);
    }
  }
  return c;
}

void* orc_scene_create(int nv, const float* verts, int nn, const float* normals, int ntri,
                       const int* vidx, const int* nidx, int nmat, const orc_material* mats,
                       const int* matid) {
  Scene* s = new (std::nothrow) Scene;
  if (!s) return nullptr;
  s->nv = nv;
  s->nn = nn;
  s->ntri = ntri;
  s->nmat = nmat;
  s->verts.resize(nv);
  for (int i = 0; i < nv; i++) s->verts[i] = v3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  s->normals.resize(nn);
  for (int i = 0; i < nn; i++) s->normals[i] = v3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
  s->vidx.assign(vidx, vidx + 3 * (size_t)ntri);
  if (nidx)
    s->nidx.assign(nidx, nidx + 3 * (size_t)ntri);
  else
    s->nidx = s->vidx;
  if (matid)
    s->matid.assign(matid, matid + ntri);
  else
    s->matid.assign(ntri, 0);
  s->mats.resize(nmat);
  for (int m = 0; m < nmat; m++) {
    Material& M = s->mats[m];
    std::memcpy(&M, &mats[m], sizeof(Material));
  }
  build(*s);
  return s;
}

void orc_scene_destroy(void* h) { delete (Scene*)h; }

// New vertex positions on the same triangles: refit (fixed topology) or a
// full rebuild.
void orc_scene_set_vertices(void* h, const float* verts, int rebuild) {
  Scene* s = (Scene*)h;
  for (int i = 0; i < s->nv; i++) s->verts[i] = v3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  if (rebuild)
    build(*s);
  else
    refit(*s);
}

// Export of the build products.  boxes: 6 floats per entry (lo xyz, hi xyz);
// the reference holds them as doubles but every value is a float.
void orc_export(void* h, double* smin3, double* smax3, int* codes_unsorted, int* codes, uint32_t* ids,
                int* nodes3, float* node_boxes, float* tri_boxes) {
  Scene* s = (Scene*)h;
  const int n = s->ntri, nn = n > 0 ? 2 * n - 1 : 0;
  if (smin3) {
    smin3[0] = s->smin.x, smin3[1] = s->smin.y, smin3[2] = s->smin.z;
  }
  if (smax3) {
    smax3[0] = s->smax.x, smax3[1] = s->smax.y, smax3[2] = s->smax.z;
  }
  if (codes_unsorted) std::memcpy(codes_unsorted, s->codes_unsorted.data(), n * sizeof(int));
  if (codes) std::memcpy(codes, s->codes.data(), n * sizeof(int));
  if (ids) std::memcpy(ids, s->ids.data(), n * sizeof(uint32_t));
  auto put = [](float* dst, const Box& b) {
    dst[0] = (float)b.lo.x, dst[1] = (float)b.lo.y, dst[2] = (float)b.lo.z;
    dst[3] = (float)b.hi.x, dst[4] = (float)b.hi.y, dst[5] = (float)b.hi.z;
  };
  for (int i = 0; i < nn; i++) {
    if (nodes3) {
      nodes3[3 * i] = s->parent[i];
      nodes3[3 * i + 1] = s->left[i];
      nodes3[3 * i + 2] = s->right[i];
    }
    if (node_boxes) put(node_boxes + 6 * i, s->nbox[i]);
  }
  if (tri_boxes)
    for (int i = 0; i < n; i++) put(tri_boxes + 6 * i, s->tri_box[i]);
}

// Trace n rays (6 doubles each: origin, direction).  any=0: closest hit
// (BVH_d::intersect); any=1: first hit in DFS order (BVH_d::intersectAny).
// ids[i] = triangle id or -1; t[i]; normal3 (closest only, optional).
// Returns the number of rays whose traversal overflowed the 64-entry stack.
int orc_trace(void* h, const double* rays, int n, int any, int* ids, double* t, double* normal3,
              int nthreads) {
  const Scene* s = (const Scene*)h;
  int overflow = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : overflow)
#endif
  for (int i = 0; i < n; i++) {
    const double* r = rays + 6 * (size_t)i;
    Hit hh;
    int res = traverse(*s, v3(r[0], r[1], r[2]), v3(r[3], r[4], r[5]), any != 0, &hh);
    if (res < 0) overflow++;
    if (res > 0) {
      ids[i] = hh.id;
      if (t) t[i] = hh.t;
      if (normal3 && !any) {
        V3 N = hit_normal(*s, hh);
        normal3[3 * i] = N.x, normal3[3 * i + 1] = N.y, normal3[3 * i + 2] = N.z;
      }
    } else {
      ids[i] = -1;
      if (t) t[i] = 0.0;
    }
  }
  return overflow;
}

// The pixel kernel runRayTracerKernelRec (kernels/raytracer.cu:95-166) with
// traceRay (raytracer.cu:169-249), Material::shade (kernels/material.cu:6-40)
// and the positional Light (kernels/Light.cu:5-86), for rows [row0, row1) of
// a W x H image (py counted from the top as in the reference), spp samples.
//
// Outputs (memory index idx = (H-py-1)*W + px, bottom-up as in the reference):
//   rgb8[3*idx]           (unsigned char)(255*clamp(mean)) (inc/raytracer.h:53-63)
//   color[3*idx]          the mean before clamping (optional)
//   hit_id[idx*spp + k]   closest-hit triangle of sample k, -1 miss (optional)
//   hit_t[idx*spp + k]    its t (optional)
//   shadow[idx*spp + k]   1 if the shadow ray's first hit occluded the light,
//                         0 if lit, -1 if the primary ray missed (optional)
//   shadow_id[idx*spp+k]  the occluding triangle when shadow is 1, else -1 (optional)
//   rays_out[(idx*spp+k)*6]  the primary ray (optional)
// rays_in (optional) replaces the generated primary ray of every sample; the
// random draws are still consumed as in the reference.  seed: 0 for the
// reference's streams; otherwise seed * 0x9E3779B1 is XORed into each pixel's
// hash input (the library's independent-render mode).
// Returns the number of stack overflows.
int orc_render(void* h, const orc_camera* cam, const orc_light* light, int W, int H, int spp, int row0,
               int row1, uint8_t* rgb8, double* color, int* hit_id, double* hit_t, int* shadow,
               const double* rays_in, double* rays_out, int nthreads, int* shadow_id, uint32_t seed) {
  const Scene* s = (const Scene*)h;
  const int gx = (W + 15) / 16;  // gridDim.x of the 16x16 launch (raytracer.cu:56-58)
  int overflow = 0;
  const double invW = 1.0 / double(W), invH = 1.0 / double(H);
  const double aspect = double(W) / double(H);
  const double angle = tan(M_PI * 0.5 * cam->fov / 180.0f);  // raytracer.cu:130
  const double aperture = 1 / cam->fstop;  // Camera::getAperature
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for collapse(2) schedule(dynamic, 64) reduction(+ : overflow)
#endif
  for (int py = row0; py < row1; py++) {
    for (int px = 0; px < W; px++) {  // pixels are independent: all cores share any band of rows
      const int idx = (H - py - 1) * W + px;
      // getGlobalIdx_2D_2D (inc/indexing.h:4-9) for block (px/16, py/16),
      // thread (px%16, py%16); initPNRG seeds it with wangHash.
      uint32_t g = (uint32_t)(((py / 16) * gx + px / 16) * 256 + (py % 16) * 16 + (px % 16));
      uint32_t st = wang_hash(g ^ (seed * 0x9E3779B1u));  // seed 0: the reference's stream
      double xx = (2 * ((px + 0.5) * invW) - 1) * angle * aspect;
      double yy = (1 - 2 * ((py + 0.5) * invH)) * angle;
      V3 acc = v3(0, 0, 0);
      for (int k = 0; k < spp; k++) {
        const size_t si = (size_t)idx * spp + k;
        double dofAngle = 2 * M_PI * rand_double(st);
        double dofRadius = aperture * sqrt(rand_double(st)) / 2.0;
        V3 org = v3(dofRadius * cos(dofAngle), dofRadius * sin(dofAngle), 0);
        V3 dir = v3(xx, yy, -1.0);
        dir = normalize(dir) * cam->focal_point - org;
        dir = normalize(dir);
        if (rays_in) {
          const double* r = rays_in + 6 * si;
          org = v3(r[0], r[1], r[2]);
          dir = v3(r[3], r[4], r[5]);
        }
        if (rays_out) {
          double* r = rays_out + 6 * si;
          r[0] = org.x, r[1] = org.y, r[2] = org.z, r[3] = dir.x, r[4] = dir.y, r[5] = dir.z;
        }
        // traceRay, raytracer.cu:169-249
        Hit hh;
        int res = traverse(*s, org, dir, false, &hh);
        if (res < 0) overflow++;
        V3 col;
        int sh = -1, shid = -1;
        if (res > 0)
          col = shade_hit(*s, cam, light, org, dir, hh, hit_normal(*s, hh), st, &sh, &shid, &overflow);
        else
          col = v3(0.9, 0.9, 0.9);
        acc = acc + col;
        if (hit_id) hit_id[si] = res > 0 ? hh.id : -1;
        if (hit_t) hit_t[si] = res > 0 ? hh.t : 0.0;
        if (shadow) shadow[si] = sh;
        if (shadow_id) shadow_id[si] = shid;
      }
      acc = v3(acc.x / double(spp), acc.y / double(spp), acc.z / double(spp));
      if (color) {
        color[3 * (size_t)idx] = acc.x, color[3 * (size_t)idx + 1] = acc.y, color[3 * (size_t)idx + 2] = acc.z;
      }
      // AverageSuperSamplingKernel clamp (scene.cu:127-140), then
      // pullRaytracedImage's (unsigned char)(255.0*x) (inc/raytracer.h:53-63).
      double cc[3] = {acc.x, acc.y, acc.z};
      for (int ch = 0; ch < 3; ch++) {
        double v = cc[ch];
        if (v < 0) v = 0.0;
        if (v > 1) v = 1.0;
        if (rgb8) rgb8[3 * (size_t)idx + ch] = (uint8_t)(255.0 * v);
      }
    }
  }
  return overflow;
}

// orc_render with recursive traceRay (trace_rec): up to `depth` levels of
// reflected and refracted rays below each primary ray, whose shading draws
// from the pixel's stream in depth-first order.  optics[4*m] = kr xyz, ior of
// material m; NULL takes kr = ks (Scene_h::LoadObj sets kr to the MTL's
// specular colour, src/scene.cpp:29) and ior = 1 (tinyobjloader's default).
// Outputs as orc_render (hit_id/hit_t: the primary ray's closest hit);
// counts[2] (optional): closest-hit rays traced, shadow rays traced.
int orc_render_rec(void* h, const orc_camera* cam, const orc_light* light, int W, int H, int spp, int depth,
                   const double* optics, uint8_t* rgb8, double* color, int* hit_id, double* hit_t,
                   const double* rays_in, double* rays_out, int nthreads, int64_t* counts, uint32_t seed) {
  const Scene* s = (const Scene*)h;
  std::vector<double> opt(4 * (size_t)s->nmat);
  for (int m = 0; m < s->nmat; m++) {
    for (int c = 0; c < 3; c++) opt[4 * m + c] = optics ? optics[4 * m + c] : s->mats[m].ks[c];
    opt[4 * m + 3] = optics ? optics[4 * m + 3] : 1.0;
  }
  const int gx = (W + 15) / 16;
  int overflow = 0;
  int64_t nrays = 0, nshadow = 0;
  const double invW = 1.0 / double(W), invH = 1.0 / double(H);
  const double aspect = double(W) / double(H);
  const double angle = tan(M_PI * 0.5 * cam->fov / 180.0f);
  const double aperture = 1 / cam->fstop;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for collapse(2) schedule(dynamic, 16) reduction(+ : overflow, nrays, nshadow)
#endif
  for (int py = 0; py < H; py++) {
    for (int px = 0; px < W; px++) {
      const int idx = (H - py - 1) * W + px;
      uint32_t st = wang_hash((uint32_t)(((py / 16) * gx + px / 16) * 256 + (py % 16) * 16 + (px % 16)) ^
                              (seed * 0x9E3779B1u));
      double xx = (2 * ((px + 0.5) * invW) - 1) * angle * aspect;
      double yy = (1 - 2 * ((py + 0.5) * invH)) * angle;
      V3 acc = v3(0, 0, 0);
      for (int k = 0; k < spp; k++) {
        const size_t si = (size_t)idx * spp + k;
        double dofAngle = 2 * M_PI * rand_double(st);
        double dofRadius = aperture * sqrt(rand_double(st)) / 2.0;
        V3 org = v3(dofRadius * cos(dofAngle), dofRadius * sin(dofAngle), 0);
        V3 dir = v3(xx, yy, -1.0);
        dir = normalize(dir) * cam->focal_point - org;
        dir = normalize(dir);
        if (rays_in) {
          const double* r = rays_in + 6 * si;
          org = v3(r[0], r[1], r[2]);
          dir = v3(r[3], r[4], r[5]);
        }
        if (rays_out) {
          double* r = rays_out + 6 * si;
          r[0] = org.x, r[1] = org.y, r[2] = org.z, r[3] = dir.x, r[4] = dir.y, r[5] = dir.z;
        }
        Hit first;
        int res = 0;
        int ov = 0;
        int64_t c[2] = {0, 0};
        acc = acc + trace_rec(*s, cam, light, opt.data(), org, dir, depth, st, &ov, &first, &res, c);
        overflow += ov;
        nrays += c[0], nshadow += c[1];
        if (hit_id) hit_id[si] = res > 0 ? first.id : -1;
        if (hit_t) hit_t[si] = res > 0 ? first.t : 0.0;
      }
      acc = v3(acc.x / double(spp), acc.y / double(spp), acc.z / double(spp));
      if (color) {
        color[3 * (size_t)idx] = acc.x, color[3 * (size_t)idx + 1] = acc.y, color[3 * (size_t)idx + 2] = acc.z;
      }
      double cc[3] = {acc.x, acc.y, acc.z};
      for (int ch = 0; ch < 3; ch++) {
        double v = cc[ch];
        if (v < 0) v = 0.0;
        if (v > 1) v = 1.0;
        if (rgb8) rgb8[3 * (size_t)idx + ch] = (uint8_t)(255.0 * v);
      }
    }
  }
  if (counts) counts[0] = nrays, counts[1] = nshadow;
  return overflow;
}

// Adjoint of the mean colour (and mean hit t) of orc_render with respect to
// the vertices, the light position and each material's kd: the float64
// reference for the GPU adjoint (no counterpart in the reference).  The
// samples are regenerated exactly as in orc_render; which triangle is hit and
// whether the shadow ray is blocked are held fixed, the specular term is
// treated as constant, and the float roundings inside normalize()/norm() are
// taken as exact scalings.  grad_rgb[idx*3], grad_depth[idx] (may be NULL);
// outputs are accumulated into grad_v[V*3], grad_light[3], grad_kd[M*3].
void orc_adjoint(void* h, const orc_camera* cam, const orc_light* light, int W, int H, int spp,
                 const double* grad_rgb, const double* grad_depth, double* grad_v, double* grad_light,
                 double* grad_kd, int nthreads) {
  const Scene* s = (const Scene*)h;
  const int gx = (W + 15) / 16;
  const double invW = 1.0 / double(W), invH = 1.0 / double(H);
  const double aspect = double(W) / double(H);
  const double angle = tan(M_PI * 0.5 * cam->fov / 180.0f);
  const double aperture = 1 / cam->fstop;
  const V3 lpos = v3(light->position[0], light->position[1], light->position[2]);
  const double lcol[3] = {light->color[0], light->color[1], light->color[2]};
  auto add = [](double* p, double v) {
#ifdef _OPENMP
#pragma omp atomic
#endif
    *p += v;
  };
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int py = 0; py < H; py++) {
    for (int px = 0; px < W; px++) {
      const int idx = (H - py - 1) * W + px;
      uint32_t g = (uint32_t)(((py / 16) * gx + px / 16) * 256 + (py % 16) * 16 + (px % 16));
      uint32_t st = wang_hash(g);
      double xx = (2 * ((px + 0.5) * invW) - 1) * angle * aspect;
      double yy = (1 - 2 * ((py + 0.5) * invH)) * angle;
      const double G[3] = {grad_rgb[3 * (size_t)idx] / spp, grad_rgb[3 * (size_t)idx + 1] / spp,
                           grad_rgb[3 * (size_t)idx + 2] / spp};
      const double Gd = grad_depth ? grad_depth[idx] / spp : 0.0;
      for (int k = 0; k < spp; k++) {
        double dofAngle = 2 * M_PI * rand_double(st);
        double dofRadius = aperture * sqrt(rand_double(st)) / 2.0;
        V3 org = v3(dofRadius * cos(dofAngle), dofRadius * sin(dofAngle), 0);
        V3 dir = normalize(v3(xx, yy, -1.0)) * cam->focal_point - org;
        dir = normalize(dir);
        Hit hh;
        if (traverse(*s, org, dir, false, &hh) <= 0) continue;
        V3 q = org + (hh.t * dir);
        const int mid = s->matid[hh.id];
        const Material& m = s->mats[mid];
        V3 nA = s->normals[s->nidx[3 * hh.id]], nB = s->normals[s->nidx[3 * hh.id + 1]],
           nC = s->normals[s->nidx[3 * hh.id + 2]];
        V3 Nr = (1.0 - (hh.alpha + hh.beta)) * nA + hh.alpha * nB + hh.beta * nC;
        double sN = 1.0 / (double)sqrtf((float)(Nr.x * Nr.x + Nr.y * Nr.y + Nr.z * Nr.z));
        V3 N = Nr * sN;
        double r[3];
        light_draws(st, r);
        V3 off = v3(r[0] * light->radius - 0.5, r[1] * light->radius - 0.5, r[2] * light->radius - 0.5);
        V3 Lp = lpos + off - q;
        double sL = 1.0 / (double)sqrtf((float)(Lp.x * Lp.x + Lp.y * Lp.y + Lp.z * Lp.z));
        V3 L = Lp * sL;
        double dist = norm(lpos - q);
        double fall = light->constant_term + (light->linear_term + light->quadratic_term * dist) * dist;
        bool tiny = fabs(fall) < kRayEps;
        fall = tiny ? 1.0 : 1.0 / fall;
        double datt = fmin(1.0, fall);
        double satt[3] = {1, 1, 1};
        Hit sh;
        int omid = -1;
        bool otrans = false;
        if (traverse(*s, q, L, true, &sh) > 0 && sh.t < norm(lpos - q) && !(sh.t < kRayEps)) {
          omid = s->matid[sh.id];
          const Material& om = s->mats[omid];
          otrans = om.kt[0] == 0 && om.kt[1] == 0 && om.kt[2] == 0;
          for (int c = 0; c < 3; c++) satt[c] = otrans ? om.kd[c] * (1 - om.kt[c]) : 0.0;
        }
        double NL = dot(N, L);
        double lam = NL < 0 ? 0 : NL;
        // specular value (constant for the gradient)
        V3 Vv = v3(cam->eye[0], cam->eye[1], cam->eye[2]) - q;
        Vv = normalize(v3(-Vv.x, -Vv.y, -Vv.z));
        V3 R = normalize((-2.0 * dot(L, N)) * N + L);
        double sp = (double)powf((float)fmax(0.0, dot(R, Vv)), (float)m.shininess);
        double S_lam = 0.0, gdatt = 0.0;
        for (int c = 0; c < 3; c++) {
          double w = G[c] * lcol[c];
          double dsv = m.kd[c] * lam + m.ks[c] * sp;
          add(grad_kd + 3 * mid + c, w * datt * satt[c] * lam);
          if (omid >= 0 && otrans) add(grad_kd + 3 * omid + c, w * datt * dsv * (1 - s->mats[omid].kt[c]));
          S_lam += w * datt * satt[c] * m.kd[c];
          gdatt += w * satt[c] * dsv;
        }
        if (!(NL > 0)) S_lam = 0.0;
        double gdist = 0.0;
        if (!tiny && fall < 1.0) {
          double fr = 1.0 / fall;
          gdist = gdatt * (-(light->linear_term + 2.0 * light->quadratic_term * dist) / (fr * fr));
        }
        V3 gLp = v3((N.x - NL * L.x) * sL * S_lam, (N.y - NL * L.y) * sL * S_lam, (N.z - NL * L.z) * sL * S_lam);
        V3 u = dist > 0 ? (1.0 / dist) * (lpos - q) : v3(0, 0, 0);
        V3 gP = gLp + gdist * u;
        for (int c = 0; c < 3; c++) add(grad_light + c, comp(gP, c));
        V3 gq = v3(-gP.x, -gP.y, -gP.z);
        V3 gN = v3((L.x - NL * N.x) * sN * S_lam, (L.y - NL * N.y) * sN * S_lam, (L.z - NL * N.z) * sN * S_lam);
        double g_al = dot(gN, nB - nA), g_be = dot(gN, nC - nA);
        double g_t = dot(gq, dir) + Gd;
        const int ia = s->vidx[3 * hh.id], ib = s->vidx[3 * hh.id + 1], ic = s->vidx[3 * hh.id + 2];
        V3 A = s->verts[ia], Bv = s->verts[ib], Cv = s->verts[ic];
        V3 ma = v3(-dir.x, -dir.y, -dir.z), mb = Bv - A, mc = Cv - A;
        V3 bc = cross(mb, mc), ca = cross(mc, ma), ab = cross(ma, mb);
        double det = dot(ma, bc);
        if (det == 0.0) continue;
        double id = -1.0 / det;
        V3 w = v3(id * (g_t * bc.x + g_al * ca.x + g_be * ab.x), id * (g_t * bc.y + g_al * ca.y + g_be * ab.y),
                  id * (g_t * bc.z + g_al * ca.z + g_be * ab.z));
        double wa = 1.0 - (hh.alpha + hh.beta), wb = hh.alpha, wc = hh.beta;
        for (int c = 0; c < 3; c++) {
          add(grad_v + 3 * ia + c, wa * comp(w, c));
          add(grad_v + 3 * ib + c, wb * comp(w, c));
          add(grad_v + 3 * ic + c, wc * comp(w, c));
        }
      }
    }
  }
}

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"

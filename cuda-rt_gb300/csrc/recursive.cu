// recursive.cu -- traceRay with reflected and refracted rays on sm_103a.
//
// The reference's traceRay (kernels/raytracer.cu:169-249) takes a depth and
// carries a Whitted-style reflection/refraction block (raytracer.cu:196-237)
// that is commented out, so its renders stop at shade().  k_pixels_rec runs
// that block: below every primary ray, while depth > 0, a reflective
// material (kr != 0) adds kr % traceRay(reflected ray, depth - 1), then a
// transmissive one (kt != 0) adds kt % traceRay(refracted ray, depth - 1)
// unless the refracted ray is totally internally reflected.  As written the
// block tests Refl()/Trans(), which setBools() defines as isZero(kr) and
// isZero(kt) (inc/material.h:27-31): it would trace the rays of materials
// that cannot reflect and add zero.  The kernel follows the evident intent
// (trace when the coefficient is non-zero).  Secondary rays start at
// q = r.at(t) with no offset and use the closest-hit search of the primary
// rays (negative t accepted, |t| < RAY_EPSILON rejected).
//
// Every shade() draws three numbers from the pixel's mrand stream, so the
// stream position of a ray depends on every hit before it in depth-first
// order, across the pixel's samples too.  Each lane walks one sample's ray
// tree depth first with an explicit frame stack (at most depth + 1 frames,
// in local memory), starting its stream where the earlier samples' walks are
// guessed to end and walking again when a guess proves wrong (k_pixels_rec);
// the sums are formed in the recursion's order (shade, + kr % reflected,
// + kt % refracted), so the colours equal a recursive evaluation bit for
// bit.  The traversals are warp-synchronous: each step of the loop traces
// the next ray of every lane that has one, then the shadow rays of the lanes
// whose ray hit.
#include "crt_internal.h"

namespace crt {

namespace {

// The most lanes a pixel's samples take when there are secondary rays (fewer
// when spp is smaller): on the depth-3 mirror/glass frame (1280x720, 4 spp)
// 2 lanes took 16.0 ms, 4 lanes 18.3 ms (more walks start from wrong guesses)
// and 1 lane 19.0 ms.  Without secondary rays (depth 0) one lane per pixel
// is fastest (3.3 against 3.5 ms): there is no tree to overlap.
constexpr int kRecLanesPerPixel = 2;

struct Frame {
  D3 c;        // colour so far: shade(), then each child's contribution
  D3 q, N, d;  // hit point, smooth normal, incoming direction
  int mid;     // material
  int stage;   // 0 no child yet, 1 reflected child out, 2 refracted child out, 3 done
};

__device__ __forceinline__ bool nonzero3(const double* k) { return !(k[0] == 0 && k[1] == 0 && k[2] == 0); }

// kr and ior of material m: the caller's table, or (optics NULL) kr = ks, as
// Scene_h::LoadObj sets it (src/scene.cpp:29), and tinyobjloader's ior of 1.
__device__ __forceinline__ const double* kr_of(const DOptics* optics, const DMat* mats, int m) {
  return optics ? optics[m].kr : mats[m].ks;
}
__device__ __forceinline__ double ior_of(const DOptics* optics, int m) { return optics ? optics[m].ior : 1.0; }

// The next child ray of frame f (the commented block's order: reflection,
// then refraction), or false when f has no more children.
__device__ bool next_child(Frame& f, const DOptics* __restrict__ optics, const DMat* __restrict__ mats, D3& org,
                           D3& dir) {
  if (f.stage == 0) {
    f.stage = 1;
    if (nonzero3(kr_of(optics, mats, f.mid))) {
      // Rdir = -2.0*(r.getDirection()*i.N)*i.N + r.getDirection(); normalize
      dir = normalize_exact((-2.0 * dot(f.d, f.N)) * f.N + f.d);
      org = f.q;
      return true;
    }
  }
  if (f.stage == 1) {
    f.stage = 3;
    if (nonzero3(mats[f.mid].kt)) {
      D3 n = f.N;
      const D3 rd = f.d;
      const D3 rcos = dot(d3(-rd.x, -rd.y, -rd.z), n) * n;  // n*(-rd*n)
      const D3 rsin = rcos + rd;
      const double etai = 1.0, etat = ior_of(optics, f.mid);
      double eta;
      if (dot(rd, n) < 0) {
        eta = etai / etat;
        n = d3(-n.x, -n.y, -n.z);
      } else {
        eta = etat / etai;
      }
      const D3 tsin = eta * rsin;
      const double TIR = 1 - dot(tsin, tsin);
      if (TIR >= 0) {
        const D3 tcos = sqrt(TIR) * n;
        dir = normalize_exact(tcos + tsin);
        org = f.q;
        f.stage = 2;
        return true;
      }
    }
  }
  f.stage = 3;
  return false;
}

// A child's colour v returns to its parent frame f.
__device__ __forceinline__ void add_child(Frame& f, const DOptics* __restrict__ optics,
                                          const DMat* __restrict__ mats, D3 v) {
  const double* k = f.stage == 1 ? kr_of(optics, mats, f.mid) : mats[f.mid].kt;
  f.c = f.c + d3(k[0] * v.x, k[1] * v.y, k[2] * v.z);
}

struct PixelRay {
  D3 org, dir;
};

// Primary ray of the next sample: two draws (lens angle and radius), the
// thin-lens ray of runRayTracerKernelRec (raytracer.cu:141-152).
__device__ __forceinline__ PixelRay primary(const RenderArgs& A, D3 fdir, uint32_t& st) {
  double ox, oy;
  lens_origin(A.lens_cs, A.lens_sqrt, A.aperture, st, ox, oy);
  const D3 org = d3(ox, oy, 0.0);
  return PixelRay{org, normalize_exact(fdir - org)};
}

// One lane per sample, G lanes per pixel (a warp covers 32 / G pixels of a
// compact tile, as in the plain pixel kernel).  A sample's place in its
// pixel's mrand stream is 2 draws per earlier sample plus 3 per hit of the
// earlier samples' ray trees, so each lane guesses the hit counts of the
// earlier samples of its wave (the counts the same lanes saw in the last
// wave; one hit each at first), starts its stream there and walks its
// sample's ray tree.  A lane whose earlier lanes all saw the counts they were
// guessed to see had the right start (induction from the group's first lane,
// whose start is always right), so its tree is the sequential one; the
// others walk again with the counts just seen, and each round settles at
// least one more lane per group.  The colours are summed in sample order.
// The tree of a sample is walked depth first with an explicit frame stack,
// as the recursion of traceRay; every step traces the next ray of every lane
// that has one, then the shadow rays of the lanes whose ray hit.
__global__ void __launch_bounds__(128) k_pixels_rec(DScene S, RenderArgs A, const DOptics* __restrict__ optics,
                                                    int depth) {
  const unsigned full = 0xffffffffu;
  float rb[6], B, D;
  scene_consts(S, rb, B, D);
  const int lane = threadIdx.x & 31;
  const int G = A.group, tw = group_tile_w(G), th = group_tile_h(G);
  const int g = lane & (G - 1);
  const int base = lane - g;
  const unsigned gmask = (G == 32) ? full : (((1u << G) - 1u) << base);
  const unsigned below = gmask & ((1u << lane) - 1u);  // the lanes of my group before me
  const int tiles_x = (A.W + tw - 1) / tw, tiles_y = (A.row1 - A.row0 + th - 1) / th;
  const int gx = (A.W + 15) / 16;
  const D3 lpos = d3(A.lpos[0], A.lpos[1], A.lpos[2]);
  Frame fr[kMaxRecDepth];
  unsigned long long nrays = 0, nshadow = 0;  // for A.stats (accepted walks only)
  int hguess = 1;  // the hit count this lane saw in its last walk
  int region = home_region(A.regions_x, A.regions_y);
  bool home = true;
  while (true) {
    int tile = 0;
    if (lane == 0) tile = claim_tile(A.counter, tiles_x, tiles_y, A.regions_x, A.regions_y, region, home);
    tile = __shfl_sync(full, tile, 0);
    if (tile < 0) break;
    const int pp = lane / G;  // this lane's pixel in the tile
    const int px = (tile % tiles_x) * tw + (pp % tw);
    const int py = A.row0 + (tile / tiles_x) * th + (pp / tw);
    const bool valid = px < A.W && py < A.row1;
    const int idx = (A.H - py - 1) * A.W + px;
    uint32_t wst =
        wang_hash((uint32_t)(((py / 16) * gx + px / 16) * 256 + (py % 16) * 16 + (px % 16)) ^ A.seed_mix);
    const double xx = (2 * ((px + 0.5) * A.invW) - 1) * A.angle * A.aspect;
    const double yy = (1 - 2 * ((py + 0.5) * A.invH)) * A.angle;
    D3 fdir = normalize_exact(d3(xx, yy, -1.0));
    fdir = d3(fdir.x * A.focal, fdir.y * A.focal, fdir.z * A.focal);
    D3 acc = d3(0, 0, 0);
    const int waves = valid ? (A.spp + G - 1) / G : 0;
    const int wmax = __reduce_max_sync(full, waves);
    for (int w = 0; w < wmax; w++) {
      const int k = w * G + g;
      const bool act = w < waves && k < A.spp;
      bool settled = !act;
      int H = hguess;  // the count the later lanes of my group assume for my walk
      // the walk's results
      D3 v = d3(0, 0, 0);
      int hits = 0, prim_id = -1;
      double prim_t = 0.0;
      PixelRay prim{d3(0, 0, 0), d3(0, 0, 1)};
      uint32_t st_end = wst;
      unsigned long long wr = 0, ws = 0;
      while (true) {
        // where my walk starts in the stream: the group's earlier lanes' draws
        int off = act ? 2 + 3 * H : 0, run = off;
        for (int o = 1; o < G; o <<= 1) {
          const int y = __shfl_up_sync(full, run, o);
          if (g >= o) run += y;
        }
        off = run - off;
        bool busy = !settled;
        uint32_t st = wst;
        int lvl = 0;
        PixelRay ray{d3(0, 0, 0), d3(0, 0, 1)};
        if (busy) {
          for (int t = 0; t < off; t++) xorshift32(st);
          ray = primary(A, fdir, st);
          prim = ray;
          hits = 0, wr = 0, ws = 0, prim_id = -1, prim_t = 0.0;
        }
        while (__any_sync(full, busy)) {
          RayC rc;
          if (busy)
            ray_setup(rc, ray.org.x, ray.org.y, ray.org.z, ray.dir.x, ray.dir.y, ray.dir.z, B, D);
          else
            ray_setup(rc, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, B, D);
          HitRec h;
          const int res = traverse<false>(S, rc, rb, h, busy);
          if (res < 0) atomicOr(&S.g->err, kErrStack);
          const bool hit = busy && res > 0;
          wr += busy, ws += hit, hits += hit;
          if (busy && lvl == 0) prim_id = hit ? h.id : -1, prim_t = hit ? h.t : 0.0;
          // Light::getDirection (three draws) and the shadow ray of each hit
          D3 q = d3(0, 0, 0), L = d3(0, 0, 1);
          double dist = 0.0;
          RayC sr;
          if (hit) {
            q = ray.org + (h.t * ray.dir);
            const double r0 = rand_double(st), r1 = rand_double(st), r2 = rand_double(st);
            const D3 off3 = d3(r0 * A.lradius - 0.5, r1 * A.lradius - 0.5, r2 * A.lradius - 0.5);
            L = normalize_exact(lpos + off3 - q);
            dist = norm_exact(lpos - q);
            ray_setup(sr, q.x, q.y, q.z, L.x, L.y, L.z, B, D);
          } else {
            ray_setup(sr, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, B, D);
          }
          HitRec sh;
          const int sres = traverse<true>(S, sr, rb, sh, hit);
          if (sres < 0) atomicOr(&S.g->err, kErrStack);
          if (!busy) continue;
          // Material::shade (kernels/material.cu:6-40), as the plain pixel kernel
          D3 c = d3(0.9, 0.9, 0.9);
          D3 N = d3(0, 0, 0);
          int mid = 0;
          if (hit) {
            N = hit_normal(S, h);
            mid = __ldg(S.matid + h.id);
            const DMat& m = S.mats[mid];
            D3 I = d3(m.ke[0] + m.ka[0] * 0.0, m.ke[1] + m.ka[1] * 0.0, m.ke[2] + m.ka[2] * 0.0);
            double fall = A.latt[0] + (A.latt[1] + A.latt[2] * dist) * dist;
            fall = fabs(fall) < kRayEps ? 1.0 : 1.0 / fall;
            const double datt = fmin(1.0, fall);
            D3 satt = d3(1, 1, 1);
            if (sres > 0 && sh.t < dist && !(sh.t < kRayEps)) {
              const DMat& om = S.mats[__ldg(S.matid + sh.id)];
              const bool otrans = om.kt[0] == 0 && om.kt[1] == 0 && om.kt[2] == 0;  // Trans() = isZero(kt)
              satt = otrans ? d3(om.kd[0] * (1 - om.kt[0]), om.kd[1] * (1 - om.kt[1]), om.kd[2] * (1 - om.kt[2]))
                            : d3(0, 0, 0);
            }
            const D3 att = datt * satt;
            double lam = dot(N, L);
            if (lam < 0) lam = 0;
            const D3 diffuse = d3(m.kd[0] * lam, m.kd[1] * lam, m.kd[2] * lam);
            D3 ds = diffuse;
            if (!phong_vanishes(m, I))
              ds = diffuse + phong_term(S.mats + mid, L, N, q, d3(A.eye[0], A.eye[1], A.eye[2]));
            c = I + d3(att.x * ds.x * A.lcol[0], att.y * ds.y * A.lcol[1], att.z * ds.z * A.lcol[2]);
          }
          // depth-first walk: descend into this ray's first child, or return its
          // colour up the frames until one has another child or the tree ends
          if (hit && lvl < depth) {
            Frame& f = fr[lvl];
            f.c = c, f.q = q, f.N = N, f.d = ray.dir, f.mid = mid, f.stage = 0;
            if (next_child(f, optics, S.mats, ray.org, ray.dir)) {
              lvl++;
              continue;
            }
            c = f.c;
          }
          while (true) {
            if (lvl == 0) {
              v = c;
              busy = false;
              st_end = st;
              break;
            }
            Frame& f = fr[lvl - 1];
            add_child(f, optics, S.mats, c);
            if (next_child(f, optics, S.mats, ray.org, ray.dir)) break;
            c = f.c;
            lvl--;
          }
        }
        // a walk is the sequential one when every earlier lane of its group saw
        // the count it was guessed to see
        const unsigned wrong = __ballot_sync(full, act && H != hits) & below;
        if (!settled && wrong == 0u) {
          settled = true;
          nrays += wr, nshadow += ws;
          const int64_t si = (int64_t)idx * A.spp + k;
          if (A.hit_id) A.hit_id[si] = prim_id;
          if (A.hit_t) A.hit_t[si] = prim_t;
          if (A.rays) {
            double* r = A.rays + 6 * si;
            r[0] = prim.org.x, r[1] = prim.org.y, r[2] = prim.org.z;
            r[3] = prim.dir.x, r[4] = prim.dir.y, r[5] = prim.dir.z;
          }
        }
        if (__all_sync(full, settled)) break;
        if (act) H = hits;
      }
      if (act) hguess = hits;
      // sum in sample order (the reference adds the samples one by one)
      for (int t = 0; t < G; t++) {
        const double cx = __shfl_sync(full, v.x, base + t), cy = __shfl_sync(full, v.y, base + t),
                     cz = __shfl_sync(full, v.z, base + t);
        if (w < waves && w * G + t < A.spp) acc = acc + d3(cx, cy, cz);
      }
      // the next wave starts where the group's last sample ended
      wst = __shfl_sync(full, st_end, base + G - 1);
    }
    if (!valid || A.spp <= 0 || g != 0) continue;
    const double inv = (double)A.spp;
    acc = d3(acc.x / inv, acc.y / inv, acc.z / inv);
    if (A.rgbf) {
      A.rgbf[3 * (int64_t)idx] = (float)acc.x;
      A.rgbf[3 * (int64_t)idx + 1] = (float)acc.y;
      A.rgbf[3 * (int64_t)idx + 2] = (float)acc.z;
    }
    if (A.rgbd) {
      A.rgbd[3 * (int64_t)idx] = acc.x;
      A.rgbd[3 * (int64_t)idx + 1] = acc.y;
      A.rgbd[3 * (int64_t)idx + 2] = acc.z;
    }
    if (A.rgb8) {
      const double cc[3] = {acc.x, acc.y, acc.z};
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        double c = cc[ch];
        if (c < 0) c = 0.0;
        if (c > 1) c = 1.0;
        A.rgb8[3 * (int64_t)idx + ch] = (uint8_t)(255.0 * c);
      }
    }
  }
  if (A.stats) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      nrays += __shfl_xor_sync(full, nrays, o);
      nshadow += __shfl_xor_sync(full, nshadow, o);
    }
    if (lane == 0) {
      atomicAdd(A.stats, nrays);
      atomicAdd(A.stats + 1, nshadow);
    }
  }
}

}  // namespace

cudaError_t launch_render_recursive(const DScene& S, const RenderArgs& a, const DOptics* optics, int depth,
                                    cudaStream_t st) {
  if (depth < 0 || depth > kMaxRecDepth) return cudaErrorInvalidValue;
  RenderArgs r = a;
  r.group = depth > 0 ? lanes_per_pixel(a.spp, kRecLanesPerPixel) : 1;
  const int tw = group_tile_w(r.group), th = group_tile_h(r.group);
  // (one rectangle: the cost of a pixel's ray trees varies too much for rectangles of equal size)
  cudaError_t e = set_tile_regions(r, (r.W + tw - 1) / tw, (r.row1 - r.row0 + th - 1) / th, false, st);
  if (e != cudaSuccess) return e;
  int bps = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_pixels_rec, 128, 0);
  k_pixels_rec<<<num_sms() * (bps > 0 ? bps : 1), 128, 0, st>>>(S, r, optics, depth);
  return cudaGetLastError();
}

}  // namespace crt

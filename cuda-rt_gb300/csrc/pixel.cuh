// pixel.cuh -- the pixel function shared by the single-scene pixel kernel
// (trace.cu) and the batched form's render (batch_kernel.cuh).
#pragma once
#include "crt_internal.h"

namespace crt {

namespace {

enum PixelMode { kRender = 0, kRenderStats = 1, kAdjoint = 2 };

// Warp-reduced atomic add of a double (light gradient: few addresses).
__device__ __forceinline__ void warp_add(double* dst, double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(dst, v);
}

// runRayTracerKernelRec (kernels/raytracer.cu:95-166) per pixel, with
// traceRay (raytracer.cu:169-249), Material::shade (kernels/material.cu:6-40)
// and the positional Light (kernels/Light.cu:5-86).  MODE kAdjoint re-runs the
// same samples (same rays, hits and shadow tests: nothing is stored between
// the forward and the adjoint) and accumulates d loss / d (vertices, light
// position, albedo) for the Lambert and distance terms; visibility (which
// triangle is hit, whether the shadow ray is blocked) is held fixed.
//
// All 32 lanes of the warp call it together.  G lanes (a power of two) share
// one pixel and trace G of its samples at once, in waves of G samples; valid
// false marks a pixel outside the image (its lanes compute and write
// nothing).  The samples of a pixel share one mrand stream: sample k draws
// two numbers for the lens and, when its primary ray hits, three for the
// light, so where sample k starts in the stream depends on which earlier
// samples hit.  Each lane guesses those hits (`pred`: the last wave's
// majority), traces, and the lanes whose guess of an earlier sample proved
// wrong trace again with the hits just observed; at least one more sample of
// every group is settled per round, and the settled rays are exactly the
// sequential ones.  Colours and depths are then summed in sample order.
template <int MODE, int SHORT = 0, bool NC = true>
__device__ __forceinline__ void pixel(const DScene& S, const RenderArgs& A, int px, int py, bool valid, int G,
                                      unsigned& pred, float rb[6], float B, float D, TravStats& ts, D3& glight,
                                      int2* ring = nullptr) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int g = lane & (G - 1);
    const int base = lane - g;
    const unsigned gmask = (G == 32) ? full : (((1u << G) - 1u) << base);
    const unsigned below = gmask & ((1u << lane) - 1u);  // the lanes of my group before me
    const int gx = (A.W + 15) / 16;  // gridDim.x of the reference's 16x16 launch
    const D3 lpos = d3(A.lpos[0], A.lpos[1], A.lpos[2]);
    const int idx = (A.H - py - 1) * A.W + px;
    // getGlobalIdx_2D_2D (inc/indexing.h:4-9) of the pixel's thread in the
    // reference launch, seeded by initPNRG (kernels/mrand.cu:38-41).
    const uint32_t gid = (uint32_t)(((py / 16) * gx + px / 16) * 256 + (py % 16) * 16 + (px % 16));
    uint32_t wst = wang_hash(gid ^ A.seed_mix);  // stream position at the start of the wave
    const double xx = (2 * ((px + 0.5) * A.invW) - 1) * A.angle * A.aspect;
    const double yy = (1 - 2 * ((py + 0.5) * A.invH)) * A.angle;
    // the pinhole direction scaled to the focal plane: the same for every sample
    D3 fdir = normalize_exact(d3(xx, yy, -1.0));
    fdir = d3(fdir.x * A.focal, fdir.y * A.focal, fdir.z * A.focal);
    D3 acc = d3(0, 0, 0);
    double depth = 0.0;
    D3 G3 = d3(0, 0, 0);
    double Gd = 0.0;
    if (MODE == kAdjoint && valid) {
      const double inv = 1.0 / (double)A.spp;
      G3 = d3(A.grad_rgb[3 * (int64_t)idx] * inv, A.grad_rgb[3 * (int64_t)idx + 1] * inv,
              A.grad_rgb[3 * (int64_t)idx + 2] * inv);
      Gd = A.grad_depth ? A.grad_depth[idx] * inv : 0.0;
    }
    const int waves = (A.spp + G - 1) / G;
    for (int w = 0; w < waves; w++) {
      const int k = w * G + g;
      const bool act = valid && k < A.spp;
      const unsigned actm = __ballot_sync(full, act);
      const int64_t si = (int64_t)idx * A.spp + k;
      // primary rays, speculating on the hits of the group's earlier samples
      unsigned guess = pred;
      bool done = !act;
      HitRec h;
      int res = 0;
      D3 org = d3(0, 0, 0), dir = d3(0, 0, 1);
      uint32_t st = wst;
      unsigned hits;
      while (true) {
        RayC rc;
        if (!done) {
          st = wst;
          for (int t = 0; t < g; t++) {
            xorshift32(st);
            xorshift32(st);
            if ((guess >> (base + t)) & 1u) {
              xorshift32(st);
              xorshift32(st);
              xorshift32(st);
            }
          }
          // sincos gives sin and cos bit for bit (checked for every angle 2*pi*u
          // the float-valued mrand draw u can take)
          double ox, oy;
          lens_origin(A.lens_cs, A.lens_sqrt, A.aperture, st, ox, oy);
          org = d3(ox, oy, 0.0);
          dir = normalize_exact(fdir - org);
          ray_setup(rc, org.x, org.y, org.z, dir.x, dir.y, dir.z, B, D);
        } else {
          ray_setup(rc, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, B, D);
        }
        HitRec ht;
        const int r = traverse<false, MODE == kRenderStats, SHORT, NC>(S, rc, rb, ht, !done, &ts, ring);
        if (!done) h = ht, res = r;
        hits = __ballot_sync(full, act && res > 0);
        // a lane is settled when every earlier sample of its group was guessed right
        if (((guess ^ hits) & actm & below) == 0u) done = true;
        guess = hits;
        if (__all_sync(full, done)) break;
      }
      if (res < 0) atomicOr(&S.g->err, kErrStack);
      const bool hit = act && res > 0;
      if (MODE != kAdjoint && A.rays && act) {
        double* rr = A.rays + 6 * si;
        rr[0] = org.x, rr[1] = org.y, rr[2] = org.z, rr[3] = dir.x, rr[4] = dir.y, rr[5] = dir.z;
      }
      // traceRay up to the shadow ray (lanes with a hit): only what the
      // shadow ray needs is computed before it, to keep little state live
      // across the walk; the rest of the shading follows it
      D3 q, L;
      double sL = 0.0, dist = 0.0;
      RayC sr;
      if (hit) {
        q = org + (h.t * dir);
        // Light::getDirection: three draws (x, y, z), times radius, minus 0.5
        const double r0 = rand_double(st), r1 = rand_double(st), r2 = rand_double(st);
        const D3 off = d3(r0 * A.lradius - 0.5, r1 * A.lradius - 0.5, r2 * A.lradius - 0.5);
        const D3 Lp = lpos + off - q;
        sL = 1.0 / (double)sqrtf(__double2float_rn(Lp.x * Lp.x + Lp.y * Lp.y + Lp.z * Lp.z));
        L = d3(Lp.x * sL, Lp.y * sL, Lp.z * sL);
        dist = norm_exact(lpos - q);
        ray_setup(sr, q.x, q.y, q.z, L.x, L.y, L.z, B, D);
      } else {
        ray_setup(sr, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, B, D);
      }
      // the next wave starts where the group's last sample ended
      wst = __shfl_sync(full, st, base + G - 1);
      // Light::shadowAttenuation: any-hit from q towards the light
      HitRec s;
      const int sres = traverse<true, MODE == kRenderStats, SHORT, NC>(S, sr, rb, s, hit, &ts, ring);
      if (sres < 0) atomicOr(&S.g->err, kErrStack);
      D3 N;
      double sN = 0.0, fall = 0.0, datt = 0.0;
      bool tiny = false;
      if (hit) {
        // smooth normal, bvh.cu:357-364 (hit_normal, kept apart for the adjoint)
        const int na = S.nidx[3 * h.id], nb = S.nidx[3 * h.id + 1], nc = S.nidx[3 * h.id + 2];
        const D3 nA = d3(S.normals[3 * na], S.normals[3 * na + 1], S.normals[3 * na + 2]);
        const D3 nB = d3(S.normals[3 * nb], S.normals[3 * nb + 1], S.normals[3 * nb + 2]);
        const D3 nC = d3(S.normals[3 * nc], S.normals[3 * nc + 1], S.normals[3 * nc + 2]);
        const D3 Nr = (1.0 - (h.alpha + h.beta)) * nA + h.alpha * nB + h.beta * nC;
        sN = 1.0 / (double)sqrtf(__double2float_rn(Nr.x * Nr.x + Nr.y * Nr.y + Nr.z * Nr.z));
        N = d3(Nr.x * sN, Nr.y * sN, Nr.z * sN);
        // Light::distanceAttenuation
        fall = A.latt[0] + (A.latt[1] + A.latt[2] * dist) * dist;
        tiny = fabs(fall) < kRayEps;
        fall = tiny ? 1.0 : 1.0 / fall;
        datt = fmin(1.0, fall);
      }
      D3 col = d3(0.9, 0.9, 0.9);
      int sh = -1, shid = -1;
      if (hit) {
        const int mid = __ldg(S.matid + h.id);
        const DMat m = S.mats[mid];
        D3 I = d3(m.ke[0] + m.ka[0] * 0.0, m.ke[1] + m.ka[1] * 0.0, m.ke[2] + m.ka[2] * 0.0);
        D3 satt = d3(1, 1, 1);
        sh = 0;
        int omid = -1;
        bool otrans = false;
        DMat om;
        if (sres > 0 && s.t < dist && !(s.t < kRayEps)) {  // dist = norm(lpos - q), Light.cu:14-16
          sh = 1;
          shid = s.id;
          omid = __ldg(S.matid + s.id);
          om = S.mats[omid];
          otrans = om.kt[0] == 0 && om.kt[1] == 0 && om.kt[2] == 0;  // Trans() = isZero(kt)
          satt = otrans ? d3(om.kd[0] * (1 - om.kt[0]), om.kd[1] * (1 - om.kt[1]), om.kd[2] * (1 - om.kt[2]))
                        : d3(0, 0, 0);
        }
        const D3 att = datt * satt;
        const double NL = dot(N, L);
        double lam = NL;
        if (lam < 0) lam = 0;
        const D3 diffuse = d3(m.kd[0] * lam, m.kd[1] * lam, m.kd[2] * lam);
        D3 ds = diffuse;
        if (!phong_vanishes(m, I)) ds = diffuse + phong_term(S.mats + mid, L, N, q, d3(A.eye[0], A.eye[1], A.eye[2]));
        I = I + d3(att.x * ds.x * A.lcol[0], att.y * ds.y * A.lcol[1], att.z * ds.z * A.lcol[2]);
        col = I;
        if (MODE == kAdjoint) {
          const double Gc[3] = {G3.x, G3.y, G3.z};
          const double sa[3] = {satt.x, satt.y, satt.z};
          const double dsv[3] = {ds.x, ds.y, ds.z};
          double S_lam = 0.0, gdatt = 0.0;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const double w = Gc[c] * A.lcol[c];
            // d/d kd of the hit triangle's material (Lambert term)
            const double gkd = w * datt * sa[c] * lam;
            if (gkd != 0.0) atomicAdd(A.grad_albedo + 3 * mid + c, gkd);
            // d/d kd of an opaque occluder's material: the reference's shadow
            // attenuation is kd % (1 - kt) of the occluder (Light.cu:22-24)
            if (sh == 1 && otrans) {
              const double go = w * datt * dsv[c] * (1 - om.kt[c]);
              if (go != 0.0) atomicAdd(A.grad_albedo + 3 * omid + c, go);
            }
            S_lam += w * datt * sa[c] * m.kd[c];
            gdatt += w * sa[c] * dsv[c];
          }
          if (!(NL > 0)) S_lam = 0.0;  // lam = max(N.L, 0)
          // datt = min(1, 1/fall(dist)), fall = a + (b + c dist) dist
          double gdist = 0.0;
          if (!tiny && fall < 1.0) {
            const double fr = 1.0 / fall;  // the falloff polynomial itself
            gdist = gdatt * (-(A.latt[1] + 2.0 * A.latt[2] * dist) / (fr * fr));
          }
          // lam through L = Lp / |Lp|, Lp = P + off - q
          const D3 gLp = d3((N.x - NL * L.x) * sL * S_lam, (N.y - NL * L.y) * sL * S_lam,
                            (N.z - NL * L.z) * sL * S_lam);
          const D3 u = (dist > 0.0) ? (1.0 / dist) * (lpos - q) : d3(0, 0, 0);
          const D3 gP = gLp + gdist * u;
          glight = glight + gP;
          const D3 gq = d3(-gP.x, -gP.y, -gP.z);
          // lam through N = Nr / |Nr|, Nr = (1-a-b) nA + a nB + b nC
          const int na = S.nidx[3 * h.id], nb = S.nidx[3 * h.id + 1], nc = S.nidx[3 * h.id + 2];
          const D3 nA = d3(S.normals[3 * na], S.normals[3 * na + 1], S.normals[3 * na + 2]);
          const D3 nB = d3(S.normals[3 * nb], S.normals[3 * nb + 1], S.normals[3 * nb + 2]);
          const D3 nC = d3(S.normals[3 * nc], S.normals[3 * nc + 1], S.normals[3 * nc + 2]);
          const D3 gN = d3((L.x - NL * N.x) * sN * S_lam, (L.y - NL * N.y) * sN * S_lam,
                           (L.z - NL * N.z) * sN * S_lam);
          const double g_al = dot(gN, nB - nA), g_be = dot(gN, nC - nA);
          const double g_t = dot(gq, dir) + Gd;  // q = o + t d, and the depth output
          // (t, alpha, beta) solve [-d | E1 | E2] x = o - A; moving the hit's
          // barycentric point by delta moves x by -M^-1 delta, so
          // d loss / d delta = -M^-T g, split over A, B, C by (1-a-b, a, b).
          const int ia = S.vidx[3 * h.id], ib = S.vidx[3 * h.id + 1], ic = S.vidx[3 * h.id + 2];
          const D3 Av = d3(S.verts[3 * ia], S.verts[3 * ia + 1], S.verts[3 * ia + 2]);
          const D3 Bv = d3(S.verts[3 * ib], S.verts[3 * ib + 1], S.verts[3 * ib + 2]);
          const D3 Cv = d3(S.verts[3 * ic], S.verts[3 * ic + 1], S.verts[3 * ic + 2]);
          const D3 ma = d3(-dir.x, -dir.y, -dir.z), mb = Bv - Av, mc = Cv - Av;
          const D3 bc = d3(mb.y * mc.z - mb.z * mc.y, mb.z * mc.x - mb.x * mc.z, mb.x * mc.y - mb.y * mc.x);
          const D3 ca = d3(mc.y * ma.z - mc.z * ma.y, mc.z * ma.x - mc.x * ma.z, mc.x * ma.y - mc.y * ma.x);
          const D3 ab = d3(ma.y * mb.z - ma.z * mb.y, ma.z * mb.x - ma.x * mb.z, ma.x * mb.y - ma.y * mb.x);
          const double det = dot(ma, bc);
          if (det != 0.0) {
            const double id = -1.0 / det;
            const D3 w = d3(id * (g_t * bc.x + g_al * ca.x + g_be * ab.x), id * (g_t * bc.y + g_al * ca.y + g_be * ab.y),
                            id * (g_t * bc.z + g_al * ca.z + g_be * ab.z));
            const double wa = 1.0 - (h.alpha + h.beta), wb = h.alpha, wc = h.beta;
            atomicAdd(A.grad_verts + 3 * ia, wa * w.x), atomicAdd(A.grad_verts + 3 * ia + 1, wa * w.y);
            atomicAdd(A.grad_verts + 3 * ia + 2, wa * w.z);
            atomicAdd(A.grad_verts + 3 * ib, wb * w.x), atomicAdd(A.grad_verts + 3 * ib + 1, wb * w.y);
            atomicAdd(A.grad_verts + 3 * ib + 2, wb * w.z);
            atomicAdd(A.grad_verts + 3 * ic, wc * w.x), atomicAdd(A.grad_verts + 3 * ic + 1, wc * w.y);
            atomicAdd(A.grad_verts + 3 * ic + 2, wc * w.z);
          }
        }
      }
      if (MODE != kAdjoint && act) {
        if (A.hit_id) A.hit_id[si] = hit ? h.id : -1;
        if (A.hit_t) A.hit_t[si] = hit ? h.t : 0.0;
        if (A.shadow) A.shadow[si] = sh;
        if (A.shadow_id) A.shadow_id[si] = shid;
      }
      // sum in sample order (the reference adds the samples one by one)
      for (int t = 0; t < G; t++) {
        const double cx = __shfl_sync(full, col.x, base + t), cy = __shfl_sync(full, col.y, base + t),
                     cz = __shfl_sync(full, col.z, base + t);
        const double dt = __shfl_sync(full, hit ? h.t : 0.0, base + t);
        if (w * G + t < A.spp) {
          acc = acc + d3(cx, cy, cz);
          if ((hits >> (base + t)) & 1u) depth += dt;
        }
      }
      // guess for the next wave: the group's majority
      const int nh = __popc(hits & gmask), na = __popc(actm & gmask);
      pred = __ballot_sync(full, 2 * nh >= na);
    }
    if (MODE == kAdjoint || !valid || g != 0) return;
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
    if (A.depth) A.depth[idx] = depth / inv;
    if (A.rgb8) {
      const double cc[3] = {acc.x, acc.y, acc.z};
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        double v = cc[ch];
        if (v < 0) v = 0.0;
        if (v > 1) v = 1.0;
        A.rgb8[3 * (int64_t)idx + ch] = (uint8_t)(255.0 * v);
      }
    }
}

template <int MODE>
__device__ __forceinline__ void flush_stats(const RenderArgs& A, const TravStats& ts, const D3& glight) {
  if (MODE == kRenderStats) {
    unsigned long long a = ts.nodes, b = ts.tris;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(A.stats, a);
      atomicAdd(A.stats + 1, b);
    }
  }
  if (MODE == kAdjoint) {
    warp_add(A.grad_light, glight.x);
    warp_add(A.grad_light + 1, glight.y);
    warp_add(A.grad_light + 2, glight.z);
  }
}

}  // namespace

}  // namespace crt

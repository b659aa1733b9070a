// trace.cu -- traversal and the pixel kernel on sm_103a.
//
// k_trace<ANY>  closest hit (BVH_d::intersect) or first hit in left-first
//               DFS order (BVH_d::intersectAny) for a batch of double rays.
// k_render      runRayTracerKernelRec (kernels/raytracer.cu:95-166) with
//               traceRay (raytracer.cu:169-249), Material::shade
//               (kernels/material.cu:6-40) and the positional Light
//               (kernels/Light.cu:5-86).  Persistent: each warp claims
//               8x4-pixel tiles from a counter, one pixel per lane; a lane
//               runs its pixel's samples in order because the mrand stream
//               couples them (a hit consumes three extra draws).
#include "crt_internal.h"

namespace crt {

namespace {

template <bool ANY>
__global__ void __launch_bounds__(128) k_trace(DScene S, const double* __restrict__ rays, int64_t n,
                                               int* __restrict__ ids, double* __restrict__ tout,
                                               double* __restrict__ nout) {
  float rb[6], B, D;
  scene_consts(S, rb, B, D);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double* r = rays + 6 * i;
    RayC rc;
    ray_setup(rc, r[0], r[1], r[2], r[3], r[4], r[5], B, D);
    HitRec h;
    const int res = traverse<ANY>(S, rc, rb, h);
    if (res < 0) atomicOr(&S.g->err, kErrStack);
    const bool hit = res > 0;
    ids[i] = hit ? h.id : -1;
    if (tout) tout[i] = hit ? h.t : 0.0;
    if (!ANY && nout && hit) {
      const D3 N = hit_normal(S, h);
      nout[3 * i] = N.x, nout[3 * i + 1] = N.y, nout[3 * i + 2] = N.z;
    }
  }
}

__device__ __forceinline__ DMat load_mat(const DScene& S, int tri) {
  return S.mats[__ldg(S.matid + tri)];
}

constexpr int kTileW = 8, kTileH = 4;

template <bool STATS>
__global__ void __launch_bounds__(128, 4) k_render(DScene S, RenderArgs A) {
  TravStats ts;
  float rb[6], B, D;
  scene_consts(S, rb, B, D);
  const int lane = threadIdx.x & 31;
  const int tiles_x = (A.W + kTileW - 1) / kTileW;
  const int tiles_y = (A.row1 - A.row0 + kTileH - 1) / kTileH;
  const int ntiles = tiles_x * tiles_y;
  const int gx = (A.W + 15) / 16;  // gridDim.x of the reference's 16x16 launch
  const D3 lpos = d3(A.lpos[0], A.lpos[1], A.lpos[2]);
  while (true) {
    int tile = 0;
    if (lane == 0) tile = (int)atomicAdd(A.counter, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= ntiles) break;
    const int px = (tile % tiles_x) * kTileW + (lane % kTileW);
    const int py = A.row0 + (tile / tiles_x) * kTileH + (lane / kTileW);
    if (px >= A.W || py >= A.row1) continue;
    const int idx = (A.H - py - 1) * A.W + px;
    // getGlobalIdx_2D_2D (inc/indexing.h:4-9) of the pixel's thread in the
    // reference launch, seeded by initPNRG (kernels/mrand.cu:38-41).
    const uint32_t gid = (uint32_t)(((py / 16) * gx + px / 16) * 256 + (py % 16) * 16 + (px % 16));
    uint32_t st = wang_hash(gid);
    const double xx = (2 * ((px + 0.5) * A.invW) - 1) * A.angle * A.aspect;
    const double yy = (1 - 2 * ((py + 0.5) * A.invH)) * A.angle;
    D3 acc = d3(0, 0, 0);
    for (int k = 0; k < A.spp; k++) {
      const int64_t si = (int64_t)idx * A.spp + k;
      const double dofAngle = 2 * 3.14159265358979323846 * rand_double(st);
      const double dofRadius = A.aperture * sqrt(rand_double(st)) / 2.0;
      D3 org = d3(0.0, 0.0, 0.0);
      if (dofRadius != 0.0) {  // a zero radius gives +-0 components, which no later operation can tell apart
        org = d3(dofRadius * cos(dofAngle), dofRadius * sin(dofAngle), 0.0);
      }
      D3 dir = normalize_exact(d3(xx, yy, -1.0));
      dir = d3(dir.x * A.focal, dir.y * A.focal, dir.z * A.focal) - org;
      dir = normalize_exact(dir);
      if (A.rays) {
        double* rr = A.rays + 6 * si;
        rr[0] = org.x, rr[1] = org.y, rr[2] = org.z, rr[3] = dir.x, rr[4] = dir.y, rr[5] = dir.z;
      }
      RayC rc;
      ray_setup(rc, org.x, org.y, org.z, dir.x, dir.y, dir.z, B, D);
      HitRec h;
      const int res = traverse<false, STATS>(S, rc, rb, h, &ts);
      if (res < 0) atomicOr(&S.g->err, kErrStack);
      D3 col;
      int sh = -1;
      if (res > 0) {
        const D3 q = org + (h.t * dir);
        const DMat m = load_mat(S, h.id);
        const D3 N = hit_normal(S, h);
        D3 I = d3(m.ke[0] + m.ka[0] * 0.0, m.ke[1] + m.ka[1] * 0.0, m.ke[2] + m.ka[2] * 0.0);
        D3 V = d3(A.eye[0], A.eye[1], A.eye[2]) - q;
        V = normalize_exact(d3(-V.x, -V.y, -V.z));
        // Light::getDirection: three draws (x, y, z), times radius, minus 0.5
        const double r0 = rand_double(st), r1 = rand_double(st), r2 = rand_double(st);
        const D3 off = d3(r0 * A.lradius - 0.5, r1 * A.lradius - 0.5, r2 * A.lradius - 0.5);
        const D3 L = normalize_exact(lpos + off - q);
        // Light::distanceAttenuation
        const double dist = norm_exact(lpos - q);
        double fall = A.latt[0] + (A.latt[1] + A.latt[2] * dist) * dist;
        fall = (fabs(fall) < kRayEps) ? 1.0 : 1.0 / fall;
        const double datt = fmin(1.0, fall);
        // Light::shadowAttenuation: any-hit from q towards the light
        D3 satt = d3(1, 1, 1);
        RayC sr;
        ray_setup(sr, q.x, q.y, q.z, L.x, L.y, L.z, B, D);
        HitRec s;
        const int sres = traverse<true, STATS>(S, sr, rb, s, &ts);
        if (sres < 0) atomicOr(&S.g->err, kErrStack);
        sh = 0;
        if (sres > 0 && s.t < norm_exact(lpos - q) && !(s.t < kRayEps)) {
          sh = 1;
          const DMat om = load_mat(S, s.id);
          const bool trans = om.kt[0] == 0 && om.kt[1] == 0 && om.kt[2] == 0;  // Trans() = isZero(kt)
          satt = trans ? d3(om.kd[0] * (1 - om.kt[0]), om.kd[1] * (1 - om.kt[1]), om.kd[2] * (1 - om.kt[2]))
                       : d3(0, 0, 0);
        }
        const D3 att = datt * satt;
        double lam = dot(N, L);
        if (lam < 0) lam = 0;
        const D3 diffuse = d3(m.kd[0] * lam, m.kd[1] * lam, m.kd[2] * lam);
        D3 R = (-2.0 * dot(L, N)) * N + L;
        R = normalize_exact(R);
        double sp = dot(R, V);
        sp = (double)powf(__double2float_rn(fmax(0.0, sp)), __double2float_rn(m.shininess));
        const D3 spec = d3(m.ks[0] * sp, m.ks[1] * sp, m.ks[2] * sp);
        const D3 ds = diffuse + spec;
        I = I + d3(att.x * ds.x * A.lcol[0], att.y * ds.y * A.lcol[1], att.z * ds.z * A.lcol[2]);
        col = I;
      } else {
        col = d3(0.9, 0.9, 0.9);
      }
      acc = acc + col;
      if (A.hit_id) A.hit_id[si] = res > 0 ? h.id : -1;
      if (A.hit_t) A.hit_t[si] = res > 0 ? h.t : 0.0;
      if (A.shadow) A.shadow[si] = sh;
    }
    const double inv = (double)A.spp;
    acc = d3(acc.x / inv, acc.y / inv, acc.z / inv);
    if (A.rgbf) {
      A.rgbf[3 * (int64_t)idx] = (float)acc.x;
      A.rgbf[3 * (int64_t)idx + 1] = (float)acc.y;
      A.rgbf[3 * (int64_t)idx + 2] = (float)acc.z;
    }
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
  if (STATS) {
    unsigned long long a = ts.nodes, b = ts.tris;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
      atomicAdd(A.stats, a);
      atomicAdd(A.stats + 1, b);
    }
  }
}

}  // namespace

cudaError_t launch_render(const DScene& S, const RenderArgs& a, cudaStream_t st) {
  cudaMemsetAsync(a.counter, 0, sizeof(unsigned), st);
  int bps = 0;
  if (a.stats) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_render<true>, 128, 0);
    k_render<true><<<num_sms() * (bps > 0 ? bps : 1), 128, 0, st>>>(S, a);
  } else {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_render<false>, 128, 0);
    k_render<false><<<num_sms() * (bps > 0 ? bps : 1), 128, 0, st>>>(S, a);
  }
  return cudaGetLastError();
}

cudaError_t launch_trace(const DScene& S, const double* rays, int64_t n, bool any, int* ids, double* t,
                         double* normals, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  int bps = 0;
  if (any)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_trace<true>, 128, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_trace<false>, 128, 0);
  if (bps <= 0) bps = 1;
  const int64_t need = (n + 127) / 128;
  const int grid = (int)(need < (int64_t)num_sms() * bps ? need : (int64_t)num_sms() * bps);
  if (any)
    k_trace<true><<<grid, 128, 0, st>>>(S, rays, n, ids, t, nullptr);
  else
    k_trace<false><<<grid, 128, 0, st>>>(S, rays, n, ids, t, normals);
  return cudaGetLastError();
}

}  // namespace crt

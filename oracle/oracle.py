"""ctypes front end of the CPU oracle (crt_oracle.cpp) and of the reference
compiled for the host (oracle/_ref/libcrtref.so, see ref/build_ref.py).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libcrtref.so")


def build_oracle(quiet=False) -> str:
    src = os.path.join(HERE, "crt_oracle.cpp")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                               "-o", LIB, src])
        if not quiet:
            print(f"oracle: built {LIB}")
    return LIB


class _Cam(C.Structure):
    _fields_ = [("fov", C.c_double), ("focal_point", C.c_double), ("fstop", C.c_double), ("eye", C.c_double * 3)]


class _Light(C.Structure):
    _fields_ = [("color", C.c_double * 3), ("position", C.c_double * 3), ("radius", C.c_double),
                ("constant_term", C.c_double), ("linear_term", C.c_double), ("quadratic_term", C.c_double)]


def _ptr(a, ct):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


_libs = {}


def _load(path, prefix):
    key = (path, prefix)
    if key in _libs:
        return _libs[key]
    lib = C.CDLL(path)
    vp = C.c_void_p
    getattr(lib, prefix + "scene_create").restype = vp
    getattr(lib, prefix + "scene_create").argtypes = [C.c_int, vp, C.c_int, vp, C.c_int, vp, vp, C.c_int, vp, vp]
    getattr(lib, prefix + "scene_destroy").argtypes = [vp]
    getattr(lib, prefix + "export").argtypes = [vp] * 9
    getattr(lib, prefix + "trace").argtypes = [vp, vp, C.c_int, C.c_int, vp, vp, vp, C.c_int]
    _libs[key] = lib
    return lib


class OracleScene:
    """One mesh built by the oracle (prefix 'orc_') or by the reference's own
    code on the CPU (prefix 'ref_')."""

    def __init__(self, mesh, kind="oracle"):
        if kind == "oracle":
            self.lib, self.p = _load(build_oracle(quiet=True), "orc_"), "orc_"
        else:
            if not os.path.exists(REF_LIB):
                raise FileNotFoundError(REF_LIB)
            self.lib, self.p = _load(REF_LIB, "ref_"), "ref_"
        self.kind = kind
        self.mesh = mesh
        self._keep = [np.ascontiguousarray(mesh.verts, np.float32), np.ascontiguousarray(mesh.normals, np.float32),
                      np.ascontiguousarray(mesh.vidx, np.int32), np.ascontiguousarray(mesh.nidx, np.int32),
                      np.ascontiguousarray(mesh.materials, np.float64), np.ascontiguousarray(mesh.matid, np.int32)]
        v, n, vi, ni, mats, mid = self._keep
        self.n = int(vi.shape[0])
        self.h = getattr(self.lib, self.p + "scene_create")(
            v.shape[0], v.ctypes.data, n.shape[0], n.ctypes.data, self.n, vi.ctypes.data, ni.ctypes.data,
            mats.shape[0], mats.ctypes.data, mid.ctypes.data)
        if not self.h:
            raise MemoryError("oracle scene")

    def close(self):
        if getattr(self, "h", None):
            getattr(self.lib, self.p + "scene_destroy")(self.h)
            self.h = None

    __del__ = close

    def set_vertices(self, verts, rebuild: bool):
        assert self.kind == "oracle"
        v = np.ascontiguousarray(verts, np.float32)
        self._keep[0] = v
        self.lib.orc_scene_set_vertices.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        self.lib.orc_scene_set_vertices(self.h, v.ctypes.data, int(rebuild))

    def export(self) -> dict:
        n = self.n
        nn = max(2 * n - 1, 0)
        out = dict(smin=np.zeros(3), smax=np.zeros(3), codes_unsorted=np.zeros(n, np.int32),
                   codes=np.zeros(n, np.int32), ids=np.zeros(n, np.uint32), nodes=np.zeros((nn, 3), np.int32),
                   node_boxes=np.zeros((nn, 6), np.float32), tri_boxes=np.zeros((n, 6), np.float32))
        r = getattr(self.lib, self.p + "export")(self.h, *[out[k].ctypes.data for k in (
            "smin", "smax", "codes_unsorted", "codes", "ids", "nodes", "node_boxes", "tri_boxes")])
        if self.kind == "ref" and r:
            raise AssertionError("reference box value not representable as float")
        return out

    def trace(self, rays: np.ndarray, any_hit=False, nthreads=0):
        rays = np.ascontiguousarray(rays, np.float64).reshape(-1, 6)
        m = rays.shape[0]
        ids = np.zeros(m, np.int32)
        t = np.zeros(m, np.float64)
        nrm = np.zeros((m, 3), np.float64)
        getattr(self.lib, self.p + "trace")(self.h, rays.ctypes.data, m, int(any_hit), ids.ctypes.data,
                                            t.ctypes.data, nrm.ctypes.data, nthreads)
        return ids, t, nrm

    def render(self, cam, light, width, height, spp=None, rows=None, aux=False, rays_in=None, rays_out=False,
               nthreads=0, seed=0):
        """Render rows [r0, r1) (default: all).  The reference ('ref') always
        takes 20 samples per pixel."""
        r0, r1 = rows if rows is not None else (0, height)
        c = _Cam(cam.fov, cam.focal_point, cam.fstop, (C.c_double * 3)(*cam.eye))
        L = _Light((C.c_double * 3)(*light.color), (C.c_double * 3)(*light.position), light.radius,
                   light.constant_term, light.linear_term, light.quadratic_term)
        npx = width * height
        rgb = np.zeros((npx, 3), np.uint8)
        col = np.zeros((npx, 3), np.float64)
        if self.kind == "ref":
            if spp not in (None, 20):
                raise ValueError("the reference's pixel kernel always takes 20 samples")
            f = self.lib.ref_render
            f.argtypes = [C.c_void_p, C.POINTER(_Cam), C.POINTER(_Light), C.c_int, C.c_int, C.c_int, C.c_int,
                          C.c_void_p, C.c_void_p, C.c_int]
            f(self.h, C.byref(c), C.byref(L), width, height, r0, r1, rgb.ctypes.data, col.ctypes.data, nthreads)
            return dict(rgb=rgb, color=col)
        spp = 20 if spp is None else spp
        hid = np.zeros(npx * spp, np.int32) if aux else None
        ht = np.zeros(npx * spp, np.float64) if aux else None
        sh = np.zeros(npx * spp, np.int32) if aux else None
        shid = np.zeros(npx * spp, np.int32) if aux else None
        ro = np.zeros((npx * spp, 6), np.float64) if rays_out else None
        ri = None if rays_in is None else np.ascontiguousarray(rays_in, np.float64)
        f = self.lib.orc_render
        f.restype = C.c_int
        f.argtypes = [C.c_void_p, C.POINTER(_Cam), C.POINTER(_Light), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                      C.c_void_p, C.c_uint32]
        g = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        ov = f(self.h, C.byref(c), C.byref(L), width, height, spp, r0, r1, rgb.ctypes.data, col.ctypes.data,
               g(hid), g(ht), g(sh), g(ri), g(ro), nthreads, g(shid), seed)
        out = dict(rgb=rgb, color=col, overflow=ov)
        if aux:
            out.update(hit_id=hid, hit_t=ht, shadow=sh, shadow_id=shid)
        if rays_out:
            out["rays"] = ro
        return out


def _render_rec(self, cam, light, width, height, spp, depth, optics=None, rays_in=None, rays_out=False, nthreads=0,
                seed=0):
    """orc_render_rec: traceRay with `depth` levels of reflection and
    refraction.  optics: (num_materials, 4) kr xyz + ior, or None (kr = ks,
    ior = 1)."""
    assert self.kind == "oracle"
    c = _Cam(cam.fov, cam.focal_point, cam.fstop, (C.c_double * 3)(*cam.eye))
    L = _Light((C.c_double * 3)(*light.color), (C.c_double * 3)(*light.position), light.radius,
               light.constant_term, light.linear_term, light.quadratic_term)
    npx = width * height
    rgb = np.zeros((npx, 3), np.uint8)
    col = np.zeros((npx, 3), np.float64)
    hid = np.zeros(npx * spp, np.int32)
    ht = np.zeros(npx * spp, np.float64)
    ro = np.zeros((npx * spp, 6), np.float64) if rays_out else None
    ri = None if rays_in is None else np.ascontiguousarray(rays_in, np.float64)
    op = None if optics is None else np.ascontiguousarray(optics, np.float64).reshape(-1, 4)
    g = lambda a: None if a is None else a.ctypes.data  # noqa: E731
    f = self.lib.orc_render_rec
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.POINTER(_Cam), C.POINTER(_Light), C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                  C.c_uint32]
    counts = np.zeros(2, np.int64)
    ov = f(self.h, C.byref(c), C.byref(L), width, height, spp, depth, g(op), rgb.ctypes.data, col.ctypes.data,
           hid.ctypes.data, ht.ctypes.data, g(ri), g(ro), nthreads, counts.ctypes.data, seed)
    out = dict(rgb=rgb, color=col, hit_id=hid, hit_t=ht, overflow=ov, counts=counts.tolist())
    if rays_out:
        out["rays"] = ro
    return out


OracleScene.render_recursive = _render_rec


def _adjoint(self, cam, light, width, height, spp, grad_rgb, grad_depth=None, nthreads=0):
    """Float64 reference gradient (orc_adjoint)."""
    assert self.kind == "oracle"
    c = _Cam(cam.fov, cam.focal_point, cam.fstop, (C.c_double * 3)(*cam.eye))
    L = _Light((C.c_double * 3)(*light.color), (C.c_double * 3)(*light.position), light.radius,
               light.constant_term, light.linear_term, light.quadratic_term)
    g = np.ascontiguousarray(grad_rgb, np.float64)
    gd = None if grad_depth is None else np.ascontiguousarray(grad_depth, np.float64)
    gv = np.zeros((self.mesh.verts.shape[0], 3))
    gl = np.zeros(3)
    gk = np.zeros((np.asarray(self.mesh.materials).reshape(-1, 16).shape[0], 3))
    f = self.lib.orc_adjoint
    f.argtypes = [C.c_void_p, C.POINTER(_Cam), C.POINTER(_Light), C.c_int, C.c_int, C.c_int, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    f(self.h, C.byref(c), C.byref(L), width, height, spp, g.ctypes.data, None if gd is None else gd.ctypes.data,
      gv.ctypes.data, gl.ctypes.data, gk.ctypes.data, nthreads)
    return dict(vertices=gv, light=gl, kd=gk)


OracleScene.adjoint = _adjoint


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def camera_angle(fov):
    """tan(pi*0.5*fov/180) as the reference's pixel kernel computes it."""
    return math.tan(math.pi * 0.5 * fov / 180.0)

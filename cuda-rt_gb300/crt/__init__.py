"""Python front end of libcrt.so (the C ABI in include/crt.h), via ctypes.

The names mirror the reference's host API (inc/raytracer.h, inc/scene.h,
inc/camera.h, inc/Light.h): a ``Scene`` is Scene_d with its BVH_d, built on
construction like ``Scene_d::operator=(const Scene_h&)``; ``render`` is
RayTracer::run + pullRaytracedImage.  Buffers may be NumPy arrays (host) or
torch CUDA tensors (device); the library copies as needed.

The CUDA library is required: importing ``crt`` raises if libcrt.so is
missing, and nothing here falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import data  # noqa: F401
from .build import LIB as LIB_PATH

__all__ = ["CrtError", "Scene", "Batch", "load_obj_native", "write_bmp", "lib", "sort_pairs", "sort_pairs_noalloc", "morton", "STATUS", "render_args"]

STATUS = {0: "CRT_OK", 1: "CRT_INVALID_ARG", 2: "CRT_OOM", 3: "CRT_CUDA_ERROR", 4: "CRT_STACK_OVERFLOW",
          5: "CRT_TIMEOUT", 6: "CRT_NOT_BUILT"}


class CrtError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class _Material(C.Structure):
    _fields_ = [("ka", C.c_double * 3), ("kd", C.c_double * 3), ("ks", C.c_double * 3), ("kt", C.c_double * 3),
                ("ke", C.c_double * 3), ("shininess", C.c_double)]


class _MeshDesc(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("num_vertices", C.c_int32), ("normals", C.c_void_p),
                ("num_normals", C.c_int32), ("vertex_indices", C.c_void_p), ("normal_indices", C.c_void_p),
                ("num_triangles", C.c_int32), ("materials", C.c_void_p), ("num_materials", C.c_int32),
                ("material_ids", C.c_void_p)]


class _Camera(C.Structure):
    _fields_ = [("fov", C.c_double), ("focal_point", C.c_double), ("fstop", C.c_double), ("eye", C.c_double * 3)]


class _Light(C.Structure):
    _fields_ = [("color", C.c_double * 3), ("position", C.c_double * 3), ("radius", C.c_double),
                ("constant_term", C.c_double), ("linear_term", C.c_double), ("quadratic_term", C.c_double)]


class _RenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("row_begin", C.c_int32),
                ("row_end", C.c_int32), ("seed", C.c_uint32)]


class _RenderOut(C.Structure):
    _fields_ = [("rgb8", C.c_void_p), ("rgb_f32", C.c_void_p), ("hit_id", C.c_void_p), ("hit_t", C.c_void_p),
                ("shadow", C.c_void_p), ("rays", C.c_void_p), ("traversal_stats", C.c_void_p),
                ("rgb_f64", C.c_void_p), ("depth", C.c_void_p), ("shadow_id", C.c_void_p)]


class _BatchView(C.Structure):
    _fields_ = [("camera", _Camera), ("light", _Light), ("width", C.c_int32), ("height", C.c_int32),
                ("spp", C.c_int32)]


class _BatchTuning(C.Structure):
    _fields_ = [("block_size", C.c_int32), ("lanes_per_pixel", C.c_int32), ("stack", C.c_int32),
                ("render_ms", C.c_float), ("launches", C.c_int32)]


_lib = None


def lib():
    """Load libcrt.so (build it first with ``__graft_entry__.build()``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libcrt.so not built ({LIB_PATH}); run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        sig = {
            "crt_scene_create": [vp, vp, vp],
            "crt_scene_create_borrowed": [vp, vp, vp],
            "crt_scene_destroy": [vp],
            "crt_scene_set_vertices": [vp, vp, C.c_int, vp],
            "crt_bvh_build": [vp, vp],
            "crt_bvh_refit": [vp, vp],
            "crt_bvh_export": [vp, vp, vp, vp, vp, vp, vp],
            "crt_trace_closest": [vp, vp, i64, vp, vp, vp, vp],
            "crt_trace_shadow": [vp, vp, i64, vp, vp, vp],
            "crt_render": [vp, vp, vp, vp, vp, vp],
            "crt_render_recursive": [vp, vp, vp, vp, i32, vp, vp, vp],
            "crt_set_lens_tables": [i32],
            "crt_morton": [vp, i32, vp, i32, vp, vp, vp],
            "crt_hierarchy": [vp, vp, i32, vp, vp],
            "crt_refit": [vp, i32, vp, i32, vp, vp, vp, vp],
            "crt_sort_pairs": [vp, vp, vp, vp, i32, i32, vp],
            "crt_sort_pairs_noalloc": [vp, vp, vp, vp, i32, i32, vp],
            "crt_scene_check": [vp, vp],
            "crt_scene_set_materials": [vp, vp, i32, vp],
            "crt_adjoint_lambert": [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp],
            "crt_batch_create": [vp, vp, i32, vp, vp],
            "crt_batch_destroy": [vp],
            "crt_batch_run": [vp, i32, vp, vp],
            "crt_batch_set_tuning": [vp, vp],
            "crt_batch_autotune": [vp, vp, vp],
            "crt_batch_export": [vp, i32, vp, vp, vp, vp, vp, vp],
            "crt_batch_check": [vp, vp],
            "crt_obj_load": [C.c_char_p, C.c_char_p, vp],
            "crt_obj_mesh": [vp, vp],
            "crt_obj_optics": [vp, vp],
            "crt_obj_free": [vp],
            "crt_write_bmp": [C.c_char_p, i32, i32, vp],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L.crt_last_error_string.restype = C.c_char_p
        L.crt_version.restype = C.c_char_p
        _lib = L
    return _lib


def _check(status):
    if status != 0:
        raise CrtError(status, lib().crt_last_error_string().decode())


def _addr(a):
    """Address of a contiguous NumPy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array is not C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor is not contiguous")
        return a.data_ptr()
    raise TypeError(type(a))


def _kind(a):
    """(kind, item size, element count) of a NumPy array or torch tensor;
    kind is NumPy's letter: u unsigned, i signed, f floating point."""
    if isinstance(a, np.ndarray):
        return a.dtype.kind, a.dtype.itemsize, a.size
    name = str(a.dtype).replace("torch.", "")
    kind = "u" if name.startswith(("uint", "bool")) else "i" if name.startswith(("int", "long", "short")) else \
        "f" if name.startswith(("float", "double", "half", "bfloat")) else "?"
    return kind, a.element_size(), a.numel()


def _need(a, name, kinds, itemsize, count):
    """A caller's buffer that the library reads or writes `count` elements of:
    the C ABI takes bare pointers, so type and size are checked here."""
    if a is None:
        return
    k, size, n = _kind(a)
    if k not in kinds or size != itemsize:
        raise TypeError(f"{name}: {a.dtype} is not the {kinds[0]}{8 * itemsize} the library uses")
    if n < count:
        raise ValueError(f"{name}: {n} elements, {count} needed")


# crt_render_out's buffers: (key, kinds, item size, elements per pixel, per sample, fixed)
_RENDER_OUT = (("rgb8", "u", 1, 3, 0, 0), ("rgb_f32", "f", 4, 3, 0, 0), ("hit_id", "i", 4, 0, 1, 0),
               ("hit_t", "f", 8, 0, 1, 0), ("shadow", "i", 4, 0, 1, 0), ("rays", "f", 8, 0, 6, 0),
               ("traversal_stats", "ui", 8, 0, 0, 2), ("rgb_f64", "f", 8, 3, 0, 0), ("depth", "f", 8, 1, 0, 0),
               ("shadow_id", "i", 4, 0, 1, 0))


def _render_out(out, npx, ns):
    """crt_render_out over the dict's buffers, each checked for its type and
    for the full image's size (a row band writes at full-image indices)."""
    for key, kinds, size, per_px, per_s, fixed in _RENDER_OUT:
        _need(out.get(key), key, kinds, size, per_px * npx + per_s * ns + fixed)
    return _RenderOut(*[_addr(out.get(k[0])) for k in _RENDER_OUT])


def _stream(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


class Scene:
    """Scene_d + BVH_d: a mesh on the GPU with its LBVH (built on construction).
    borrow=True (crt_scene_create_borrowed): the mesh's arrays are CUDA
    tensors that the scene uses in place (kept referenced here); rewrite the
    vertex tensor and call set_vertices(None, rebuild) to refit from it."""

    def __init__(self, mesh, stream=None, borrow=False):
        self._keep = []

        def hold(a, dt):
            if a is None:
                return None
            if isinstance(a, np.ndarray):
                a = np.ascontiguousarray(a, dt)
            self._keep.append(a)
            return _addr(a)

        mats = mesh.materials
        if not hasattr(mats, "data_ptr"):  # device tensors are passed as they are
            mats = np.ascontiguousarray(np.asarray(mats, np.float64).reshape(-1, 16))
        self.ntri = int(mesh.vidx.shape[0])
        self.nv = int(mesh.verts.shape[0])
        self.nmat = int(mats.shape[0])
        d = _MeshDesc(hold(mesh.verts, np.float32), self.nv, hold(mesh.normals, np.float32),
                      int(mesh.normals.shape[0]), hold(mesh.vidx, np.int32), hold(mesh.nidx, np.int32), self.ntri,
                      hold(mats, np.float64), int(mats.shape[0]), hold(mesh.matid, np.int32))
        h = C.c_void_p()
        create = lib().crt_scene_create_borrowed if borrow else lib().crt_scene_create
        _check(create(C.byref(d), _stream(stream), C.byref(h)))
        self.h = h
        if not borrow:
            self._keep = []

    def close(self):
        if getattr(self, "h", None):
            lib().crt_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_vertices(self, verts, rebuild: bool, stream=None):
        """New vertex positions (None: a borrowing scene re-reads its own)."""
        if isinstance(verts, np.ndarray):
            verts = np.ascontiguousarray(verts, np.float32)
        _need(verts, "vertices", "f", 4, 3 * self.nv)
        _check(lib().crt_scene_set_vertices(self.h, _addr(verts), int(bool(rebuild)), _stream(stream)))

    def build(self, stream=None):
        _check(lib().crt_bvh_build(self.h, _stream(stream)))

    def refit(self, stream=None):
        _check(lib().crt_bvh_refit(self.h, _stream(stream)))

    def check(self, stream=None):
        _check(lib().crt_scene_check(self.h, _stream(stream)))

    def set_materials(self, materials, stream=None):
        """Replace the material table ((M, 16) float64: ka kd ks kt ke, shininess)."""
        m = materials
        if isinstance(m, np.ndarray):
            m = np.ascontiguousarray(m, np.float64)
        _check(lib().crt_scene_set_materials(self.h, _addr(m), int(m.shape[0]), _stream(stream)))

    def adjoint(self, camera, light, width, height, spp, grad_rgb, grad_depth=None, out=None, stream=None):
        """crt_adjoint_lambert: d loss / d (vertices, light position, kd) given
        d loss / d rgb_f64 (and optionally d loss / d depth)."""
        cam, lt, p = render_args(camera, light, width, height, spp, None)
        if out is None:
            out = dict(vertices=np.zeros((self.nv, 3), np.float64), light=np.zeros(3, np.float64),
                       kd=np.zeros((self.nmat, 3), np.float64))
        npx = width * height
        for a, name, count in ((grad_rgb, "grad_rgb", 3 * npx), (grad_depth, "grad_depth", npx),
                               (out.get("vertices"), "vertices", 3 * self.nv), (out.get("light"), "light", 3),
                               (out.get("kd"), "kd", 3 * self.nmat)):
            _need(a, name, "f", 8, count)
        _check(lib().crt_adjoint_lambert(self.h, C.byref(cam), C.byref(lt), C.byref(p), _addr(grad_rgb),
                                         _addr(grad_depth), _addr(out.get("vertices")), _addr(out.get("light")),
                                         _addr(out.get("kd")), _stream(stream)))
        return out

    def export(self) -> dict:
        n = self.ntri
        nn = max(2 * n - 1, 0)
        out = dict(scene_box=np.zeros(6, np.float32), codes=np.zeros(n, np.int32), ids=np.zeros(n, np.uint32),
                   nodes=np.zeros((nn, 3), np.int32), node_boxes=np.zeros((nn, 6), np.float32))
        _check(lib().crt_bvh_export(self.h, *[_addr(out[k]) for k in ("scene_box", "codes", "ids", "nodes",
                                                                        "node_boxes")], None))
        return out

    def trace(self, rays, any_hit=False, normals=False, stream=None):
        """rays: (n, 6) float64 (NumPy or CUDA tensor).  Returns ids, t[, normals]."""
        n = int(rays.shape[0])
        if isinstance(rays, np.ndarray):
            rays = np.ascontiguousarray(rays, np.float64)
            ids, t = np.zeros(n, np.int32), np.zeros(n, np.float64)
            nrm = np.zeros((n, 3), np.float64) if normals and not any_hit else None
        else:
            import torch
            _need(rays, "rays", "f", 8, 6 * n)
            ids = torch.empty(n, dtype=torch.int32, device=rays.device)
            t = torch.empty(n, dtype=torch.float64, device=rays.device)
            nrm = torch.empty((n, 3), dtype=torch.float64, device=rays.device) if normals and not any_hit else None
        if any_hit:
            _check(lib().crt_trace_shadow(self.h, _addr(rays), n, _addr(ids), _addr(t), _stream(stream)))
        else:
            _check(lib().crt_trace_closest(self.h, _addr(rays), n, _addr(ids), _addr(t), _addr(nrm),
                                           _stream(stream)))
        return (ids, t, nrm) if normals and not any_hit else (ids, t)

    def render(self, camera, light, width, height, spp, rows=None, out=None, aux=False, rays=False, rgbf=False,
               rgbd=False, stream=None, seed=0):
        """RayTracer::run + pullRaytracedImage.  Returns a dict of NumPy
        arrays unless `out` (a dict of preallocated buffers) is given."""
        cam, lt, p = render_args(camera, light, width, height, spp, rows, seed)
        if out is None:
            npx, ns = width * height, width * height * spp
            out = dict(rgb8=np.zeros((npx, 3), np.uint8))
            if rgbf:
                out["rgb_f32"] = np.zeros((npx, 3), np.float32)
            if rgbd:
                out["rgb_f64"] = np.zeros((npx, 3), np.float64)
                out["depth"] = np.zeros(npx, np.float64)
            if aux:
                out.update(hit_id=np.zeros(ns, np.int32), hit_t=np.zeros(ns, np.float64),
                           shadow=np.zeros(ns, np.int32), shadow_id=np.zeros(ns, np.int32))
            if rays:
                out["rays"] = np.zeros((ns, 6), np.float64)
        o = _render_out(out, width * height, width * height * spp)
        _check(lib().crt_render(self.h, C.byref(cam), C.byref(lt), C.byref(p), C.byref(o), _stream(stream)))
        return out


    def render_recursive(self, camera, light, width, height, spp, depth, optics=None, rows=None, rays=False,
                         out=None, stream=None):
        """crt_render_recursive: traceRay with `depth` levels of reflected and
        refracted rays.  optics: (num_materials, 4) array of kr xyz and ior,
        or None (kr = ks, ior = 1).  Returns rgb8, rgb_f64, the primary hit_id
        and hit_t, and (rays=True) the primary rays, unless `out` (a dict of
        preallocated buffers: rgb8, rgb_f32, rgb_f64, hit_id, hit_t, rays) is
        given."""
        cam, lt, p = render_args(camera, light, width, height, spp, rows)
        npx, ns = width * height, width * height * spp
        if out is None:
            out = dict(rgb8=np.zeros((npx, 3), np.uint8), rgb_f64=np.zeros((npx, 3), np.float64),
                       hit_id=np.zeros(ns, np.int32), hit_t=np.zeros(ns, np.float64))
            if rays:
                out["rays"] = np.zeros((ns, 6), np.float64)
        if optics is None or hasattr(optics, "data_ptr"):
            op = optics  # None, or a device tensor of num_materials x 4 doubles
        else:
            op = np.ascontiguousarray(optics, np.float64).reshape(-1, 4)
        _need(op, "optics", "f", 8, 4 * self.nmat)
        o = _render_out(out, npx, ns)
        _check(lib().crt_render_recursive(self.h, C.byref(cam), C.byref(lt), C.byref(p), int(depth), _addr(op),
                                          C.byref(o), _stream(stream)))
        return out


class Batch:
    """Many meshes, each with its own camera, light and image size, built and
    rendered together (crt_batch_*).  `meshes` are data.Mesh objects, `views`
    (camera, light, width, height, spp) tuples."""

    def __init__(self, meshes, views, stream=None):
        keep = []

        def hold(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dt)
            keep.append(a)
            return a.ctypes.data

        M = len(meshes)
        descs = (_MeshDesc * M)()
        vws = (_BatchView * M)()
        self.sizes, self.ntri = [], []
        for m, (mesh, (cam, light, w, h, spp)) in enumerate(zip(meshes, views)):
            mats = np.asarray(mesh.materials, np.float64).reshape(-1, 16)
            descs[m] = _MeshDesc(hold(mesh.verts, np.float32), int(mesh.verts.shape[0]),
                                 hold(mesh.normals, np.float32), int(mesh.normals.shape[0]),
                                 hold(mesh.vidx, np.int32), hold(mesh.nidx, np.int32), int(mesh.vidx.shape[0]),
                                 hold(mats, np.float64), int(mats.shape[0]), hold(mesh.matid, np.int32))
            c, lt, _ = render_args(cam, light, w, h, spp)
            vws[m] = _BatchView(c, lt, w, h, spp)
            self.sizes.append((w, h, spp))
            self.ntri.append(int(mesh.vidx.shape[0]))
        self.M = M
        self.pixels = [w * h for (w, h, _) in self.sizes]
        self.offsets = np.concatenate([[0], np.cumsum(self.pixels)]).astype(np.int64)
        self.rays = sum(w * h * s for (w, h, s) in self.sizes)
        h = C.c_void_p()
        _check(lib().crt_batch_create(descs, vws, M, _stream(stream), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().crt_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, out=None, graph=True, stream=None):
        """Build and render everything; `out` is a (total pixels, 3) uint8
        NumPy array or CUDA tensor, or None to keep the images on the device."""
        _need(out, "out", "u", 1, 3 * sum(self.pixels))
        _check(lib().crt_batch_run(self.h, int(bool(graph)), _addr(out), _stream(stream)))
        return out

    def images(self, out):
        """Split run()'s concatenated output into per-mesh (W*H, 3) views."""
        return [out[self.offsets[m]:self.offsets[m + 1]] for m in range(self.M)]

    def set_tuning(self, block_size, lanes_per_pixel, stack, launches=2):
        """launches = 1: build and render in one persistent launch; 2: the
        render in a launch of its own."""
        t = _BatchTuning(block_size, lanes_per_pixel, stack, 0.0, launches)
        _check(lib().crt_batch_set_tuning(self.h, C.byref(t)))

    def autotune(self, stream=None):
        t = _BatchTuning()
        _check(lib().crt_batch_autotune(self.h, C.byref(t), _stream(stream)))
        return dict(block_size=t.block_size, lanes_per_pixel=t.lanes_per_pixel, stack=t.stack,
                    launches=t.launches, render_ms=float(t.render_ms))

    def check(self, stream=None):
        _check(lib().crt_batch_check(self.h, _stream(stream)))

    def export(self, m, stream=None) -> dict:
        n = self.ntri[m]
        nn = 2 * n - 1
        out = dict(scene_box=np.zeros(6, np.float32), codes=np.zeros(n, np.int32), ids=np.zeros(n, np.uint32),
                   nodes=np.zeros((nn, 3), np.int32), node_boxes=np.zeros((nn, 6), np.float32))
        _check(lib().crt_batch_export(self.h, m, *[_addr(out[k]) for k in ("scene_box", "codes", "ids", "nodes",
                                                                            "node_boxes")], _stream(stream)))
        return out


def load_obj_native(path, mtl_dir=None, with_optics=False):
    """crt_obj_load: the library's OBJ/MTL reader (host only), as a data.Mesh;
    with_optics also returns crt_obj_optics as a (num_materials, 4) array of
    kr xyz (= Ks) and ior (= Ni)."""
    from .data import Mesh
    h = C.c_void_p()
    _check(lib().crt_obj_load(os.fsencode(path), None if mtl_dir is None else os.fsencode(mtl_dir), C.byref(h)))
    try:
        d = _MeshDesc()
        _check(lib().crt_obj_mesh(h, C.byref(d)))

        def arr(ptr, n, ct, dt, shape):
            if n == 0:
                return np.zeros(shape, dt)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), (n,)).astype(dt).reshape(shape)

        n, nv, nn, nm = d.num_triangles, d.num_vertices, d.num_normals, d.num_materials
        optics = np.zeros((nm, 4), np.float64)
        _check(lib().crt_obj_optics(h, optics.ctypes.data))
        mesh = Mesh(arr(d.vertices, 3 * nv, C.c_float, np.float32, (nv, 3)),
                    arr(d.vertex_indices, 3 * n, C.c_int32, np.int32, (n, 3)),
                    arr(d.normals, 3 * nn, C.c_float, np.float32, (nn, 3)),
                    arr(d.normal_indices, 3 * n, C.c_int32, np.int32, (n, 3)),
                    arr(d.material_ids, n, C.c_int32, np.int32, (n,)),
                    arr(d.materials, 16 * nm, C.c_double, np.float64, (nm, 16)))
        return (mesh, optics) if with_optics else mesh
    finally:
        lib().crt_obj_free(h)


def write_bmp(path, rgb8, width, height):
    """crt_write_bmp: a 24-bit BMP of an rgb8 image in the library's bottom-up order."""
    a = np.ascontiguousarray(rgb8, np.uint8)
    assert a.size == 3 * width * height
    _check(lib().crt_write_bmp(os.fsencode(path), width, height, a.ctypes.data))


def render_args(camera, light, width, height, spp, rows=None, seed=0):
    cam = _Camera(camera.fov, camera.focal_point, camera.fstop, (C.c_double * 3)(*camera.eye))
    lt = _Light((C.c_double * 3)(*light.color), (C.c_double * 3)(*light.position), light.radius,
                light.constant_term, light.linear_term, light.quadratic_term)
    r0, r1 = rows if rows is not None else (0, 0)
    return cam, lt, _RenderParams(width, height, spp, r0, r1, seed)


def _need_words(a, name, count, allow_none=False):
    """A 1-D array of 4-byte integers with at least `count` elements (the
    stage entry points take bare device pointers to 32-bit words)."""
    if a is None:
        if allow_none:
            return
        raise ValueError(f"{name}: an array is required")
    if len(a.shape) != 1:
        raise ValueError(f"{name}: {len(a.shape)}-D, a 1-D array is required")
    _need(a, name, "iu", 4, count)


def morton(verts, vidx, scene_box, codes, stream=None):
    """crt_morton on device tensors."""
    n = int(vidx.shape[0])
    _need(verts, "verts", "f", 4, 3 * int(verts.shape[0]))
    _need(vidx, "vidx", "i", 4, 3 * n)
    _need(scene_box, "scene_box", "f", 4, 6)
    _need_words(codes, "codes", n)
    _check(lib().crt_morton(_addr(verts), int(verts.shape[0]), _addr(vidx), n, _addr(scene_box),
                            _addr(codes), _stream(stream)))


def _sort_args(keys_in, vals_in, keys_out, vals_out):
    _need_words(keys_in, "keys_in", 0)
    n = int(keys_in.shape[0])
    _need_words(vals_in, "vals_in", n, allow_none=True)
    _need_words(keys_out, "keys_out", n)
    _need_words(vals_out, "vals_out", n)
    return n


def sort_pairs(keys_in, vals_in, keys_out, vals_out, key_bits=32, stream=None):
    """crt_sort_pairs on device tensors (stable LSD radix sort; 1-D 32-bit
    integer arrays, outputs at least as long as keys_in, no overlap)."""
    n = _sort_args(keys_in, vals_in, keys_out, vals_out)
    _check(lib().crt_sort_pairs(_addr(keys_in), _addr(vals_in), _addr(keys_out), _addr(vals_out), n, key_bits,
                                _stream(stream)))


def sort_pairs_noalloc(keys_in, vals_in, keys_out, vals_out, key_bits=32, stream=None):
    """crt_sort_pairs_noalloc on device tensors: the same sort with its scratch
    in a fixed device array (at most CRT_SORT_NOALLOC_MAX_PAIRS pairs)."""
    n = _sort_args(keys_in, vals_in, keys_out, vals_out)
    _check(lib().crt_sort_pairs_noalloc(_addr(keys_in), _addr(vals_in), _addr(keys_out), _addr(vals_out), n,
                                        key_bits, _stream(stream)))


SORT_NOALLOC_MAX_PAIRS = 1 << 20

# The component of the area-light offset that each of the three light draws
# of a hit goes to (first, second, third draw): the order in which nvcc
# evaluates randVec3d's constructor arguments in the reference
# (kernels/mrand.cu:33-35), which the pixel kernels follow.
LIGHT_DRAW_ORDER = (0, 1, 2)


def camera_angle(fov):
    return math.tan(math.pi * 0.5 * fov / 180.0)

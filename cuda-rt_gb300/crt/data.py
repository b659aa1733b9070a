"""Seeded synthetic scenes for the parity tests and the benchmark.

Every mesh is generated in float64 with NumPy's PCG64 (``default_rng``),
moved into the reference's camera frame, and only then rounded to float32, so
that the CUDA path and the CPU oracle read identical bytes.

The reference's pixel kernel has a fixed camera: at the origin, looking down
-z, +y up (kernels/raytracer.cu:126-154).  A workload with a camera elsewhere
is expressed by applying the rigid world-to-camera transform to the geometry
and the light (``view_transform``); the renderer then sees exactly what a
camera at that pose would.

The positional light of the reference is offset by -0.5 on every axis when
its radius is 0 (kernels/Light.cu:71-80: ``offset = rand*radius; offset -=
0.5``).  ``light_for`` adds 0.5 so that the effective light sits at the
requested position.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "Mesh", "Camera", "Light", "Scene", "view_transform", "light_for", "soup", "icosphere",
    "config0", "config1", "config2_frame", "config3", "config4", "lambert_material", "load_obj", "Animation",
    "optics_scene",
]


@dataclass
class Mesh:
    verts: np.ndarray          # (V, 3) float32
    vidx: np.ndarray           # (N, 3) int32
    normals: np.ndarray        # (Nn, 3) float32
    nidx: np.ndarray           # (N, 3) int32
    matid: np.ndarray          # (N,) int32
    materials: np.ndarray      # (M, 16) float64: ka kd ks kt ke (3 each), shininess

    @property
    def ntri(self) -> int:
        return int(self.vidx.shape[0])


@dataclass
class Camera:
    """The Camera getters the reference's pixel kernel reads (inc/camera.h)."""
    fov: float = 60.0               # vertical, degrees (Camera::setfov)
    focal_point: float = 1.0        # Camera::setFocalPoint
    fstop: float = math.inf         # Camera::setFstop; aperture = 1/fstop, lens radius = aperture/2
    eye: tuple = (0.0, 0.0, 0.0)    # Camera() default; only the specular term reads it


@dataclass
class Light:
    """Light_h (inc/Light.h:7-29), positional."""
    position: tuple = (1.0, 1.0, 1.0)
    color: tuple = (1.0, 1.0, 1.0)
    radius: float = 0.0
    constant_term: float = 1.0
    linear_term: float = 0.0
    quadratic_term: float = 0.0


@dataclass
class Scene:
    mesh: Mesh
    camera: Camera
    light: Light
    width: int
    height: int
    spp: int
    name: str = ""
    extra: dict = field(default_factory=dict)


def lambert_material(kd=0.8) -> np.ndarray:
    """One Material row: Lambert albedo kd, no ambient/specular/emission/transmission."""
    m = np.zeros(16, np.float64)
    m[3:6] = kd
    return m


def view_transform(p: np.ndarray, cam_pos, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), direction=False):
    """World -> reference camera frame (camera at origin looking down -z).

    ``direction=True`` transforms direction vectors (rotation only)."""
    c = np.asarray(cam_pos, np.float64)
    f = np.asarray(target, np.float64) - c
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(up, np.float64))
    if np.linalg.norm(r) < 1e-12:  # looking along `up`
        r = np.cross(f, np.array([1.0, 0.0, 0.0]))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    R = np.stack([r, u, -f])  # rows: camera x, y, z axes
    q = np.asarray(p, np.float64)
    if not direction:
        q = q - c
    return q @ R.T


def light_for(world_pos, cam_pos, target=(0.0, 0.0, 0.0)) -> tuple:
    """Light position to pass so the reference's lit point is `world_pos`."""
    p = view_transform(np.asarray(world_pos, np.float64)[None], cam_pos, target)[0]
    return tuple(float(x) + 0.5 for x in p)


def _face_normals(v: np.ndarray, idx: np.ndarray) -> np.ndarray:
    a, b, c = v[idx[:, 0]], v[idx[:, 1]], v[idx[:, 2]]
    n = np.cross(b - a, c - a)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return n / ln


def soup(n: int, seed: int = 0, scale: float = 1.0, sigma: float = 0.01, cam_pos=(0.0, 0.0, -3.0),
         rng=None) -> Mesh:
    """Triangle soup: centroids ~ U[-1,1]^3, vertices = centroid + N(0, sigma^2)
    per axis, the whole mesh scaled by `scale`; face normals as per-vertex normals."""
    rng = rng if rng is not None else np.random.default_rng(seed)
    cent = rng.uniform(-1.0, 1.0, size=(n, 3))
    v = (cent[:, None, :] + rng.normal(0.0, sigma, size=(n, 3, 3))) * scale
    v = v.reshape(-1, 3)
    v = view_transform(v, cam_pos)
    vidx = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    v32 = v.astype(np.float32)
    fn = _face_normals(v32.astype(np.float64), vidx)
    normals = np.repeat(fn, 3, axis=0).astype(np.float32)
    return Mesh(v32, vidx, normals, vidx.copy(), np.zeros(n, np.int32), lambert_material()[None])


_ICO_V = None


def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return v, f


def _geodesic(nu: int):
    """Class-I geodesic sphere of frequency nu: 20*nu^2 faces, 10*nu^2+2 vertices
    (unit directions, shared vertices deduplicated exactly)."""
    cv, cf = _icosahedron()
    edges = {}
    for f in cf:
        for a, b in ((f[0], f[1]), (f[1], f[2]), (f[2], f[0])):
            key = (min(a, b), max(a, b))
            if key not in edges:
                edges[key] = len(edges)
    ne = len(edges)
    assert ne == 30
    n_int = (nu - 1) * (nu - 2) // 2
    nvert = 12 + ne * (nu - 1) + 20 * n_int
    pos = np.zeros((nvert, 3), np.float64)
    pos[:12] = cv
    k = np.arange(1, nu, dtype=np.float64) / nu
    for (a, b), e in edges.items():
        p = cv[a][None] + (cv[b] - cv[a])[None] * k[:, None]
        pos[12 + e * (nu - 1): 12 + (e + 1) * (nu - 1)] = p
    # grid (i, j), i + j <= nu, of every face
    ii, jj = np.meshgrid(np.arange(nu + 1), np.arange(nu + 1), indexing="ij")
    mask = ii + jj <= nu
    gi, gj = ii[mask], jj[mask]
    gid = -np.ones((nu + 1, nu + 1), np.int64)
    faces = []
    int_base = 12 + ne * (nu - 1)
    interior = (gi > 0) & (gj > 0) & (gi + gj < nu)
    li = np.cumsum(interior) - 1
    for fi, (A, B, C) in enumerate(cf):
        ids = np.empty(gi.shape, np.int64)

        def edge_pt(u, v, t):  # point t/nu from corner u towards corner v
            e = edges[(min(u, v), max(u, v))]
            tt = t if u < v else nu - t
            return 12 + e * (nu - 1) + (tt - 1)

        for m in range(gi.size):
            i, j = int(gi[m]), int(gj[m])
            if interior[m]:
                continue
            if i == 0 and j == 0:
                ids[m] = A
            elif i == nu:
                ids[m] = B
            elif j == nu:
                ids[m] = C
            elif j == 0:
                ids[m] = edge_pt(A, B, i)
            elif i == 0:
                ids[m] = edge_pt(A, C, j)
            else:  # i + j == nu
                ids[m] = edge_pt(B, C, j)
        ids[interior] = int_base + fi * n_int + li[interior]
        P = cv[A][None] + (cv[B] - cv[A])[None] * (gi[interior] / nu)[:, None] + \
            (cv[C] - cv[A])[None] * (gj[interior] / nu)[:, None]
        pos[ids[interior]] = P
        gid[gi, gj] = ids
        i, j = np.meshgrid(np.arange(nu), np.arange(nu), indexing="ij")
        up = (i + j) <= nu - 1
        tu = np.stack([gid[i[up], j[up]], gid[i[up] + 1, j[up]], gid[i[up], j[up] + 1]], 1)
        dn = (i + j) <= nu - 2
        td = np.stack([gid[i[dn] + 1, j[dn]], gid[i[dn] + 1, j[dn] + 1], gid[i[dn], j[dn] + 1]], 1)
        faces.append(tu)
        faces.append(td)
    tris = np.concatenate(faces).astype(np.int32)
    pos /= np.linalg.norm(pos, axis=1, keepdims=True)
    return pos, tris


def icosphere(nu: int, seed: int = 1, amp: float = 0.05, cam_pos=(0.0, 0.0, -3.0), frame: int | None = None,
              frames: int = 60, rng=None):
    """Geodesic icosphere (20*nu^2 faces) displaced radially by
    amp * sum_k sin(f_k * (u . a_k) + phi_k), k = 1..4, with f_k ~ U[1, 8],
    phi_k ~ U[0, 2pi) and random unit axes a_k; area-weighted vertex normals.

    ``frame`` animates it as in the refit workload:
    v += 0.02 * sin(2 pi frame/frames + 5 x0) * n0 (x0, n0 of the rest pose)."""
    rng = rng if rng is not None else np.random.default_rng(seed)
    u, tris = _geodesic(nu)
    f = rng.uniform(1.0, 8.0, 4)
    ph = rng.uniform(0.0, 2.0 * np.pi, 4)
    ax = rng.normal(size=(4, 3))
    ax /= np.linalg.norm(ax, axis=1, keepdims=True)
    r = 1.0 + amp * np.sin((u @ ax.T) * f[None] + ph[None]).sum(1)
    v = u * r[:, None]
    n = _vertex_normals(v, tris)
    if frame is not None:
        v = v + (0.02 * np.sin(2.0 * np.pi * frame / frames + 5.0 * v[:, 0]))[:, None] * n
    vc = view_transform(v, cam_pos)
    nc = view_transform(n, cam_pos, direction=True)
    return Mesh(vc.astype(np.float32), tris, nc.astype(np.float32), tris.copy(),
                np.zeros(tris.shape[0], np.int32), lambert_material()[None])


def _vertex_normals(v, tris):
    a, b, c = v[tris[:, 0]], v[tris[:, 1]], v[tris[:, 2]]
    fn = np.cross(b - a, c - a)  # area-weighted
    n = np.zeros_like(v)
    for k in range(3):
        np.add.at(n, tris[:, k], fn)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    return n


def config0(n=100_000, width=640, height=480, spp=1) -> Scene:
    """Plain method, small: 100k-triangle soup, pinhole camera at (0,0,-3)
    looking +z, 60 deg vertical fov, 640x480, 1 spp, light at (2,2,-2)."""
    cam_pos = (0.0, 0.0, -3.0)
    mesh = soup(n, seed=0, cam_pos=cam_pos)
    return Scene(mesh, Camera(fov=60.0, focal_point=1.0, fstop=math.inf),
                 Light(position=light_for((2.0, 2.0, -2.0), cam_pos)), width, height, spp, "config0")


def config1(nu=224, width=1920, height=1080, spp=16) -> Scene:
    """Plain method, large: nu=224 icosphere (1,003,520 faces), 1920x1080,
    16 spp, thin lens with aperture radius 0.05 (fstop 10) focused at 3.0,
    light at (3,3,-3)."""
    cam_pos = (0.0, 0.0, -3.0)
    mesh = icosphere(nu, seed=1, cam_pos=cam_pos)
    return Scene(mesh, Camera(fov=60.0, focal_point=3.0, fstop=1.0 / (2 * 0.05)),
                 Light(position=light_for((3.0, 3.0, -3.0), cam_pos)), width, height, spp, "config1")


class Animation:
    """The refit workload's animated mesh: the large configuration's icosphere
    with v_f = v_0 + 0.02 sin(2 pi f / frames + 5 x_0) n_0 (x_0, n_0 of the
    rest pose, world space).  Frames are produced from float64 rest data, so
    frame f always has the same float32 bytes."""

    def __init__(self, nu=224, frames=60, seed=1, cam_pos=(0.0, 0.0, -3.0)):
        rng = np.random.default_rng(seed)
        u, tris = _geodesic(nu)
        f = rng.uniform(1.0, 8.0, 4)
        ph = rng.uniform(0.0, 2.0 * np.pi, 4)
        ax = rng.normal(size=(4, 3))
        ax /= np.linalg.norm(ax, axis=1, keepdims=True)
        r = 1.0 + 0.05 * np.sin((u @ ax.T) * f[None] + ph[None]).sum(1)
        self.v0 = u * r[:, None]
        self.n0 = _vertex_normals(self.v0, tris)
        self.tris = tris
        self.frames = frames
        self.cam_pos = cam_pos
        nc = view_transform(self.n0, cam_pos, direction=True)
        # frame 0 (its topology is the one the refit path keeps)
        self.mesh0 = Mesh(self.vertices(0), tris, nc.astype(np.float32), tris.copy(),
                          np.zeros(tris.shape[0], np.int32), lambert_material()[None])

    def vertices(self, frame: int) -> np.ndarray:
        v = self.v0 + (0.02 * np.sin(2.0 * np.pi * frame / self.frames + 5.0 * self.v0[:, 0]))[:, None] * self.n0
        return view_transform(v, self.cam_pos).astype(np.float32)

    def scene(self, width=1280, height=720, spp=4) -> Scene:
        return Scene(self.mesh0, Camera(fov=60.0, focal_point=3.0, fstop=1.0 / (2 * 0.05)),
                     Light(position=light_for((3.0, 3.0, -3.0), self.cam_pos)), width, height, spp, "config2")


def config2_frame(frame: int, nu=224, width=1280, height=720, spp=4) -> Scene:
    """Refit vs rebuild: the config-1 mesh at animation frame `frame` of 60."""
    cam_pos = (0.0, 0.0, -3.0)
    mesh = icosphere(nu, seed=1, cam_pos=cam_pos, frame=frame, frames=60)
    return Scene(mesh, Camera(fov=60.0, focal_point=3.0, fstop=1.0 / (2 * 0.05)),
                 Light(position=light_for((3.0, 3.0, -3.0), cam_pos)), width, height, spp, f"config2_f{frame}")


def config3(count=256, lo=1_000, hi=500_000, width=256, height=256, spp=4, seed=2) -> list:
    """Batched form: `count` soups, triangle counts log-uniform in [lo, hi],
    cube scale ~ U[0.5, 4], each with a camera at a random point of the radius-4
    sphere looking at the origin, aperture radius 0.02 (fstop 25) focused at 4."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)
    scales = rng.uniform(0.5, 4.0, count)
    dirs = rng.normal(size=(count, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    scenes = []
    for m in range(count):
        cam_pos = tuple(4.0 * dirs[m])
        mesh = soup(int(sizes[m]), scale=float(scales[m]), cam_pos=cam_pos, rng=rng)
        light_world = tuple(np.asarray(cam_pos) * 0.5 + np.array([2.0, 2.0, 0.0]))
        scenes.append(Scene(mesh, Camera(fov=60.0, focal_point=4.0, fstop=1.0 / (2 * 0.02)),
                            Light(position=light_for(light_world, cam_pos)), width, height, spp, f"config3_m{m}"))
    return scenes


def config4(nu=100, width=512, height=512, spp=4, perturbed=False) -> Scene:
    """Differentiable form: nu=100 icosphere (200,000 faces), 512x512, 4 spp,
    pinhole, Lambert with a per-triangle albedo, light at (3,3,-3).  With
    `perturbed`, vertices get N(0, 0.005^2) noise (seed 3): the target image."""
    cam_pos = (0.0, 0.0, -3.0)
    mesh = icosphere(nu, seed=1, cam_pos=cam_pos)
    n = mesh.ntri
    mats = np.zeros((n, 16), np.float64)
    alb = np.random.default_rng(4).uniform(0.5, 0.9, (n, 3))
    mats[:, 3:6] = alb
    mesh.materials = mats
    mesh.matid = np.arange(n, dtype=np.int32)
    if perturbed:
        noise = np.random.default_rng(3).normal(0.0, 0.005, mesh.verts.shape)
        mesh.verts = (mesh.verts.astype(np.float64) + noise).astype(np.float32)
    return Scene(mesh, Camera(fov=60.0, focal_point=1.0, fstop=math.inf),
                 Light(position=light_for((3.0, 3.0, -3.0), cam_pos)), width, height, spp, "config4")


def load_obj(path: str) -> Mesh:
    """Minimal Wavefront OBJ/MTL reader with tinyobjloader's conventions as the
    reference calls it (src/scene.cpp:6-58): polygons fan-triangulated, per-face
    material ids, Ka/Kd/Ks/Kt(Tf)/Ke/Ns from the MTL file next to the OBJ
    (colours default to 0, shininess to 1).  The C ABI's crt_obj_load reads the
    same files to the same arrays."""
    import os
    verts, normals, vidx, nidx, matid = [], [], [], [], []
    mat_names, mats = {}, []
    cur = -1
    base = os.path.dirname(path)

    def read_mtl(fn):
        m = None
        if not os.path.exists(os.path.join(base, fn)):  # tinyobjloader warns and goes on
            return
        with open(os.path.join(base, fn)) as f:
            for line in f:
                t = line.split()
                if not t:
                    continue
                if t[0] == "newmtl":
                    m = np.zeros(16, np.float64)
                    m[15] = 1.0  # tinyobjloader's default shininess
                    mat_names[t[1]] = len(mats)
                    mats.append(m)
                elif m is not None:
                    key = {"Ka": 0, "Kd": 3, "Ks": 6, "Kt": 9, "Tf": 9, "Ke": 12}.get(t[0])
                    if key is not None:
                        m[key:key + 3] = [float(x) for x in t[1:4]]
                    elif t[0] == "Ns":
                        m[15] = float(t[1])

    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                verts.append([float(x) for x in t[1:4]])
            elif t[0] == "vn":
                normals.append([float(x) for x in t[1:4]])
            elif t[0] == "mtllib":
                read_mtl(t[1])
            elif t[0] == "usemtl":
                cur = mat_names.get(t[1], -1)
            elif t[0] == "f":
                corners = []
                for c in t[1:]:
                    parts = c.split("/")
                    vi = int(parts[0])
                    vi = vi - 1 if vi > 0 else len(verts) + vi
                    ni = -1
                    if len(parts) >= 3 and parts[2]:
                        ni = int(parts[2])
                        ni = ni - 1 if ni > 0 else len(normals) + ni
                    corners.append((vi, ni))
                for k in range(1, len(corners) - 1):
                    tri = (corners[0], corners[k], corners[k + 1])
                    vidx.append([c[0] for c in tri])
                    nidx.append([c[1] for c in tri])
                    matid.append(cur)
    if not mats:
        mats.append(lambert_material())
    matid = np.array(matid, np.int32)
    matid[matid < 0] = 0
    return Mesh(np.array(verts, np.float32).reshape(-1, 3), np.array(vidx, np.int32).reshape(-1, 3),
                np.array(normals, np.float32).reshape(-1, 3), np.array(nidx, np.int32).reshape(-1, 3),
                matid, np.array(mats, np.float64).reshape(-1, 16))


def _quad(p0, du, dv):
    p0, du, dv = (np.asarray(x, np.float64) for x in (p0, du, dv))
    v = np.stack([p0, p0 + du, p0 + du + dv, p0 + dv])
    n = np.cross(du, dv)
    n /= np.linalg.norm(n)
    return v, np.array([[0, 1, 2], [0, 2, 3]]), np.repeat(n[None], 4, 0)


def _sphere(center, radius, nu):
    u, tris = _geodesic(nu)
    return np.asarray(center) + radius * u, np.asarray(tris), u


def optics_scene(emissive=False, nu=6, specular=False):
    """A floor, a mirror wall behind a glass sphere (20*nu^2 faces) and a
    smaller diffuse sphere, seen from (0, 0, -3): the reflection/refraction
    workload.  Materials: 0 floor, 1 mirror, 2 glass (ior 1.5), 3 diffuse.
    Returns (mesh, optics (4, 4): kr xyz + ior per material).  emissive:
    only ke is set (shade() = ke whatever the light).  specular=False leaves
    ks = 0 (the Phong term's powf is the one operation whose result may
    differ between CUDA and the host's libm in the last bit)."""
    parts = [(_quad((-2, -0.8, -2), (0, 0, 4), (4, 0, 0)), 0),
             (_quad((-1.5, -0.8, 1.5), (0, 2.3, 0), (3, 0, 0)), 1),
             (_sphere((0.3, 0.0, 0.0), 0.5, nu), 2),
             (_sphere((-0.7, -0.45, 0.4), 0.35, max(nu // 2, 1)), 3)]
    V, T, Nv, mid = [], [], [], []
    off = 0
    for (v, t, n), m in parts:
        V.append(v)
        Nv.append(n)
        T.append(t + off)
        mid.append(np.full(len(t), m, np.int32))
        off += len(v)
    cam = (0.0, 0.0, -3.0)
    v = view_transform(np.concatenate(V), cam).astype(np.float32)
    n = view_transform(np.concatenate(Nv), cam, direction=True).astype(np.float32)
    tris = np.concatenate(T).astype(np.int32)
    mats = np.zeros((4, 16))
    ka, kd, ks, kt, ke, sh = slice(0, 3), slice(3, 6), slice(6, 9), slice(9, 12), slice(12, 15), 15
    if emissive:
        mats[0, ke] = (0.3, 0.5, 0.2)
        mats[1, ke] = (0.05, 0.05, 0.1)
        mats[2, ke] = (0.02, 0.01, 0.0)
        mats[3, ke] = (0.7, 0.2, 0.1)
    else:
        mats[0, kd] = (0.8, 0.7, 0.6)
        mats[1, kd] = 0.1
        mats[2, kd] = 0.05
        mats[3, kd] = (0.2, 0.4, 0.9)
        if specular:
            mats[1, ks] = 0.8
            mats[2, ks] = 0.1
            mats[3, ks] = 0.3
    mats[:, sh] = 1.0
    mats[1, sh] = 20.0
    mats[2, kt] = (0.9, 0.9, 0.85)
    optics = np.array([[0, 0, 0, 1.0], [0.8, 0.8, 0.8, 1.0], [0.1, 0.1, 0.1, 1.5], [0, 0, 0, 1.0]])
    mesh = Mesh(v, tris, n, tris.copy(), np.concatenate(mid), mats)
    return mesh, optics

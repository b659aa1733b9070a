"""Generate the golden fixtures in this directory from the reference itself.

The reference (mbartling/cuda-rt) ships no tests and no golden vectors.  Its
hot-path device code, compiled for the host by oracle/ref/build_ref.py
(oracle/_ref/libcrtref.so), is run here on:
  * the reference's own small test scenes (objs/testyz, objs/tests), read
    with tinyobjloader's conventions (crt.data.load_obj), and
  * seeded synthetic scenes (a triangle soup, an icosphere, degenerate sets).
Each fixture stores the inputs and the reference's outputs: scene box,
Morton codes before and after the sort, sorted ids, the radix tree
(parent/left/right) and its boxes, closest-hit and any-hit results for a
seeded ray set (including axis-parallel rays and rays starting on box
planes), and a 32x32 rendered image at the reference's fixed 20 samples per
pixel.  The GPU machine has no reference checkout; these files travel instead.

Run (in a container with the reference checkout):
    python oracle/ref/build_ref.py && python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cuda-rt_gb300"))

from crt import data  # noqa: E402
from oracle.oracle import OracleScene, ref_available  # noqa: E402

from oracle.ref.build_ref import default_reference  # noqa: E402

REF = default_reference()

OBJ_FIXTURES = ["testyz/bvh_simple1", "testyz/bvh_simple2", "testyz/bvh_simple3", "testyz/bvh_simple4",
                "testyz/bvh_simple5", "testyz/bvh_simple6", "testyz/oneplane", "testyz/oneplane2",
                "testyz/oneplane3", "testyz/sanity1", "testyz/distance1", "testyz/distance2",
                "testyz/occlusion1", "tests/orientation"]


def ray_set(mesh, seed, n_rand=192):
    """Seeded rays aimed at a mesh: random, axis-parallel, and from vertex planes."""
    rng = np.random.default_rng(seed)
    v = mesh.verts.astype(np.float64)
    lo, hi = v.min(0), v.max(0)
    c, ext = 0.5 * (lo + hi), np.maximum(hi - lo, 1e-3)
    rays = []
    o = c + (rng.uniform(-1, 1, (n_rand, 3)) * ext)
    tgt = c + (rng.uniform(-0.5, 0.5, (n_rand, 3)) * ext)
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays.append(np.hstack([o, d]))
    # from the reference camera position (origin) toward points of the mesh
    tgt = v[rng.integers(0, len(v), 48)] + rng.normal(0, 1e-3, (48, 3))
    d = tgt / np.linalg.norm(tgt, axis=1, keepdims=True)
    rays.append(np.hstack([np.zeros((48, 3)), d]))
    # axis-parallel rays (1/d = +-inf on two axes)
    for ax in range(3):
        for sgn in (1.0, -1.0):
            o = c + rng.uniform(-0.6, 0.6, (8, 3)) * ext
            o[:, ax] = c[ax] - sgn * 2 * ext[ax]
            d = np.zeros((8, 3))
            d[:, ax] = sgn
            rays.append(np.hstack([o, d]))
    # origins exactly on vertex planes, axis-parallel directions: (b - e) * inf = NaN slabs
    idx = rng.integers(0, len(v), 16)
    for i, vi in enumerate(idx):
        ax = i % 3
        o = c + rng.uniform(-0.3, 0.3, 3) * ext
        o[(ax + 1) % 3] = v[vi, (ax + 1) % 3]
        d = np.zeros(3)
        d[ax] = 1.0 if i % 2 else -1.0
        o[ax] = c[ax] - d[ax] * 2 * ext[ax]
        rays.append(np.hstack([o, d])[None])
    return np.vstack(rays)


def fixture(name, mesh, camera, light, seed, out_dir):
    ref = OracleScene(mesh, "ref")
    ex = ref.export()
    rays = ray_set(mesh, seed)
    ci, ct, cn = ref.trace(rays, any_hit=False)
    ai, at, _ = ref.trace(rays, any_hit=True)
    img = ref.render(camera, light, 32, 32)
    np.savez_compressed(
        os.path.join(out_dir, name + ".npz"),
        verts=mesh.verts, vidx=mesh.vidx, normals=mesh.normals, nidx=mesh.nidx, matid=mesh.matid,
        materials=mesh.materials,
        camera=np.array([camera.fov, camera.focal_point, camera.fstop, *camera.eye]),
        light=np.array([*light.position, *light.color, light.radius, light.constant_term, light.linear_term,
                        light.quadratic_term]),
        smin=ex["smin"], smax=ex["smax"], codes_unsorted=ex["codes_unsorted"], codes=ex["codes"], ids=ex["ids"],
        nodes=ex["nodes"], node_boxes=ex["node_boxes"], tri_boxes=ex["tri_boxes"],
        rays=rays, closest_id=ci, closest_t=ct, closest_n=cn, any_id=ai, any_t=at,
        rgb8=img["rgb"], color=img["color"])
    print(f"{name}: {mesh.ntri} triangles, {len(rays)} rays, {(ci >= 0).mean():.2f} hit")


def main():
    if not ref_available():
        sys.exit("oracle/_ref/libcrtref.so missing: run python oracle/ref/build_ref.py")
    out_dir = HERE
    for i, rel in enumerate(OBJ_FIXTURES):
        mesh = data.load_obj(os.path.join(REF, "objs", rel + ".obj"))
        cam = data.Camera(fov=35.0, focal_point=10.0, fstop=8.0 if i % 2 else math.inf)
        light = data.Light(position=(1.0, 1.0, 1.0), constant_term=1.0)
        fixture("obj_" + rel.replace("/", "_"), mesh, cam, light, 100 + i, out_dir)
    # synthetic scenes in the benchmark's conventions
    s0 = data.config0(n=3000, width=32, height=32)
    fixture("soup3000", s0.mesh, s0.camera, s0.light, 7, out_dir)
    s1 = data.config1(nu=10)  # 2000 faces
    fixture("icosphere_nu10_dof", s1.mesh, s1.camera, s1.light, 8, out_dir)
    # degenerate sets: every centroid equal (all codes equal: the index
    # tie-break of delta()), a planar set (0/0 in the Morton normalisation)
    rng = np.random.default_rng(9)
    n = 300
    base = rng.normal(0, 0.01, (n, 3, 3))
    base -= base.mean(1, keepdims=True)
    v = (base + np.array([0.0, 0.0, -3.0])).reshape(-1, 3).astype(np.float32)
    vidx = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    nrm = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (3 * n, 1))
    m = data.Mesh(v, vidx, nrm, vidx.copy(), np.zeros(n, np.int32), data.lambert_material()[None])
    fixture("same_centroid300", m, data.Camera(fov=60.0), data.Light(position=(1.5, 2.5, -0.5)), 10, out_dir)
    xy = rng.uniform(-1, 1, (n, 3, 2))
    v = np.concatenate([xy, np.full((n, 3, 1), -3.0)], 2).reshape(-1, 3).astype(np.float32)
    m = data.Mesh(v, vidx, nrm, vidx.copy(), np.zeros(n, np.int32), data.lambert_material()[None])
    fixture("planar300", m, data.Camera(fov=60.0), data.Light(position=(1.5, 2.5, -0.5)), 11, out_dir)


if __name__ == "__main__":
    main()

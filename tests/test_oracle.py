"""The CPU oracle against the reference's own outputs.

* golden fixtures (tests/golden, generated by the reference's device code
  compiled for the host, see tests/golden/make_golden.py): every build
  product, closest/any-hit traces and the 20-spp image must match exactly;
* live comparison with oracle/_ref (only where the reference checkout was
  available to build it) on fresh seeded scenes.
"""
import math
import os

import numpy as np
import pytest

from conftest import assert_equal, golden_camera_light, golden_files, golden_mesh

from crt import data
from oracle.oracle import OracleScene, ref_available


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_reference_golden(path):
    z = np.load(path)
    mesh = golden_mesh(z)
    o = OracleScene(mesh)
    ex = o.export()
    for k in ("smin", "smax", "codes_unsorted", "codes", "ids", "nodes", "node_boxes", "tri_boxes"):
        assert_equal(ex[k], z[k], k)
    ci, ct, cn = o.trace(z["rays"], any_hit=False)
    assert_equal(ci, z["closest_id"], "closest id")
    assert_equal(ct, z["closest_t"], "closest t")
    hit = ci >= 0
    assert_equal(cn[hit], z["closest_n"][hit], "closest normal")
    ai, at, _ = o.trace(z["rays"], any_hit=True)
    assert_equal(ai, z["any_id"], "any id")
    assert_equal(at, z["any_t"], "any t")
    cam, light = golden_camera_light(z)
    img = o.render(cam, light, 32, 32, spp=20)
    assert_equal(img["color"], z["color"], "pixel colour")
    assert_equal(img["rgb"], z["rgb8"], "rgb8")


needs_ref = pytest.mark.skipif(not ref_available(), reason="oracle/_ref not built (no reference checkout)")


def _same_build(mesh):
    a, b = OracleScene(mesh).export(), OracleScene(mesh, "ref").export()
    for k in a:
        assert_equal(a[k], b[k], k)


@needs_ref
@pytest.mark.parametrize("n", [1, 2, 3, 5, 64, 777, 20000])
def test_build_matches_reference_soup(n):
    _same_build(data.soup(n, seed=n))


@needs_ref
def test_build_matches_reference_duplicates_and_planar():
    rng = np.random.default_rng(5)
    n = 500
    # many duplicated centroids on a coarse grid: long runs of equal codes
    cent = rng.integers(0, 4, (n, 3)).astype(np.float64) / 3.0
    off = rng.normal(0, 0.001, (n, 3, 3))
    off -= off.mean(1, keepdims=True)
    v = (cent[:, None, :] + off).reshape(-1, 3).astype(np.float32)
    vidx = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    nrm = np.tile(np.array([[0, 0, 1]], np.float32), (3 * n, 1))
    _same_build(data.Mesh(v, vidx, nrm, vidx.copy(), np.zeros(n, np.int32), data.lambert_material()[None]))
    # planar in z
    v2 = v.copy()
    v2[:, 2] = -2.0
    _same_build(data.Mesh(v2, vidx, nrm, vidx.copy(), np.zeros(n, np.int32), data.lambert_material()[None]))


@needs_ref
def test_render_matches_reference_dof_icosphere():
    sc = data.config1(nu=12)
    a, b = OracleScene(sc.mesh), OracleScene(sc.mesh, "ref")
    ra = a.render(sc.camera, sc.light, 48, 32, spp=20)
    rb = b.render(sc.camera, sc.light, 48, 32)
    assert_equal(ra["color"], rb["color"], "colour")
    assert_equal(ra["rgb"], rb["rgb"], "rgb8")


@needs_ref
def test_render_rows_band_matches_reference():
    sc = data.config0(n=4000, width=64, height=48)
    a, b = OracleScene(sc.mesh), OracleScene(sc.mesh, "ref")
    ra = a.render(sc.camera, sc.light, 64, 48, spp=20, rows=(16, 32))
    rb = b.render(sc.camera, sc.light, 64, 48, rows=(16, 32))
    assert_equal(ra["rgb"], rb["rgb"], "rgb8")


@needs_ref
def test_trace_matches_reference_random_rays():
    sc = data.config0(n=5000)
    a, b = OracleScene(sc.mesh), OracleScene(sc.mesh, "ref")
    rng = np.random.default_rng(0)
    o = rng.uniform(-2, 2, (3000, 3)) + np.array([0, 0, -3.0])
    d = rng.normal(size=(3000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.hstack([o, d])
    for anyh in (False, True):
        ia, ta, na = a.trace(rays, any_hit=anyh)
        ib, tb, nb = b.trace(rays, any_hit=anyh)
        assert_equal(ia, ib, "ids")
        assert_equal(ta, tb, "t")


def test_oracle_light_offset_convention():
    """light_for() compensates the reference's -0.5 light offset (Light.cu:73-74)."""
    p = data.light_for((2.0, 2.0, -2.0), (0.0, 0.0, -3.0))
    assert p == (-1.5, 2.5, -0.5)
    assert math.isclose(data.view_transform(np.array([[0.0, 0.0, 0.0]]), (0, 0, -3))[0, 2], -3.0)


@pytest.mark.skipif(not ref_available(), reason="oracle/_ref not built (no reference checkout here)")
def test_area_light_draw_order_of_the_host_compiled_reference():
    """randVec3d's three draws (kernels/mrand.cu:33-35) are constructor
    arguments, whose evaluation order C++ leaves to the compiler.  The
    reference compiled for the host takes them in the order of the host's
    g++: right to left on x86-64 (the first draw lands in z), left to right
    on AArch64 (as nvcc's device code, checked by
    tests/test_gpu_draw_order.py).  With an area light its image equals the
    oracle's with that order and differs from every other order."""
    import itertools
    sc = data.config0(n=3000, width=48, height=32)
    light = data.Light(position=sc.light.position, radius=0.7)
    ref = OracleScene(sc.mesh, "ref").render(sc.camera, light, 48, 32)
    o = OracleScene(sc.mesh)
    try:
        same = []
        for perm in itertools.permutations(range(3)):
            assert o.lib.orc_set_light_draw_order(*perm) == 0
            out = o.render(sc.camera, light, 48, 32, spp=20)
            if np.array_equal(out["color"], ref["color"]):
                same.append(perm)
    finally:
        import crt
        o.lib.orc_set_light_draw_order(*crt.LIGHT_DRAW_ORDER)
    import platform
    host_order = {"x86_64": (2, 1, 0), "aarch64": (0, 1, 2)}.get(platform.machine())
    assert len(same) == 1, same
    if host_order is not None:
        assert same == [host_order], same
    assert o.lib.orc_set_light_draw_order(0, 0, 1) == -1

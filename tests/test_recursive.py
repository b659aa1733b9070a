"""The oracle's recursive traceRay (reflected and refracted rays, the block of
kernels/raytracer.cu:196-237 that the reference leaves commented out), on the
CPU.  The reference never runs that block, so these tests pin the restatement
in two other ways: with depth 0, or with materials that neither reflect nor
transmit, it must equal the plain render (which is pinned to the reference);
and with emissive-only materials (shade() = ke whatever the light draws) its
colours must equal a recursion written here in Python over the oracle's
closest-hit primitive."""
import math

import numpy as np
import pytest


def optics_scene(emissive=False, nu=6, specular=False):
    from crt import data
    return data.optics_scene(emissive=emissive, nu=nu, specular=specular)


def scene_view(aperture=0.0, radius=0.0):
    from crt import data
    cam = data.Camera(fov=50.0, focal_point=3.0, fstop=math.inf if aperture == 0 else 1.0 / (2 * aperture))
    light = data.Light(position=data.light_for((2.0, 2.5, -2.0), (0.0, 0.0, -3.0)), radius=radius,
                       constant_term=1.0, linear_term=0.02, quadratic_term=0.01)
    return cam, light


@pytest.mark.parametrize("depth", [0, 3])
def test_no_reflection_or_transmission_equals_plain_render(depth):
    from oracle.oracle import OracleScene
    mesh, optics = optics_scene(specular=True)
    cam, light = scene_view(aperture=0.05, radius=0.3)
    o = OracleScene(mesh)
    plain = o.render(cam, light, 24, 16, spp=3, aux=True)
    if depth:
        optics = optics.copy()
        optics[:, :3] = 0.0
        mesh.materials[:, 9:12] = 0.0
        o = OracleScene(mesh)
        plain = o.render(cam, light, 24, 16, spp=3, aux=True)
    rec = o.render_recursive(cam, light, 24, 16, 3, depth, optics)
    assert np.array_equal(rec["color"], plain["color"])
    assert np.array_equal(rec["rgb"], plain["rgb"])
    assert np.array_equal(rec["hit_id"], plain["hit_id"])


def _normalize(a):
    s = 1.0 / float(np.sqrt(np.float32(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])))
    return [a[0] * s, a[1] * s, a[2] * s]


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _py_trace(o, mesh, optics, org, d, depth, counts):
    ids, t, nrm = o.trace(np.array([*org, *d])[None])
    counts[0] += 1
    if ids[0] < 0:
        return [0.9, 0.9, 0.9]
    m = int(mesh.matid[ids[0]])
    ke = mesh.materials[m, 12:15]
    c = [float(ke[0]) + 0.0, float(ke[1]) + 0.0, float(ke[2]) + 0.0]
    if depth <= 0:
        return c
    t = float(t[0])
    N = [float(x) for x in nrm[0]]
    q = [org[k] + t * d[k] for k in range(3)]
    kr = optics[m, :3]
    if kr.any():
        k2 = -2.0 * _dot(d, N)
        R = _normalize([k2 * N[k] + d[k] for k in range(3)])
        v = _py_trace(o, mesh, optics, q, R, depth - 1, counts)
        c = [c[k] + float(kr[k]) * v[k] for k in range(3)]
    kt = mesh.materials[m, 9:12]
    if kt.any():
        n = list(N)
        cr = _dot([-d[0], -d[1], -d[2]], n)
        rsin = [n[k] * cr + d[k] for k in range(3)]
        if _dot(d, n) < 0:
            eta = 1.0 / float(optics[m, 3])
            n = [-x for x in n]
        else:
            eta = float(optics[m, 3]) / 1.0
        tsin = [eta * x for x in rsin]
        tir = 1 - _dot(tsin, tsin)
        if tir >= 0:
            st = math.sqrt(tir)
            T = _normalize([n[k] * st + tsin[k] for k in range(3)])
            v = _py_trace(o, mesh, optics, q, T, depth - 1, counts)
            c = [c[k] + float(kt[k]) * v[k] for k in range(3)]
    return c


def test_recursion_matches_python_restatement_emissive():
    """Emissive-only materials make every shade() equal ke, so a pixel's
    colour is a pure function of the ray tree: checked against a recursion
    over the oracle's closest hit, pixel by pixel (pinhole, 1 sample)."""
    from oracle.oracle import OracleScene
    mesh, optics = optics_scene(emissive=True)
    cam, light = scene_view()
    W, H = 20, 14
    o = OracleScene(mesh)
    rec = o.render_recursive(cam, light, W, H, 1, 4, optics, rays_out=True)
    counts = [0]
    want = np.array([_py_trace(o, mesh, optics, list(r[:3]), list(r[3:]), 4, counts) for r in rec["rays"]])
    assert counts[0] > 2 * W * H  # the tree goes below the primary rays
    np.testing.assert_array_equal(rec["color"], want)


def test_depth_changes_the_image():
    """More depth adds the contributions of deeper rays: depth 1 differs from
    depth 0 on the mirror and the glass, deeper levels still change some
    pixels, and on average far less (kr, kt < 1 damp each level)."""
    from oracle.oracle import OracleScene
    mesh, optics = optics_scene()
    cam, light = scene_view()
    o = OracleScene(mesh)
    c = [o.render_recursive(cam, light, 24, 16, 1, d, optics)["color"] for d in (0, 1, 5, 6)]
    d01 = np.abs(c[1] - c[0])
    d56 = np.abs(c[3] - c[2])
    assert d01.max() > 0.05 and d56.max() > 0
    assert d56.mean() < 0.1 * d01.mean()


def test_default_optics_take_ks_as_kr_and_unit_ior():
    from oracle.oracle import OracleScene
    mesh, optics = optics_scene(specular=True)
    cam, light = scene_view()
    o = OracleScene(mesh)
    dflt = np.concatenate([mesh.materials[:, 6:9], np.ones((4, 1))], 1)
    a = o.render_recursive(cam, light, 16, 12, 2, 2, None)
    b = o.render_recursive(cam, light, 16, 12, 2, 2, dflt)
    assert np.array_equal(a["color"], b["color"])

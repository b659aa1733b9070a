"""Synthetic workload generators (no GPU)."""
import numpy as np

from crt import data


def test_icosphere_counts_and_closed():
    for nu in (1, 2, 5, 10):
        u, tris = data._geodesic(nu)
        assert tris.shape == (20 * nu * nu, 3)
        assert u.shape == (10 * nu * nu + 2, 3)
        e = np.sort(np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]]), axis=1)
        _, cnt = np.unique(e, axis=0, return_counts=True)
        assert (cnt == 2).all(), "every edge shared by exactly two faces"
        # outward orientation: face normals point away from the centre
        a, b, c = u[tris[:, 0]], u[tris[:, 1]], u[tris[:, 2]]
        assert (np.einsum("ij,ij->i", np.cross(b - a, c - a), a + b + c) > 0).all()


def test_config_sizes():
    assert data.icosphere(224).ntri == 1_003_520
    assert data.config4().mesh.ntri == 200_000
    s0 = data.config0()
    assert s0.mesh.ntri == 100_000 and s0.mesh.verts.dtype == np.float32
    assert (s0.width, s0.height, s0.spp) == (640, 480, 1)


def test_config0_is_deterministic():
    a, b = data.config0(n=1000), data.config0(n=1000)
    assert np.array_equal(a.mesh.verts, b.mesh.verts)


def test_view_transform_camera_frame():
    # camera at (0,0,-3) looking at the origin: the origin lands 3 units down -z
    p = data.view_transform(np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]]), (0.0, 0.0, -3.0))
    assert np.allclose(p[0], [0, 0, -3])
    assert np.allclose(p[1], [-1, 0, -3])  # world +x is camera -x when looking down +z


def test_config3_sizes_log_uniform():
    s = data.config3(count=8, lo=1000, hi=5000)
    n = [x.mesh.ntri for x in s]
    assert all(1000 <= k <= 5000 for k in n)

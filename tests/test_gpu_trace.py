"""Closest-hit and any-hit traversal on the GPU: hit ids, t and normals bit-exact
against the reference (golden) and the oracle."""
import os

import numpy as np
import pytest

from conftest import assert_equal, golden_files, golden_mesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: os.path.basename(p)[:-4])
def test_trace_matches_reference_golden(cuda, path):
    import crt
    z = np.load(path)
    s = crt.Scene(golden_mesh(z))
    ids, t, nrm = s.trace(z["rays"], normals=True)
    assert_equal(ids, z["closest_id"], "closest id")
    assert_equal(t, z["closest_t"], "closest t")
    hit = ids >= 0
    assert_equal(nrm[hit], z["closest_n"][hit], "normal")
    ai, at = s.trace(z["rays"], any_hit=True)
    assert_equal(ai, z["any_id"], "any id")
    assert_equal(at, z["any_t"], "any t")


def _random_rays(rng, n, centre, spread):
    o = centre + rng.uniform(-spread, spread, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # a share of axis-parallel directions (infinite 1/d components)
    k = n // 10
    d[:k] = 0.0
    d[np.arange(k), rng.integers(0, 3, k)] = rng.choice([-1.0, 1.0], k)
    return np.hstack([o, d])


@pytest.mark.parametrize("scene", ["soup", "icosphere"])
def test_trace_matches_oracle(cuda, scene):
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    m = data.soup(100_000, seed=0) if scene == "soup" else data.icosphere(64)
    g, o = crt.Scene(m), OracleScene(m)
    rng = np.random.default_rng(42)
    rays = _random_rays(rng, 20_000, np.array([0, 0, -3.0]), 1.5)
    for anyh in (False, True):
        gi, gt = g.trace(rays, any_hit=anyh)
        oi, ot, _ = o.trace(rays, any_hit=anyh)
        assert_equal(gi, oi, f"ids any={anyh}")
        assert_equal(gt, ot, f"t any={anyh}")
    g.check()


def test_trace_device_buffers(cuda):
    """Device-resident rays and outputs (torch tensors) give the same answers."""
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    torch = cuda
    m = data.soup(20_000, seed=1)
    g, o = crt.Scene(m), OracleScene(m)
    rays = _random_rays(np.random.default_rng(3), 5000, np.array([0, 0, -3.0]), 1.0)
    ids, t = g.trace(torch.from_numpy(rays).cuda())
    oi, ot, _ = o.trace(rays)
    assert_equal(ids.cpu().numpy(), oi, "ids")
    assert_equal(t.cpu().numpy(), ot, "t")


def test_empty_and_single_triangle(cuda):
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    m1 = data.soup(1, seed=4)
    g, o = crt.Scene(m1), OracleScene(m1)
    c = m1.verts.astype(np.float64).mean(0)
    rng = np.random.default_rng(0)
    o_ = c + np.array([0, 0, 1.0]) + rng.normal(0, 0.01, (500, 3))
    d = c - o_
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.hstack([o_, d])
    gi, gt = g.trace(rays)
    oi, ot, _ = o.trace(rays)
    assert_equal(gi, oi, "ids")
    assert (gi >= 0).any()
    # an empty scene: every ray misses
    m0 = data.Mesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32), np.zeros((1, 3), np.float32),
                   np.zeros((0, 3), np.int32), np.zeros(0, np.int32), data.lambert_material()[None])
    e = crt.Scene(m0)
    ei, _ = e.trace(rays)
    assert (ei == -1).all()


def test_bad_input_reports_status(cuda):
    import crt
    from crt import data
    m = data.soup(10, seed=0)
    bad = data.Mesh(m.verts, m.vidx.copy(), m.normals, m.nidx, m.matid, m.materials)
    bad.vidx[3, 1] = 10_000
    with pytest.raises(crt.CrtError) as e:
        crt.Scene(bad)
    assert e.value.status == 1
    nan = data.Mesh(m.verts.copy(), m.vidx, m.normals, m.nidx, m.matid, m.materials)
    nan.verts[5, 0] = np.nan
    with pytest.raises(crt.CrtError) as e:
        crt.Scene(nan)
    assert e.value.status == 1

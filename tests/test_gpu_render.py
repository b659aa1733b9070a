"""The pixel kernel on the GPU against the reference and the oracle.

Pinhole cameras: every double operation is IEEE-exact on both sides, so the
GPU image, per-sample hit ids and shadow bits equal the oracle's (and the
reference's) bit for bit.  Thin-lens cameras: the lens sample uses double
cos/sin, whose last bit may differ between CUDA and the host libm; the GPU's
primary rays are therefore compared with the oracle's within 4 ulp, and then
fed to the oracle, after which every hit id, shadow bit and pixel must match
exactly.
"""
import math
import os

import numpy as np
import pytest

from conftest import assert_equal, golden_camera_light, golden_files, golden_mesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: os.path.basename(p)[:-4])
def test_render_matches_reference_golden(cuda, path):
    import crt
    from oracle.oracle import OracleScene
    z = np.load(path)
    mesh = golden_mesh(z)
    cam, light = golden_camera_light(z)
    s = crt.Scene(mesh)
    out = s.render(cam, light, 32, 32, 20, rays=True, aux=True, rgbf=True)
    if math.isinf(cam.fstop):
        assert_equal(out["rgb8"], z["rgb8"], "rgb8 (pinhole)")
    else:
        # DOF: the reference image through the reference's host libm may
        # differ where a sample's lens position changed in the last bit
        diff = np.abs(out["rgb8"].astype(int) - z["rgb8"].astype(int))
        assert diff.max() <= 1 or (diff > 0).mean() < 0.01, f"max {diff.max()}"
    # and exactly with the oracle replaying the GPU's primary rays
    o = OracleScene(mesh).render(cam, light, 32, 32, spp=20, rays_in=out["rays"], aux=True)
    assert_equal(out["hit_id"], o["hit_id"], "hit id")
    assert_equal(out["shadow"], o["shadow"], "shadow")
    assert_equal(out["rgb8"], o["rgb"], "rgb8")


def _ulp_close(a, b, ulps=4):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    tol = ulps * np.spacing(np.maximum(np.abs(a), np.abs(b)))
    return np.abs(a - b) <= np.maximum(tol, 1e-300)


def test_config0_full_size_bit_exact(cuda):
    """The small plain configuration at its full size: 100k-triangle soup,
    640x480, 1 spp, pinhole; every output bit-exact against the oracle."""
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    sc = data.config0()
    g = crt.Scene(sc.mesh)
    out = g.render(sc.camera, sc.light, sc.width, sc.height, sc.spp, aux=True, rgbf=True)
    o = OracleScene(sc.mesh).render(sc.camera, sc.light, sc.width, sc.height, spp=sc.spp, aux=True)
    assert_equal(out["hit_id"], o["hit_id"], "hit id")
    assert np.array_equal(out["hit_t"], o["hit_t"]), "hit t"
    assert_equal(out["shadow"], o["shadow"], "shadow")
    assert_equal(out["rgb8"], o["rgb"], "rgb8")
    assert (out["hit_id"] >= 0).mean() > 0.05
    g.check()


def test_config1_dof_reduced_image(cuda):
    """The large configuration's mesh (1,003,520 faces) and lens (aperture
    radius 0.05, focus 3, 16 spp) on a 192x108 image."""
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    sc = data.config1()
    W, H, spp = 192, 108, 16
    g = crt.Scene(sc.mesh)
    out = g.render(sc.camera, sc.light, W, H, spp, aux=True, rays=True)
    o = OracleScene(sc.mesh)
    own = o.render(sc.camera, sc.light, W, H, spp=spp, rays_out=True, aux=True)
    # a last-bit difference in cos/sin can flip the float rounding inside the
    # reference's normalize() (sqrtf of the float-rounded squared length), so
    # a few rays move by up to ~1 float ulp; nearly all agree to 4 double ulp
    close = _ulp_close(out["rays"], own["rays"]).all(1)
    assert close.mean() > 0.99, f"{(~close).sum()} rays beyond 4 ulp"
    assert np.allclose(out["rays"], own["rays"], rtol=2.0 ** -21, atol=1e-15)
    rep = o.render(sc.camera, sc.light, W, H, spp=spp, rays_in=out["rays"], aux=True)
    assert_equal(out["hit_id"], rep["hit_id"], "hit id")
    assert_equal(out["hit_t"], rep["hit_t"], "hit t")
    assert_equal(out["shadow"], rep["shadow"], "shadow")
    assert_equal(out["rgb8"], rep["rgb"], "rgb8")
    # the oracle's own rays (host libm) give the same image within 1/255
    d = np.abs(out["rgb8"].astype(int) - own["rgb"].astype(int))
    assert d.max() <= 1 or (d > 0).mean() < 1e-3
    g.check()


def test_row_band_equals_full_render(cuda):
    import crt
    from crt import data
    sc = data.config0(n=20_000, width=128, height=96)
    g = crt.Scene(sc.mesh)
    full = g.render(sc.camera, sc.light, 128, 96, 2)
    band = g.render(sc.camera, sc.light, 128, 96, 2, rows=(17, 50))
    img_f = full["rgb8"].reshape(96, 128, 3)[::-1]  # memory rows are bottom-up
    img_b = band["rgb8"].reshape(96, 128, 3)[::-1]
    assert np.array_equal(img_f[17:50], img_b[17:50])
    assert (img_b[:17] == 0).all() and (img_b[50:] == 0).all()


def test_render_non_multiple_of_16(cuda):
    """1080-row images: the seed formula extends the reference's 16x16 grid."""
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    sc = data.config0(n=10_000)
    W, H = 72, 40
    out = crt.Scene(sc.mesh).render(sc.camera, sc.light, W, H, 3, aux=True)
    o = OracleScene(sc.mesh).render(sc.camera, sc.light, W, H, spp=3, aux=True)
    assert_equal(out["hit_id"], o["hit_id"], "hit id")
    assert_equal(out["rgb8"], o["rgb"], "rgb8")


@pytest.mark.parametrize("spp", [2, 3, 5, 7, 33])
def test_dof_sample_counts_with_partial_waves(cuda, spp):
    """Sample counts that are not a multiple of the lanes a pixel takes (the
    last wave is partial) and one above 32; thin lens on the silhouette of the
    large mesh, where samples of one pixel mix hits and misses, so the guesses
    of the stream offsets are wrong and re-traced.  Replayed rays give the
    oracle's hits and image bit for bit."""
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    sc = data.config1()
    W, H = 48, 40
    g = crt.Scene(sc.mesh)
    out = g.render(sc.camera, sc.light, W, H, spp, aux=True, rays=True)
    o = OracleScene(sc.mesh)
    own = o.render(sc.camera, sc.light, W, H, spp=spp, rays_out=True)
    assert np.allclose(out["rays"], own["rays"], rtol=2.0 ** -21, atol=1e-15)
    rep = o.render(sc.camera, sc.light, W, H, spp=spp, rays_in=out["rays"], aux=True)
    assert_equal(out["hit_id"], rep["hit_id"], "hit id")
    assert_equal(out["shadow"], rep["shadow"], "shadow")
    assert_equal(out["rgb8"], rep["rgb"], "rgb8")
    hits = (out["hit_id"].reshape(W * H, spp) >= 0)
    assert (hits.any(1) & ~hits.all(1)).any(), "no pixel mixes hits and misses"
    g.check()


def test_lens_tables_give_identical_rays(cuda):
    """The thin-lens tables (cos/sin and sqrt at every value an mrand draw
    can take, built once per device) against the inline double functions:
    every primary ray, hit and pixel of a thin-lens render is the same bit for
    bit with the tables on and off (3.7 M draws, across every binade)."""
    import crt
    from crt import data
    sc = data.config1(nu=60, width=640, height=360, spp=8)
    s = crt.Scene(sc.mesh)
    on = s.render(sc.camera, sc.light, sc.width, sc.height, sc.spp, rays=True, aux=True, rgbd=True)
    try:
        assert crt.lib().crt_set_lens_tables(0) == 0
        off = s.render(sc.camera, sc.light, sc.width, sc.height, sc.spp, rays=True, aux=True, rgbd=True)
    finally:
        crt.lib().crt_set_lens_tables(1)
    for k in ("rays", "hit_id", "shadow", "rgb_f64", "rgb8"):
        assert_equal(on[k], off[k], k)
    assert np.abs(on["rays"][:, :2]).max() > 0.01  # the lens moved the origins


def test_render_seed_mode(cuda):
    """crt_render_params.seed: 0 is the reference's streams (parity mode);
    another seed gives an independent render, the same on the GPU and in the
    oracle (area light and thin lens, so every draw matters)."""
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    sc = data.config1(nu=30, width=48, height=32, spp=4)
    light = data.Light(position=sc.light.position, radius=0.4)
    g, o = crt.Scene(sc.mesh), OracleScene(sc.mesh)
    base = g.render(sc.camera, light, 48, 32, 4, aux=True, rays=True)
    zero = g.render(sc.camera, light, 48, 32, 4, aux=True, rays=True, seed=0)
    assert_equal(zero["rays"], base["rays"], "seed 0 is the default")
    s7 = g.render(sc.camera, light, 48, 32, 4, aux=True, rays=True, rgbd=True, seed=7)
    assert (s7["rays"] != base["rays"]).any()
    ref = o.render(sc.camera, light, 48, 32, spp=4, aux=True, rays_in=s7["rays"], seed=7)
    assert_equal(s7["hit_id"], ref["hit_id"], "hit ids, seed 7")
    assert_equal(s7["shadow"], ref["shadow"], "shadow, seed 7")
    assert_equal(s7["rgb8"], ref["rgb"], "rgb8, seed 7")

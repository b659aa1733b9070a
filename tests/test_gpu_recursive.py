"""crt_render_recursive on the GPU against the oracle's recursive traceRay
(reflected and refracted rays below every primary ray).  Pinhole cameras:
bit-exact images, colours and primary hit ids.  Thin lens with an area
light: the oracle replays the GPU's primary rays (double cos/sin may differ
from the host's in the last bit), after which every colour is bit-exact,
which also pins the depth-first order of the light draws.  The Phong term
calls powf, which the reference runs as CUDA's and the oracle as the host
libm's: the two may differ in the last bit of the float result, so scenes
with a specular colour are compared within that rounding (a colour changes
by at most ks * 2^-23 per shaded hit) while hit ids stay exact."""
import numpy as np
import pytest

from conftest import assert_equal
from test_recursive import optics_scene, scene_view

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def optics_gpu(cuda):
    import crt
    from oracle.oracle import OracleScene
    mesh, optics = optics_scene()
    return crt.Scene(mesh), OracleScene(mesh), optics


@pytest.mark.parametrize("depth", [0, 1, 2, 4, 8])
def test_recursive_pinhole_bit_exact(optics_gpu, depth):
    g, o, optics = optics_gpu
    cam, light = scene_view()
    W, H, spp = 48, 40, 2
    out = g.render_recursive(cam, light, W, H, spp, depth, optics)
    ref = o.render_recursive(cam, light, W, H, spp, depth, optics)
    assert_equal(out["rgb_f64"], ref["color"], f"colour, depth {depth}")
    assert_equal(out["rgb8"], ref["rgb"], f"rgb8, depth {depth}")
    assert_equal(out["hit_id"], ref["hit_id"], "primary hit id")
    assert_equal(out["hit_t"], ref["hit_t"], "primary hit t")


def test_depth_zero_equals_plain_render(specular_gpu):
    """Same GPU, same powf: bit for bit, with highlights, lens and area light."""
    g, _, optics = specular_gpu
    cam, light = scene_view(aperture=0.05, radius=0.4)
    plain = g.render(cam, light, 40, 24, 5, rgbd=True, aux=True)
    rec = g.render_recursive(cam, light, 40, 24, 5, 0, optics)
    assert_equal(rec["rgb_f64"], plain["rgb_f64"], "colour")
    assert_equal(rec["rgb8"], plain["rgb8"], "rgb8")
    assert_equal(rec["hit_id"], plain["hit_id"], "hit id")


@pytest.mark.parametrize("spp", [1, 7])
def test_recursive_thin_lens_area_light_replayed(optics_gpu, spp):
    g, o, optics = optics_gpu
    cam, light = scene_view(aperture=0.08, radius=0.5)
    W, H, depth = 40, 32, 3
    out = g.render_recursive(cam, light, W, H, spp, depth, optics, rays=True)
    ref = o.render_recursive(cam, light, W, H, spp, depth, optics, rays_in=out["rays"])
    assert_equal(out["rgb_f64"], ref["color"], "colour")
    assert_equal(out["hit_id"], ref["hit_id"], "primary hit id")


@pytest.fixture(scope="module")
def specular_gpu(cuda):
    import crt
    from oracle.oracle import OracleScene
    mesh, optics = optics_scene(specular=True)
    return crt.Scene(mesh), OracleScene(mesh), optics


def _close_to_powf_rounding(got, ref, what):
    """Colours within the float rounding of powf; 8-bit values within 1."""
    d = np.abs(got["rgb_f64"] - ref["color"])
    assert d.max() <= 1e-5, f"{what}: colour differs by {d.max()}"
    q = np.abs(got["rgb8"].astype(int) - ref["rgb"].astype(int))
    assert q.max() <= 1 and (q == 0).mean() > 0.99, f"{what}: rgb8 differs by {q.max()}"


def test_specular_default_optics_and_row_band(specular_gpu):
    """Phong highlights; optics NULL takes kr = ks and ior = 1; a row band
    writes its rows as the full render does (bit for bit: same GPU)."""
    g, o, _ = specular_gpu
    cam, light = scene_view()
    W, H = 32, 32
    full = g.render_recursive(cam, light, W, H, 2, 3, None)
    ref = o.render_recursive(cam, light, W, H, 2, 3, None)
    assert_equal(full["hit_id"], ref["hit_id"], "primary hit id")
    _close_to_powf_rounding(full, ref, "default optics")
    band = g.render_recursive(cam, light, W, H, 2, 3, None, rows=(8, 24))
    rows = [(H - py - 1) * W + px for py in range(8, 24) for px in range(W)]
    assert_equal(band["rgb_f64"][rows], full["rgb_f64"][rows], "band")


def test_specular_plain_render(specular_gpu):
    """crt_render's Phong term (material.cu:31-35) against the oracle."""
    g, o, _ = specular_gpu
    cam, light = scene_view(aperture=0.0, radius=0.0)
    out = g.render(cam, light, 48, 40, 3, rgbd=True, aux=True)
    ref = o.render(cam, light, 48, 40, spp=3, aux=True)
    assert_equal(out["hit_id"], ref["hit_id"], "hit id")
    assert_equal(out["shadow"], ref["shadow"], "shadow")
    _close_to_powf_rounding(out, ref, "plain render")


def test_recursive_on_a_large_mesh(cuda):
    """The glass-and-mirror scene with an 81,920-face glass sphere, depth 4,
    192x128, 4 spp (pinhole): bit-exact against the oracle."""
    import crt
    from oracle.oracle import OracleScene
    mesh, optics = optics_scene(nu=64)
    cam, light = scene_view()
    out = crt.Scene(mesh).render_recursive(cam, light, 192, 128, 4, 4, optics)
    ref = OracleScene(mesh).render_recursive(cam, light, 192, 128, 4, 4, optics)
    assert_equal(out["rgb_f64"], ref["color"], "colour")


def test_recursive_rejects_bad_arguments(optics_gpu):
    import ctypes as C
    import crt
    g, _, optics = optics_gpu
    cam, light = scene_view()
    for depth in (-1, 9):
        with pytest.raises(crt.CrtError):
            g.render_recursive(cam, light, 16, 16, 1, depth, optics)
    c, lt, p = crt.render_args(cam, light, 16, 16, 1)
    shadow = np.zeros(16 * 16, np.int32)
    o = crt._RenderOut(None, None, None, None, shadow.ctypes.data, None, None, None, None, None)
    assert crt.lib().crt_render_recursive(g.h, C.byref(c), C.byref(lt), C.byref(p), 2, None, C.byref(o),
                                          None) == 1
    assert "writes" in crt.lib().crt_last_error_string().decode()


@pytest.mark.parametrize("depth", [0, 3])
def test_recursive_ray_counts(optics_gpu, depth):
    """traversal_stats of crt_render_recursive counts the rays of every
    sample's tree and their shadow rays: equal to the oracle's counts."""
    g, o, optics = optics_gpu
    cam, light = scene_view()
    W, H, spp = 40, 32, 3
    stats = np.zeros(2, np.uint64)
    out = dict(rgb_f64=np.zeros((W * H, 3)), hit_id=np.zeros(W * H * spp, np.int32), traversal_stats=stats)
    g.render_recursive(cam, light, W, H, spp, depth, optics, out=out)
    ref = o.render_recursive(cam, light, W, H, spp, depth, optics)
    assert_equal(out["rgb_f64"], ref["color"], "colour")
    assert stats.tolist() == list(ref["counts"])
    if depth == 0:
        assert stats[0] == W * H * spp and stats[1] == (out["hit_id"] >= 0).sum()



@pytest.mark.parametrize("ntri", [0, 1, 2])
def test_recursive_tiny_scenes(cuda, ntri):
    """Empty, one- and two-triangle scenes (a leaf root, a single internal
    node) with a reflecting and transmitting material, depth 4."""
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    v = np.array([[-1, -1, -3], [1, -1, -3], [0, 1, -3.5], [-1, 0.5, -2.5], [1, 0.5, -2.5], [0, -1, -2]], np.float32)
    tris = np.array([[0, 1, 2], [3, 4, 5]], np.int32)[:ntri].reshape(-1, 3)
    n = np.tile(np.array([[0, 0, 1]], np.float32), (6, 1))
    mats = np.zeros((1, 16))
    mats[0, 3:6] = 0.4
    mats[0, 9:12] = 0.5
    mats[0, 15] = 1.0
    mesh = data.Mesh(v, tris, n, tris.copy(), np.zeros(ntri, np.int32), mats)
    optics = np.array([[0.8, 0.7, 0.6, 1.3]])
    cam, light = scene_view()
    out = crt.Scene(mesh).render_recursive(cam, light, 24, 16, 2, 4, optics)
    ref = OracleScene(mesh).render_recursive(cam, light, 24, 16, 2, 4, optics)
    assert_equal(out["rgb_f64"], ref["color"], "colour")
    assert_equal(out["hit_id"], ref["hit_id"], "hit id")

"""The Python binding checks each caller buffer's type and size before it
passes the bare pointer to the C ABI (an undersized buffer would otherwise
be written past its end).  CPU only: the checks run before any library call,
so a scene handle is not needed."""
import numpy as np
import pytest


@pytest.fixture()
def scene(built):
    import crt
    s = object.__new__(crt.Scene)  # no device scene: every call below stops in the binding
    s.h, s.nv, s.nmat, s.ntri, s._keep = None, 10, 2, 4, []
    return s


def cam_light():
    from crt import data
    return data.Camera(), data.Light()


def test_render_buffers(scene):
    cam, light = cam_light()
    W, H, spp = 8, 4, 3
    with pytest.raises(ValueError, match="rgb8: 95 elements, 96 needed"):
        scene.render(cam, light, W, H, spp, out={"rgb8": np.zeros(95, np.uint8)})
    with pytest.raises(TypeError, match="rgb8"):
        scene.render(cam, light, W, H, spp, out={"rgb8": np.zeros((32, 3), np.float32)})
    with pytest.raises(ValueError, match="hit_id"):
        scene.render(cam, light, W, H, spp, out={"hit_id": np.zeros(W * H, np.int32)})  # per sample, not per pixel
    with pytest.raises(TypeError, match="hit_t"):
        scene.render(cam, light, W, H, spp, out={"hit_t": np.zeros(W * H * spp, np.float32)})
    with pytest.raises(ValueError, match="rays"):
        scene.render(cam, light, W, H, spp, out={"rays": np.zeros((W * H * spp, 3), np.float64)})
    with pytest.raises(TypeError, match="traversal_stats"):
        scene.render(cam, light, W, H, spp, out={"traversal_stats": np.zeros(2, np.uint32)})
    with pytest.raises(ValueError, match="contiguous"):
        scene.render(cam, light, W, H, spp, out={"rgb8": np.zeros((32, 6), np.uint8)[:, ::2]})


def test_recursive_optics_rows(scene):
    cam, light = cam_light()
    with pytest.raises(ValueError, match="optics: 4 elements, 8 needed"):
        scene.render_recursive(cam, light, 8, 4, 1, 2, np.zeros((1, 4)))


def test_vertices_and_adjoint_buffers(scene):
    cam, light = cam_light()
    with pytest.raises(ValueError, match="vertices"):
        scene.set_vertices(np.zeros((9, 3), np.float32), rebuild=False)
    with pytest.raises(ValueError, match="grad_rgb"):
        scene.adjoint(cam, light, 8, 4, 1, np.zeros((31, 3)))
    with pytest.raises(TypeError, match="grad_depth"):
        scene.adjoint(cam, light, 8, 4, 1, np.zeros((32, 3)), np.zeros(32, np.float32))
    with pytest.raises(ValueError, match="kd"):
        scene.adjoint(cam, light, 8, 4, 1, np.zeros((32, 3)),
                      out=dict(vertices=np.zeros((10, 3)), light=np.zeros(3), kd=np.zeros((1, 3))))


def test_torch_tensors_are_checked_too(scene):
    torch = pytest.importorskip("torch")
    cam, light = cam_light()
    with pytest.raises(TypeError, match="int64"):
        scene.render(cam, light, 8, 4, 1, out={"hit_id": torch.zeros(32, dtype=torch.int64)})
    with pytest.raises(ValueError, match="rgb_f64"):
        scene.render(cam, light, 8, 4, 1, out={"rgb_f64": torch.zeros((31, 3), dtype=torch.float64)})


def test_sort_and_morton_buffers(built):
    """crt_sort_pairs(_noalloc) and crt_morton write n 32-bit words through
    bare pointers: 1-D 4-byte integer arrays of at least n elements only."""
    import crt
    torch = pytest.importorskip("torch")
    k = torch.zeros(64, dtype=torch.int32)
    for f in (crt.sort_pairs, crt.sort_pairs_noalloc):
        with pytest.raises(ValueError, match="keys_out: 63 elements, 64 needed"):
            f(k, None, torch.zeros(63, dtype=torch.int32), torch.zeros(64, dtype=torch.int32))
        with pytest.raises(ValueError, match="vals_out"):
            f(k, None, torch.zeros(64, dtype=torch.int32), torch.zeros(10, dtype=torch.int32))
        with pytest.raises(ValueError, match="vals_in"):
            f(k, torch.zeros(32, dtype=torch.int32), torch.zeros(64, dtype=torch.int32),
              torch.zeros(64, dtype=torch.int32))
        with pytest.raises(TypeError, match="keys_out"):
            f(k, None, torch.zeros(64, dtype=torch.int64), torch.zeros(64, dtype=torch.int32))
        with pytest.raises(TypeError, match="keys_in"):
            f(torch.zeros(64, dtype=torch.float32), None, k.clone(), k.clone())
        with pytest.raises(ValueError, match="1-D"):
            f(torch.zeros((8, 8), dtype=torch.int32), None, k.clone(), k.clone())
    with pytest.raises(ValueError, match="codes: 9 elements, 10 needed"):
        crt.morton(torch.zeros((5, 3)), torch.zeros((10, 3), dtype=torch.int32), torch.zeros(6),
                   torch.zeros(9, dtype=torch.int32))
    with pytest.raises(TypeError, match="vidx"):
        crt.morton(torch.zeros((5, 3)), torch.zeros((10, 3), dtype=torch.int64), torch.zeros(6),
                   torch.zeros(10, dtype=torch.int32))

"""Borrowing scenes (crt_scene_create_borrowed): the caller's device arrays
are used in place.  Build products, hits and images equal those of a scene
that copies the same mesh; vertices rewritten in place are refitted or
rebuilt from; device-resident indices are range-checked on the device, so a
bad index is reported instead of being followed."""
import numpy as np
import pytest

from conftest import assert_equal

pytestmark = pytest.mark.gpu


def _device_mesh(mesh):
    import torch
    from crt import data
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")  # noqa: E731
    return data.Mesh(t(mesh.verts, torch.float32), t(mesh.vidx, torch.int32), t(mesh.normals, torch.float32),
                     t(mesh.nidx, torch.int32), t(mesh.matid, torch.int32),
                     t(np.asarray(mesh.materials, np.float64).reshape(-1, 16), torch.float64))


def test_borrowed_equals_copied(cuda):
    import crt
    from crt import data
    sc = data.config1(nu=40, width=96, height=64, spp=4)
    own = crt.Scene(sc.mesh)
    dm = _device_mesh(sc.mesh)
    bor = crt.Scene(dm, borrow=True)
    a, b = own.export(), bor.export()
    for k in a:
        assert_equal(b[k], a[k], k)
    ra = own.render(sc.camera, sc.light, 96, 64, 4, aux=True, rgbd=True)
    rb = bor.render(sc.camera, sc.light, 96, 64, 4, aux=True, rgbd=True)
    for k in ("hit_id", "shadow", "rgb_f64", "rgb8"):
        assert_equal(rb[k], ra[k], k)


def test_borrowed_refit_and_rebuild_in_place(cuda):
    import crt
    from crt import data
    anim = data.Animation(nu=30, frames=10)
    sc = anim.scene(width=64, height=48, spp=2)
    dm = _device_mesh(sc.mesh)
    bor = crt.Scene(dm, borrow=True)
    own = crt.Scene(sc.mesh)
    for frame, rebuild in ((3, False), (7, True)):
        v = anim.vertices(frame).astype(np.float32)
        dm.verts.copy_(__import__("torch").as_tensor(v, device="cuda"))
        bor.set_vertices(None, rebuild)
        own.set_vertices(v, rebuild)
        ra = own.render(sc.camera, sc.light, 64, 48, 2, aux=True, rgbd=True)
        rb = bor.render(sc.camera, sc.light, 64, 48, 2, aux=True, rgbd=True)
        assert_equal(rb["hit_id"], ra["hit_id"], f"hit ids, frame {frame}")
        assert_equal(rb["rgb_f64"], ra["rgb_f64"], f"colour, frame {frame}")
    with pytest.raises(crt.CrtError):
        bor.set_vertices(anim.vertices(1).astype(np.float32), False)  # a borrowing scene takes no new array
    with pytest.raises(crt.CrtError):
        bor.set_materials(np.asarray(sc.mesh.materials))


def test_device_indices_are_range_checked(cuda):
    import torch
    import crt
    from crt import data
    mesh = data.soup(500, seed=4)
    for field, bad in (("vidx", 10 ** 6), ("nidx", -1), ("matid", 3)):
        dm = _device_mesh(mesh)
        arr = getattr(dm, field)
        arr.view(-1)[77] = bad
        for borrow in (False, True):
            with pytest.raises(crt.CrtError) as e:
                crt.Scene(dm, borrow=borrow)
            assert "out of range" in str(e.value)
    dm = _device_mesh(mesh)
    s = crt.Scene(dm)  # valid device arrays, copied
    s.check()
    host = _device_mesh(mesh)
    host.verts = host.verts.cpu()
    with pytest.raises(crt.CrtError) as e:  # borrowing needs device memory throughout
        crt.Scene(host, borrow=True)
    assert "device" in str(e.value)
    torch.cuda.synchronize()

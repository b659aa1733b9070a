"""Batched form: many meshes of uneven sizes, each with its own camera, light
and image size, built and rendered by the persistent cooperative kernel (one
launch, or the render in a second one; replayed from a CUDA graph).  Every mesh's build products and image
must equal what the plain path gives for that mesh alone, bit for bit, for
every supported launch shape; the plain path is itself pinned to the oracle
(test_gpu_build, test_gpu_render), and a few meshes are checked against the
oracle here as well."""
import math

import numpy as np
import pytest

from conftest import assert_equal

pytestmark = pytest.mark.gpu


def _scenes():
    """Ragged sizes: the generator's log-uniform soups plus the edge cases one
    and two triangles; image sizes that are not multiples of any tile."""
    from crt import data
    sc = data.config3(count=10, lo=1_000, hi=20_000, width=48, height=40, spp=2, seed=5)
    sizes = [(37, 23, 1), (64, 48, 2), (16, 16, 3), (33, 1, 5), (1, 31, 1), (20, 12, 16), (9, 7, 20)]
    out = []
    for i, s in enumerate(sc):
        w, h, spp = sizes[i % len(sizes)]
        out.append((s.mesh, (s.camera, s.light, w, h, spp)))
    rng = np.random.default_rng(11)
    for n in (1, 2):
        m = data.soup(n, scale=0.5, cam_pos=(0.0, 0.0, -3.0), rng=rng)
        out.append((m, (data.Camera(fov=60.0, focal_point=1.0, fstop=math.inf),
                        data.Light(position=data.light_for((2.0, 2.0, -2.0), (0.0, 0.0, -3.0))), 24, 20, 2)))
    return out


@pytest.fixture(scope="module")
def batch_case(cuda):
    import crt
    items = _scenes()
    b = crt.Batch([m for m, _ in items], [v for _, v in items])
    return crt, items, b


def _plain(crt, items):
    imgs, exps = [], []
    for mesh, (cam, light, w, h, spp) in items:
        s = crt.Scene(mesh)
        imgs.append(s.render(cam, light, w, h, spp)["rgb8"])
        exps.append(s.export())
        s.check()
        s.close()
    return imgs, exps


def test_batch_images_and_exports_equal_plain(batch_case):
    crt, items, b = batch_case
    total = int(b.offsets[-1])
    out = np.zeros((total, 3), np.uint8)
    b.run(out, graph=True)
    b.check()
    imgs, exps = _plain(crt, items)
    for m, img in enumerate(b.images(out)):
        assert_equal(img, imgs[m], f"mesh {m} image")
        e = b.export(m)
        for k in ("scene_box", "codes", "ids", "nodes", "node_boxes"):
            assert_equal(e[k], exps[m][k], f"mesh {m} {k}")
    assert any(img.any() for img in imgs)


def test_batch_every_tuning_same_image(batch_case):
    crt, items, b = batch_case
    total = int(b.offsets[-1])
    ref = np.zeros((total, 3), np.uint8)
    b.set_tuning(128, 1, 0)
    b.run(ref, graph=False)
    for bs in (128, 256):
        for lanes in (1, 2, 4, 8, 16, 32):
            for stack in (0, 8, 16):
                for launches in (1, 2):
                    b.set_tuning(bs, lanes, stack, launches)
                    out = np.zeros_like(ref)
                    b.run(out, graph=bool(stack & 8))
                    assert_equal(out, ref, f"tuning {bs} lanes {lanes} stack {stack} launches {launches}")
    b.check()


def test_batch_graph_replay_and_autotune(batch_case):
    crt, items, b = batch_case
    total = int(b.offsets[-1])
    first = np.zeros((total, 3), np.uint8)
    b.set_tuning(128, 4, 0)
    b.run(first, graph=False)
    t = b.autotune()
    assert t["block_size"] in (128, 256) and t["lanes_per_pixel"] in (1, 2, 4, 8, 16, 32)
    assert t["stack"] in (0, 8, 16) and t["launches"] in (1, 2)
    assert t["render_ms"] > 0
    for _ in range(3):  # replays of one captured graph
        again = np.zeros_like(first)
        b.run(again, graph=True)
        assert_equal(again, first, "graph replay")
    import torch
    dev = torch.zeros((total, 3), dtype=torch.uint8, device="cuda")
    b.run(dev, graph=True)
    torch.cuda.synchronize()
    assert_equal(dev.cpu().numpy(), first, "device output")
    b.check()


def test_batch_spot_check_against_oracle(batch_case):
    from oracle.oracle import OracleScene
    crt, items, b = batch_case
    total = int(b.offsets[-1])
    out = np.zeros((total, 3), np.uint8)
    b.run(out, graph=True)
    imgs = b.images(out)
    for m in (0, 3, len(items) - 1):
        mesh, (cam, light, w, h, spp) = items[m]
        o = OracleScene(mesh)
        e, r = b.export(m), o.export()
        assert_equal(e["codes"], r["codes"], f"mesh {m} codes")
        assert_equal(e["ids"], r["ids"], f"mesh {m} ids")
        assert_equal(e["nodes"], r["nodes"], f"mesh {m} topology")
        assert_equal(e["node_boxes"], r["node_boxes"], f"mesh {m} boxes")
        ref = o.render(cam, light, w, h, spp=spp)["rgb"]
        # thin-lens rays use cos/sin, which may differ from the host's in the
        # last bit: the image is held to 1/255 per channel
        d = np.abs(imgs[m].astype(int) - ref.astype(int))
        assert d.max() <= 1, f"mesh {m}: max channel difference {d.max()}"


def test_batch_rejects_bad_input(cuda):
    import crt
    from crt import data
    rng = np.random.default_rng(0)
    m = data.soup(10, scale=1.0, cam_pos=(0.0, 0.0, -3.0), rng=rng)
    view = (data.Camera(), data.Light(), 8, 8, 1)
    with pytest.raises(crt.CrtError, match="INVALID_ARG"):
        crt.Batch([m] * 1025, [view] * 1025)
    bad = data.Mesh(m.verts, m.vidx.copy(), m.normals, m.nidx, m.matid, m.materials)
    bad.vidx[3, 1] = m.verts.shape[0]
    with pytest.raises(crt.CrtError, match="out of range"):
        crt.Batch([m, bad], [view, view])
    b = crt.Batch([m, m], [view, view])
    with pytest.raises(crt.CrtError, match="unsupported tuning"):
        b.set_tuning(64, 4, 0)  # the persistent kernel runs 128- or 256-thread blocks
    with pytest.raises(crt.CrtError, match="unsupported tuning"):
        b.set_tuning(256, 4, 0, 3)
    b.close()
    nan = data.Mesh(m.verts.copy(), m.vidx, m.normals, m.nidx, m.matid, m.materials)
    nan.verts[0, 0] = np.nan
    b = crt.Batch([m, nan], [view, view])
    b.run(None)
    with pytest.raises(crt.CrtError, match="non-finite"):
        b.check()

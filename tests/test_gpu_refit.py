"""Dynamic refit vs rebuild (the animated 1,003,520-face mesh): the GPU keeps
frame 0's topology and refits every frame (RefitBounds on fixed nodes); the
reference rebuilds.  Closest hits do not depend on the tree (the candidate set
is every triangle whose box and Moller-Trumbore test pass; only an exact t tie
could be broken differently), so per-sample hit ids and t must match the
oracle's full rebuild bit for bit at every checked frame."""
import pytest

from conftest import assert_equal

pytestmark = pytest.mark.gpu

FRAMES = (0, 1, 30, 59)


def test_refit_hits_match_rebuild_per_frame(cuda):
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    anim = data.Animation()
    sc = anim.scene()
    W, H, spp = 160, 90, 4
    g = crt.Scene(anim.mesh0)
    o = OracleScene(anim.mesh0)
    for f in range(max(FRAMES) + 1):
        if f > 0:
            g.set_vertices(anim.vertices(f), rebuild=False)  # refit on frame 0's topology
        if f not in FRAMES:
            continue
        out = g.render(sc.camera, sc.light, W, H, spp, aux=True, rays=True)
        o.set_vertices(anim.vertices(f), rebuild=True)
        ref = o.render(sc.camera, sc.light, W, H, spp=spp, rays_in=out["rays"], aux=True)
        assert_equal(out["hit_id"], ref["hit_id"], f"hit id, frame {f}")
        assert_equal(out["hit_t"], ref["hit_t"], f"hit t, frame {f}")
        assert (out["hit_id"] >= 0).mean() > 0.1
    g.check()


def test_refit_boxes_equal_rebuild_boxes_on_same_topology(cuda):
    """A refit of the rebuilt tree's own topology reproduces its boxes exactly."""
    import crt
    from crt import data
    anim = data.Animation(nu=40)
    g = crt.Scene(anim.mesh0)
    v = anim.vertices(17)
    g.set_vertices(v, rebuild=True)
    a = g.export()
    g.refit()  # same vertices, same topology
    b = g.export()
    assert_equal(a["node_boxes"], b["node_boxes"], "boxes")
    # and the refit boxes of moved vertices contain every triangle
    g.set_vertices(anim.vertices(40), rebuild=False)
    e = g.export()
    n = anim.mesh0.ntri
    leaf_boxes = e["node_boxes"][n - 1:]
    tri = anim.vertices(40)[anim.tris[e["ids"]]]
    assert (leaf_boxes[:, :3] == tri.min(1)).all() and (leaf_boxes[:, 3:] == tri.max(1)).all()


def test_refit_boxes_match_oracle_refit(cuda):
    """Refits of moved vertices on a fixed topology give the oracle's refit
    boxes bit for bit: 72,000 triangles span 141 refit blocks in 5 groups, so
    the spanning nodes' boxes come from block, group and edge boxes."""
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    anim = data.Animation(nu=60)
    g = crt.Scene(anim.mesh0)
    o = OracleScene(anim.mesh0)
    for f in (13, 41):
        v = anim.vertices(f)
        g.set_vertices(v, rebuild=False)
        o.set_vertices(v, rebuild=False)
        a, b = g.export(), o.export()
        assert_equal(a["nodes"], b["nodes"], f"topology, frame {f}")
        assert_equal(a["node_boxes"], b["node_boxes"], f"boxes, frame {f}")

"""The hand-written adjoint (crt_adjoint_lambert) on the differentiable
workload: a 200,000-face icosphere with per-triangle albedo, 512x512, 4 spp,
pinhole, Lambert with a point light; target rendered from vertices perturbed
by N(0, 0.005^2) (seed 3); L2 loss over interior pixels.

* against the oracle's float64 reference gradient (same samples, same hits);
* against central finite differences (h = 1e-3 on float32 vertices) on 64
  random vertices (all three coordinates), the light position and albedos,
  with the loss restricted to pixels whose samples hit the same triangles and
  shadow states in the base and both perturbed renders (interior pixels: no
  visibility edges), to 1e-3 relative;
* through torch.autograd (LambertRender).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(torch, W=512, H=512, spp=4):
    import crt
    from crt import data
    sc = data.config4(width=W, height=H, spp=spp)
    tgt = data.config4(width=W, height=H, spp=spp, perturbed=True)
    g = crt.Scene(sc.mesh)
    t_img = torch.empty((W * H, 3), dtype=torch.float64, device="cuda")
    gt = crt.Scene(tgt.mesh)
    gt.render(tgt.camera, tgt.light, W, H, spp, out={"rgb_f64": t_img})
    return sc, g, t_img


def _render(torch, g, sc, W, H, spp, light=None):
    n = W * H
    img = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    hid = torch.empty(n * spp, dtype=torch.int32, device="cuda")
    sid = torch.empty(n * spp, dtype=torch.int32, device="cuda")
    sh = torch.empty(n * spp, dtype=torch.int32, device="cuda")
    g.render(sc.camera, light or sc.light, W, H, spp, out={"rgb_f64": img, "hit_id": hid, "shadow": sh,
                                                           "shadow_id": sid})
    return img, hid.view(n, spp), sh.view(n, spp), sid.view(n, spp)


def test_adjoint_matches_float64_reference(cuda):
    torch = cuda
    from oracle.oracle import OracleScene
    W = H = 96
    spp = 4
    sc, g, _ = _setup(torch, W, H, spp)
    img, _, _, _ = _render(torch, g, sc, W, H, spp)
    rng = np.random.default_rng(7)
    grad = rng.normal(size=(W * H, 3))
    gdep = rng.normal(size=W * H) * 0.1
    ga = g.adjoint(sc.camera, sc.light, W, H, spp, grad, gdep)
    go = OracleScene(sc.mesh).adjoint(sc.camera, sc.light, W, H, spp, grad, gdep)
    for k in ("vertices", "light", "kd"):
        a, b = ga[k], go[k]
        scale = np.abs(b).max()
        assert scale > 0, k
        assert np.abs(a - b).max() <= 1e-9 * scale, f"{k}: {np.abs(a - b).max()} vs scale {scale}"


def _fd_check(torch, sc, g, t_img, W, H, spp, perturb, analytic, h):
    """perturb(x) moves the parameter by x (0 restores) and returns its actual
    value; analytic(grad) returns the adjoint component for d loss / d img.
    Returns central differences at h, h/2, h/4, their two-stage Richardson
    combination (cancelling the h^2 and h^4 truncation terms), and the adjoint,
    all on the same set of interior pixels: every sample hits the same
    triangle, with the same shadow state and occluder, in the base and all six
    perturbed renders."""
    perturb(0)
    img0, hid0, sh0, sid0 = _render(torch, g, sc, W, H, spp)
    steps = (1.0, 0.5, 0.25)
    r = {}
    for s in steps:
        for sign in (-1.0, 1.0):
            x = perturb(sign * s * h)
            r[sign * s] = (x,) + _render(torch, g, sc, W, H, spp)
    perturb(0)
    same = torch.ones(W * H, dtype=torch.bool, device="cuda")
    for k in r:
        _, _, hid, sh, sid = r[k]
        same &= ((hid == hid0) & (sh == sh0) & (sid == sid0)).all(1)
    m = same.to(torch.float64)[:, None]
    L = {k: (((r[k][1] - t_img) ** 2) * m).sum().item() for k in r}
    d = [(L[s] - L[-s]) / (r[s][0] - r[-s][0]) for s in steps]
    r1 = [(4.0 * d[1] - d[0]) / 3.0, (4.0 * d[2] - d[1]) / 3.0]
    r2 = (16.0 * r1[1] - r1[0]) / 15.0
    an = analytic(2.0 * (img0 - t_img) * m)
    return d[0], d[1], r2, an


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) / np.linalg.norm(a)


def test_adjoint_matches_central_differences(cuda):
    """Central differences with h = 1e-3 on float32 vertices.  h is about 8% of
    a triangle edge here, so a single central difference carries an O(h^2)
    truncation error of a few percent (it falls ~4x when h halves); the
    two-stage Richardson combination of h, h/2, h/4 cancels the h^2 and h^4
    terms and is compared at 1e-3 relative.  The plain h = 1e-3 figure is
    checked to its truncation level."""
    torch = cuda
    W = H = 512
    spp = 4
    h = 1e-3
    sc, g, t_img = _setup(torch, W, H, spp)
    mesh = sc.mesh
    v = mesh.verts.copy()
    # 64 random vertices among those the camera sees (a hit in the base render)
    _, hid0, _, _ = _render(torch, g, sc, W, H, spp)
    hit_tris = np.unique(hid0.cpu().numpy())
    hit_tris = hit_tris[hit_tris >= 0]
    rng = np.random.default_rng(11)
    verts = rng.choice(np.unique(mesh.vidx[hit_tris].ravel()), 64, replace=False)
    res = []
    for vi in verts:
        for c in range(3):
            def perturb(x, vi=vi, c=c):
                w = v.copy()
                w[vi, c] = np.float32(v[vi, c] + x)
                g.set_vertices(w, rebuild=True)
                return float(w[vi, c])

            def analytic(grad, vi=vi, c=c):
                return g.adjoint(sc.camera, sc.light, W, H, spp, grad)["vertices"][vi, c]

            res.append(_fd_check(torch, sc, g, t_img, W, H, spp, perturb, analytic, h))
    d1, d2, rx, an = map(np.array, zip(*res))
    assert np.linalg.norm(rx) > 0
    print(f"vertices: Richardson {_rel(rx, an):.2e}, h {_rel(d1, an):.2e}, h/2 {_rel(d2, an):.2e}")
    assert _rel(rx, an) <= 1e-3, f"vertices: Richardson {_rel(rx, an):.2e}, h {_rel(d1, an):.2e}, h/2 {_rel(d2, an):.2e}"
    assert _rel(d1, an) <= 0.1 and _rel(d2, an) < 0.5 * _rel(d1, an)  # O(h^2) truncation

    # light position (the passed position; a shift of the configured one)
    from crt import data
    base = sc.light
    res = []
    for c in range(3):
        def perturb(x, c=c):
            p = list(base.position)
            p[c] = p[c] + x
            sc.light = data.Light(position=tuple(p)) if x != 0 else base
            return p[c]

        def analytic(grad):
            return g.adjoint(sc.camera, base, W, H, spp, grad)["light"][c]

        res.append(_fd_check(torch, sc, g, t_img, W, H, spp, perturb, analytic, h))
        sc.light = base
    d1, d2, rx, an = map(np.array, zip(*res))
    assert _rel(rx, an) <= 1e-3 and _rel(d1, an) <= 1e-2

    # per-triangle albedo: the image is linear in kd
    mats = np.asarray(mesh.materials, np.float64).copy()
    tris = rng.choice(hit_tris, 16, replace=False)
    res = []
    for t in tris:
        def perturb(x, t=t):
            mm = mats.copy()
            mm[t, 3] += x
            g.set_materials(mm)
            return mm[t, 3]

        def analytic(grad, t=t):
            return g.adjoint(sc.camera, sc.light, W, H, spp, grad)["kd"][t, 0]

        res.append(_fd_check(torch, sc, g, t_img, W, H, spp, perturb, analytic, h))
    d1, d2, rx, an = map(np.array, zip(*res))
    assert _rel(d1, an) <= 1e-3 and _rel(rx, an) <= 1e-3


def test_autograd_function(cuda):
    torch = cuda
    from crt import autograd, data
    W = H = 64
    spp = 4
    sc = data.config4(width=W, height=H, spp=spp)
    r = autograd.Renderer(sc.mesh, sc.camera, sc.light, W, H, spp)
    verts = torch.tensor(sc.mesh.verts, device="cuda", requires_grad=True)
    lp = torch.tensor(sc.light.position, dtype=torch.float64, requires_grad=True)
    alb = torch.tensor(sc.mesh.materials[:, 3:6], dtype=torch.float64, requires_grad=True)
    img, depth = autograd.render(verts, lp, alb, r)
    loss = (img ** 2).sum() + 0.1 * depth.sum()
    loss.backward()
    direct = r.adjoint(2 * img.detach(), torch.full_like(depth, 0.1))
    assert torch.allclose(verts.grad.double(), direct["vertices"].float().double(), rtol=1e-6, atol=1e-9)
    assert torch.allclose(lp.grad, direct["light"].cpu())
    assert torch.allclose(alb.grad, direct["kd"].cpu())
    assert verts.grad.abs().sum() > 0 and lp.grad.abs().sum() > 0 and alb.grad.abs().sum() > 0

"""LBVH build on the GPU: bit-exact against the reference (golden fixtures)
and against the oracle on fresh seeded scenes, through the C ABI."""
import os

import numpy as np
import pytest

from conftest import assert_equal, golden_files, golden_mesh

pytestmark = pytest.mark.gpu


def _build_equal(gpu_ex, ref, tri_boxes=None):
    for k in ("codes", "ids", "nodes", "node_boxes"):
        assert_equal(gpu_ex[k], ref[k], k)
    box = np.concatenate([ref["smin"], ref["smax"]]).astype(np.float32)
    assert_equal(gpu_ex["scene_box"], box, "scene box")


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: os.path.basename(p)[:-4])
def test_build_matches_reference_golden(cuda, path):
    import crt
    z = np.load(path)
    s = crt.Scene(golden_mesh(z))
    _build_equal(s.export(), z)


# 512-leaf refit blocks and groups of 32 blocks (16384 leaves): sizes at and
# beside both edges, and a partial last group
@pytest.mark.parametrize("n", [1, 2, 3, 4, 31, 511, 512, 513, 2047, 2048, 2049, 16383, 16384, 16385, 16897, 100_000])
def test_build_matches_oracle_soup(cuda, n):
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    m = data.soup(n, seed=n)
    _build_equal(crt.Scene(m).export(), OracleScene(m).export())


def test_build_matches_oracle_icosphere_1m(cuda):
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    m = data.icosphere(224)
    _build_equal(crt.Scene(m).export(), OracleScene(m).export())


def test_build_duplicate_codes(cuda):
    """Runs of equal Morton codes exercise delta()'s index tie-break."""
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    rng = np.random.default_rng(1)
    n = 20000
    cent = rng.integers(0, 3, (n, 3)).astype(np.float64)
    off = rng.normal(0, 1e-4, (n, 3, 3))
    off -= off.mean(1, keepdims=True)
    v = (cent[:, None, :] + off).reshape(-1, 3).astype(np.float32)
    vidx = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    nrm = np.tile(np.array([[0, 0, 1]], np.float32), (3 * n, 1))
    m = data.Mesh(v, vidx, nrm, vidx.copy(), np.zeros(n, np.int32), data.lambert_material()[None])
    _build_equal(crt.Scene(m).export(), OracleScene(m).export())


def test_rebuild_is_idempotent(cuda):
    import crt
    from crt import data
    m = data.soup(5000, seed=3)
    s = crt.Scene(m)
    a = s.export()
    s.build()
    b = s.export()
    for k in a:
        assert_equal(a[k], b[k], k)


@pytest.mark.parametrize("n,bits", [(1, 30), (5, 30), (2048, 30), (2049, 30), (300_000, 30), (300_000, 32),
                                    (100_000, 10), (70_000, 17)])
def test_sort_pairs_stable(cuda, n, bits):
    import crt
    torch = cuda
    rng = np.random.default_rng(n + bits)
    hi = min(1 << bits, 1 << 32)
    keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 3] = keys[0]  # a long run of equal keys tests stability
    rng.shuffle(keys)
    vals = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    kin = torch.from_numpy(keys.view(np.int32)).cuda()
    vin = torch.from_numpy(vals.view(np.int32)).cuda()
    ko, vo = torch.empty_like(kin), torch.empty_like(vin)
    crt.sort_pairs(kin, vin, ko, vo, key_bits=bits)
    order = np.argsort(keys, kind="stable")
    assert_equal(ko.cpu().numpy().view(np.uint32), keys[order], "keys")
    assert_equal(vo.cpu().numpy().view(np.uint32), vals[order], "values")
    # values omitted: indices 0..n-1
    crt.sort_pairs(kin, None, ko, vo, key_bits=bits)
    assert_equal(vo.cpu().numpy(), order.astype(np.int32), "implicit values")


def test_morton_stage_matches_oracle(cuda):
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    torch = cuda
    m = data.soup(50_000, seed=11)
    ex = OracleScene(m).export()
    box = torch.tensor(np.concatenate([ex["smin"], ex["smax"]]).astype(np.float32)).cuda()
    v = torch.from_numpy(m.verts).cuda()
    vi = torch.from_numpy(m.vidx).cuda()
    codes = torch.empty(m.ntri, dtype=torch.int32, device="cuda")
    crt.morton(v, vi, box, codes)
    torch.cuda.synchronize()
    assert_equal(codes.cpu().numpy(), ex["codes_unsorted"], "codes")
    # an index one past the last vertex, and a negative one: refused, and
    # only those triangles lose their codes (their vertices are not read)
    bad = m.vidx.copy()
    bad[17, 1] = m.verts.shape[0]
    bad[4000, 2] = -1
    codes.fill_(-1)
    with pytest.raises(crt.CrtError, match="vertex index"):
        crt.morton(v, torch.from_numpy(bad).cuda(), box, codes)
    want = ex["codes_unsorted"].copy()
    want[[17, 4000]] = 0
    assert_equal(codes.cpu().numpy(), want, "codes beside the bad triangles")


def _boundary_mesh(seed):
    """Triangles whose centroids sit on, and a few float steps either side of,
    every Morton cell boundary of each axis (the cases the FP32 fast path must
    hand to the double path), inside a box fixed by one frame triangle."""
    from crt import data
    rng = np.random.default_rng(seed)
    mn = np.array([-3.7, 0.1, -1e-3], np.float32)
    mx = np.array([5.3, 0.7, 2.0e3], np.float32)
    cand = []
    for a in range(3):
        t = mn[a].astype(np.float64) + np.arange(1025) / 1024.0 * (mx[a].astype(np.float64) - mn[a])
        f = t.astype(np.float32)
        vals = [f]
        for _ in range(3):
            vals.append(np.nextafter(vals[-1], np.float32(np.inf)))
        lo = f
        for _ in range(3):
            lo = np.nextafter(lo, np.float32(-np.inf))
            vals.append(lo)
        c = np.clip(np.concatenate(vals), mn[a], mx[a])
        cand.append(c)
    n = 60000
    p = np.stack([cand[a][rng.integers(0, cand[a].size, n)] for a in range(3)], 1)
    # half degenerate (centroid = the point), half with vertices a few ulps
    # apart so that lo + hi is not a float
    d = rng.integers(1, 4, (n, 3)).astype(np.float32) * np.spacing(np.abs(p).astype(np.float32) + 1e-30)
    d[: n // 2] = 0
    tri = np.stack([p - d, p + d, p], 1).astype(np.float32)
    tri = np.clip(tri, mn, mx)
    frame = np.stack([mn, mx, mn])[None]
    v = np.concatenate([frame, tri]).reshape(-1, 3).astype(np.float32)
    nt = n + 1
    vidx = np.arange(3 * nt, dtype=np.int32).reshape(nt, 3)
    nrm = np.tile(np.array([[0, 0, 1]], np.float32), (3 * nt, 1))
    return data.Mesh(v, vidx, nrm, vidx.copy(), np.zeros(nt, np.int32), data.lambert_material()[None])


def test_morton_cell_boundaries(cuda):
    """Morton codes of centroids on and beside every cell boundary: the FP32
    fast path either gets the double formula's cell or defers to it."""
    import crt
    from oracle.oracle import OracleScene
    torch = cuda
    m = _boundary_mesh(7)
    ex = OracleScene(m).export()
    box = torch.tensor(np.concatenate([ex["smin"], ex["smax"]]).astype(np.float32)).cuda()
    codes = torch.empty(m.ntri, dtype=torch.int32, device="cuda")
    crt.morton(torch.from_numpy(m.verts).cuda(), torch.from_numpy(m.vidx).cuda(), box, codes)
    torch.cuda.synchronize()
    assert_equal(codes.cpu().numpy(), ex["codes_unsorted"], "codes")
    _build_equal(crt.Scene(m).export(), ex)


@pytest.mark.parametrize("n", [1, 2, 3, 1000, 2049, 20000])
def test_stage_hierarchy_and_refit(cuda, n):
    """crt_hierarchy and crt_refit, the stage-level entry points, on the
    sorted codes and ids of a build: the same HNode triplets and node boxes
    as the full build's export (itself bit-exact against the oracle)."""
    import torch
    import crt
    from crt import data
    mesh = data.soup(n, seed=11 + n)
    ex = crt.Scene(mesh).export()
    dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a).view(dt), device="cuda")  # noqa: E731
    codes, ids = dev(ex["codes"], np.int32), dev(ex["ids"], np.int32)
    nn = 2 * n - 1
    nodes3 = torch.full((nn * 3,), -7, dtype=torch.int32, device="cuda")
    lib = crt.lib()
    assert lib.crt_hierarchy(codes.data_ptr(), ids.data_ptr(), n, nodes3.data_ptr(), None) == 0
    assert_equal(nodes3.cpu().numpy().reshape(nn, 3), ex["nodes"], "nodes")
    verts = dev(mesh.verts.astype(np.float32), np.float32)
    vidx = dev(mesh.vidx.astype(np.int32), np.int32)
    boxes = torch.full((nn * 6,), float("nan"), dtype=torch.float32, device="cuda")
    assert lib.crt_refit(verts.data_ptr(), len(mesh.verts), vidx.data_ptr(), n, ids.data_ptr(), nodes3.data_ptr(),
                         boxes.data_ptr(), None) == 0
    assert_equal(boxes.cpu().numpy().reshape(nn, 6), ex["node_boxes"], "node boxes")
    if n >= 2:  # corrupt triplets and ids are reported, not followed
        bad = nodes3.clone()
        bad[3 * (n - 1)] = 10 ** 6
        assert lib.crt_refit(verts.data_ptr(), len(mesh.verts), vidx.data_ptr(), n, ids.data_ptr(), bad.data_ptr(),
                             boxes.data_ptr(), None) == 1
        bad_ids = ids.clone()
        bad_ids[0] = n + 5
        assert lib.crt_refit(verts.data_ptr(), len(mesh.verts), vidx.data_ptr(), n, bad_ids.data_ptr(),
                             nodes3.data_ptr(), boxes.data_ptr(), None) == 1
        assert "out of range" in lib.crt_last_error_string().decode()

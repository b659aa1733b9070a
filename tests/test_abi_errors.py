"""Argument checking of the C ABI, on the CPU: every call below is refused
before the library touches the GPU, with CRT_INVALID_ARG and a message in
crt_last_error_string(), and nothing exits the process (the reference calls
exit(1) on errors, src/scene.cpp:71-81)."""
import ctypes as C

import numpy as np
import pytest

INVALID = 1


@pytest.fixture()
def lib(built):
    import crt
    return crt.lib()


def desc(n, nv=3, nn=1, nmat=1, verts=True, mats=True):
    import crt
    keep = [np.zeros(3 * max(nv, 1), np.float32), np.zeros(3 * max(nn, 1), np.float32),
            np.zeros(3 * max(min(n, 4), 1), np.int32), crt._Material()]
    d = crt._MeshDesc(keep[0].ctypes.data if verts else None, nv, keep[1].ctypes.data, nn,
                      keep[2].ctypes.data if verts else None, None, n,
                      C.addressof(keep[3]) if mats else None, nmat, None)
    return d, keep


def error(lib):
    return lib.crt_last_error_string().decode()


def test_scene_create_refuses_bad_descriptions(lib):
    out = C.c_void_p()
    assert lib.crt_scene_create(None, None, C.byref(out)) == INVALID
    d, keep = desc(n=(1 << 28) + 1)  # above CRT_MAX_TRIANGLES: refused before any index is read
    assert lib.crt_scene_create(C.byref(d), None, C.byref(out)) == INVALID
    assert "num_triangles" in error(lib)
    d, keep = desc(n=-1)
    assert lib.crt_scene_create(C.byref(d), None, C.byref(out)) == INVALID
    d, keep = desc(n=1, nv=-3)
    assert lib.crt_scene_create(C.byref(d), None, C.byref(out)) == INVALID and "negative" in error(lib)
    d, keep = desc(n=1, verts=False)
    assert lib.crt_scene_create(C.byref(d), None, C.byref(out)) == INVALID and "vertices" in error(lib)
    d, keep = desc(n=1, mats=False)
    assert lib.crt_scene_create(C.byref(d), None, C.byref(out)) == INVALID and "material" in error(lib)
    assert not out.value


def test_null_handles_are_refused(lib):
    assert lib.crt_bvh_build(None, None) == INVALID
    assert lib.crt_bvh_refit(None, None) == INVALID
    assert lib.crt_scene_check(None, None) == INVALID
    assert lib.crt_batch_check(None, None) == INVALID
    assert lib.crt_batch_run(None, 1, None, None) == INVALID
    assert lib.crt_scene_destroy(None) == 0 and lib.crt_batch_destroy(None) == 0


def test_sort_refuses_bad_sizes(lib):
    assert lib.crt_sort_pairs(None, None, None, None, 16, 0, None) == INVALID
    assert lib.crt_sort_pairs(None, None, None, None, 16, 33, None) == INVALID
    assert lib.crt_sort_pairs(None, None, None, None, -1, 30, None) == INVALID
    assert lib.crt_sort_pairs(None, None, None, None, 0, 30, None) == 0  # nothing to sort
    assert lib.crt_sort_pairs_noalloc(None, None, None, None, (1 << 20) + 1, 30, None) == INVALID


def test_batch_create_refuses_bad_counts(lib):
    import crt
    out = C.c_void_p()
    assert lib.crt_batch_create(None, None, 4, None, C.byref(out)) == INVALID
    d, keep = desc(n=1)
    descs = (crt._MeshDesc * 1025)(*([d] * 1025))
    views = (crt._BatchView * 1025)()
    assert lib.crt_batch_create(descs, views, 1025, None, C.byref(out)) == INVALID
    assert "1024" in error(lib)
    assert lib.crt_batch_create(descs, views, 0, None, C.byref(out)) == INVALID


def test_loader_and_writer_refuse_bad_arguments(lib, tmp_path):
    h = C.c_void_p()
    assert lib.crt_obj_load(None, None, C.byref(h)) == INVALID
    assert lib.crt_write_bmp(str(tmp_path / "x.bmp").encode(), 0, 4, None) == INVALID
    assert lib.crt_obj_free(None) == 0


def _big_desc(nv, nn, n=1):
    """A description whose counts exceed a limit while its arrays are small:
    the counts are refused before any array is read."""
    import crt
    keep = [np.zeros(9, np.float32), np.zeros(9, np.float32), np.zeros(3, np.int32), crt._Material()]
    d = crt._MeshDesc(keep[0].ctypes.data, nv, keep[1].ctypes.data, nn, keep[2].ctypes.data, None, n,
                      C.addressof(keep[3]), 1, None)
    return d, keep


def test_vertex_and_normal_counts_are_bounded(lib):
    """CRT_MAX_VERTICES keeps every 3 * index float offset within int32."""
    out = C.c_void_p()
    for nv, nn in (((1 << 29) + 1, 3), (3, (1 << 29) + 1)):
        d, keep = _big_desc(nv, nn)
        assert lib.crt_scene_create(C.byref(d), None, C.byref(out)) == INVALID
        assert "CRT_MAX_VERTICES" in error(lib)
        assert lib.crt_scene_create_borrowed(C.byref(d), None, C.byref(out)) == INVALID
    assert not out.value
    big = (1 << 29) + 1
    assert lib.crt_refit(None, big, None, 4, None, None, None, None) == INVALID
    assert lib.crt_morton(None, big, None, 4, None, None, None) == INVALID
    assert lib.crt_morton(None, 3, None, (1 << 28) + 1, None, None, None) == INVALID
    assert lib.crt_morton(None, 3, None, 0, None, None, None) == 0  # nothing to do


def test_batch_create_refuses_oversized_meshes_and_views(lib):
    """Per-mesh counts, running totals and view sizes are checked in 64-bit
    before the int32 offsets of the concatenated arrays are formed."""
    import crt
    out = C.c_void_p()

    def attempt(d, width=8, height=8, spp=1, m=1):
        views = (crt._BatchView * m)()
        for v in views:
            v.width, v.height, v.spp = width, height, spp
        descs = (crt._MeshDesc * m)(*([d] * m))
        return lib.crt_batch_create(descs, views, m, None, C.byref(out))

    d, keep = _big_desc((1 << 29) + 1, 3)
    assert attempt(d) == INVALID and "size is out of range" in error(lib)
    d, keep = _big_desc(3, 3)
    assert attempt(d, width=1 << 16, height=1 << 15) == INVALID and "size is out of range" in error(lib)
    assert attempt(d, spp=(1 << 24) + 1) == INVALID and "size is out of range" in error(lib)
    # each view fits, the total pixel count does not
    assert attempt(d, width=1 << 15, height=1 << 15, m=2) == INVALID and "batch mesh 1" in error(lib)
    # each mesh fits, the total vertex count does not
    d, keep = _big_desc(1 << 28, 3)
    assert attempt(d, m=3) == INVALID and "batch mesh 2" in error(lib)
    assert not out.value


def test_sort_refuses_overlapping_arrays(lib):
    """The sort does not work in place: pass 0 of a multi-pass sort writes an
    output while later tiles still read the input.  Overlapping ranges are
    refused before any CUDA call (these addresses are never dereferenced)."""
    base = 1 << 40
    n = 1000
    cases = [
        (base, None, base + 4 * (n - 1), base + 8 * n),  # keys_out starts inside keys_in
        (base, None, base + 8 * n, base + 4 * 10),  # vals_out inside keys_in
        (base, base + 8 * n, base + 16 * n, base + 8 * n + 4),  # vals_out inside vals_in
        (base, None, base + 8 * n, base + 8 * n + 4),  # the two outputs overlap
    ]
    for f in (lib.crt_sort_pairs, lib.crt_sort_pairs_noalloc):
        for kin, vin, kout, vout in cases:
            assert f(kin, vin, kout, vout, n, 30, None) == INVALID
            assert b"overlap" in lib.crt_last_error_string()
    # adjacent, non-overlapping ranges get past this check (and stop at the
    # device-pointer check: these are not device addresses)
    assert lib.crt_sort_pairs(base, None, base + 4 * n, base + 8 * n, n, 30, None) == INVALID
    assert b"overlap" not in lib.crt_last_error_string()

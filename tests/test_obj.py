"""Scene input and image output of the drop-in CLI, on the CPU: the library's
OBJ/MTL reader (crt_obj_load) gives the same arrays as the reader the golden
fixtures were made with (crt.data.load_obj), and crt_write_bmp writes the
reference's 24-bit BMP layout (src/bitmap.cpp:99-154)."""
import os
import struct

import numpy as np
import pytest

OBJ = """# a quad, a pentagon and loose triangles over two materials
mtllib scene.mtl
mtllib missing.mtl
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0.5 1.7 0.3
v -0.25 0.125 2.0000001
v 3.14159265358979 2.718281828 -1.41421356
vn 0 0 1
vn 0 1 0
vn 0.577 0.577 0.577
vt 0 0
usemtl red
f 1//1 2//1 3//1 4//1
usemtl nosuchmaterial
f 1/1/2 3/1/2 5/1/2
usemtl glass
f -1//-1 -2//-2 -3//-3 1//1 2//2
f 6//3 7//3 5//3
"""

MTL = """newmtl red
Ka 0.1 0.2 0.3
Kd 0.8 0.1 0.1
Ks 0.5 0.5 0.5
Ns 32
newmtl glass
Kd 0.2 0.3 0.4
Tf 0.9 0.9 0.9
Ke 0.01 0.02 0.03
Ni 1.45
"""


@pytest.fixture()
def scene_dir(tmp_path, built):
    (tmp_path / "scene.obj").write_text(OBJ)
    (tmp_path / "scene.mtl").write_text(MTL)
    return tmp_path


def test_native_reader_matches_python_reader(scene_dir):
    import crt
    from crt import data
    a = crt.load_obj_native(str(scene_dir / "scene.obj"))
    b = data.load_obj(str(scene_dir / "scene.obj"))
    for k in ("verts", "vidx", "normals", "nidx", "matid", "materials"):
        x, y = getattr(a, k), getattr(b, k)
        assert x.dtype == y.dtype and x.shape == y.shape, k
        assert np.array_equal(x, y), k
    assert a.ntri == 2 + 1 + 3 + 1            # quad, triangle, pentagon (fan), triangle
    assert list(a.matid) == [0, 0, 0, 1, 1, 1, 1]  # unknown material -> 0
    assert a.materials[0, 15] == 32.0 and a.materials[1, 15] == 1.0  # tinyobjloader's default Ns
    assert np.array_equal(a.materials[1, 9:12], [0.9, 0.9, 0.9])  # Tf is the transmittance


def test_obj_optics_take_ks_and_ni(scene_dir):
    """crt_obj_optics: kr = Ks (Scene_h::LoadObj's `mat.kr = specular`,
    src/scene.cpp:29) and ior = Ni, tinyobjloader's 1 where Ni is absent."""
    import crt
    mesh, optics = crt.load_obj_native(str(scene_dir / "scene.obj"), with_optics=True)
    assert optics.shape == (2, 4)
    assert np.array_equal(optics[:, :3], mesh.materials[:, 6:9])
    assert np.array_equal(optics[:, 3], [1.0, 1.45])


def test_native_reader_rejects_faces_without_normals(tmp_path, built):
    import crt
    (tmp_path / "bad.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    with pytest.raises(crt.CrtError, match="normal"):
        crt.load_obj_native(str(tmp_path / "bad.obj"))
    with pytest.raises(crt.CrtError, match="cannot open"):
        crt.load_obj_native(str(tmp_path / "absent.obj"))
    (tmp_path / "range.obj").write_text("v 0 0 0\nvn 0 0 1\nf 1//1 2//1 9//1\n")
    with pytest.raises(crt.CrtError, match="out of range"):
        crt.load_obj_native(str(tmp_path / "range.obj"))


def test_default_material_without_mtl(tmp_path, built):
    import crt
    (tmp_path / "plain.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n")
    m = crt.load_obj_native(str(tmp_path / "plain.obj"))
    assert m.materials.shape == (1, 16) and np.array_equal(m.materials[0, 3:6], [0.8, 0.8, 0.8])


def read_bmp(path):
    raw = open(path, "rb").read()
    assert raw[:2] == b"BM"
    size, off = struct.unpack_from("<I", raw, 2)[0], struct.unpack_from("<I", raw, 10)[0]
    hsize, w, h, planes, bpp, comp = struct.unpack_from("<IiiHHI", raw, 14)
    assert (size, off, hsize, planes, bpp, comp) == (len(raw), 54, 40, 1, 24, 0)
    row = w * 3 + (-(w * 3) % 4)
    px = np.frombuffer(raw[off:], np.uint8).reshape(h, row)[:, :w * 3].reshape(h, w, 3)
    return px[..., ::-1].reshape(-1, 3)  # BGR -> RGB, rows in file order (bottom-up)


@pytest.mark.parametrize("w,h", [(5, 3), (8, 2), (1, 1)])
def test_bmp_layout(tmp_path, built, w, h):
    import crt
    rgb = np.random.default_rng(w * h).integers(0, 256, (w * h, 3), dtype=np.uint8)
    path = str(tmp_path / "img.bmp")
    crt.write_bmp(path, rgb, w, h)
    assert os.path.getsize(path) == 54 + h * (w * 3 + (-(w * 3) % 4))
    assert np.array_equal(read_bmp(path), rgb)


def _load_chunked(path, chunk, monkeypatch):
    import crt
    monkeypatch.setenv("CRT_OBJ_CHUNK_BYTES", str(chunk))
    return crt.load_obj_native(str(path), with_optics=True)


def test_reader_result_does_not_depend_on_chunks(tmp_path, built, monkeypatch):
    """The reader parses chunks of lines on all host cores; relative indices,
    mtllib and usemtl lines, CRLF endings and a last line without a newline
    read the same whatever the chunk boundaries (1 byte: every line its own
    chunk)."""
    (tmp_path / "scene.mtl").write_text(MTL)
    (tmp_path / "late.mtl").write_text("newmtl late\nKd 0.1 0.9 0.1\nKs 0.3 0.3 0.3\nNi 1.2\n")
    rng = np.random.default_rng(4)
    lines = ["mtllib scene.mtl"]
    nv = 0
    for block in range(40):
        for _ in range(6):
            lines.append("v %.7g %.7g %.7g" % tuple(rng.normal(size=3)))
            lines.append("vn %.7g %.7g %.7g" % tuple(rng.normal(size=3)))
            nv += 1
        if block == 11:
            lines.append("usemtl red")
        if block == 19:
            lines.append("mtllib late.mtl\r")
            lines.append("usemtl late")
        if block == 27:
            lines.append("usemtl")
        if block == 33:
            lines.append("usemtl glass")
        lines.append("# block %d" % block)
        lines.append("")
        k = int(rng.integers(3, 7))
        corners = ["%d//%d" % (-(j + 1), -(j + 1)) for j in range(k)]       # relative to this line
        lines.append("f " + " ".join(corners) + ("\r" if block % 3 == 0 else ""))
        i = int(rng.integers(1, nv + 1))
        lines.append("f %d//%d %d//%d %d//%d" % (i, i, nv, nv, 1, 1))
    text = "\n".join(lines)                                                     # no final newline
    (tmp_path / "c.obj").write_text(text)
    ref, ref_opt = _load_chunked(tmp_path / "c.obj", 1 << 30, monkeypatch)    # one chunk
    assert ref.ntri > 100 and set(ref.matid.tolist()) == {0, 1, 2}
    assert ref_opt.shape == (3, 4) and ref_opt[2, 3] == 1.2
    for chunk in (1, 5, 37, 300, 4096):
        got, opt = _load_chunked(tmp_path / "c.obj", chunk, monkeypatch)
        for k in ("verts", "vidx", "normals", "nidx", "matid", "materials"):
            assert np.array_equal(getattr(got, k), getattr(ref, k)), (chunk, k)
        assert np.array_equal(opt, ref_opt), chunk


@pytest.mark.parametrize("chunk", [1, 16, 1 << 30])
def test_reader_reports_the_first_error_in_file_order(tmp_path, built, monkeypatch, chunk):
    import crt
    body = ["v 0 0 0", "v 1 0 0", "v 0 1 0", "vn 0 0 1"] + ["f 1//1 2//1 3//1"] * 30
    body[20] = "f 1//1 2//1 x//1"        # line 21: a bad corner
    body[30] = "v 1 2"                   # line 31: a bad vertex, later in the file
    (tmp_path / "e.obj").write_text("\n".join(body) + "\n")
    monkeypatch.setenv("CRT_OBJ_CHUNK_BYTES", str(chunk))
    with pytest.raises(crt.CrtError, match="bad face corner at line 21$"):
        crt.load_obj_native(str(tmp_path / "e.obj"))
    (tmp_path / "big.obj").write_text("v 0 0 0\nvn 0 0 1\nf 1//1 1//1 4294967297//1\n")
    with pytest.raises(crt.CrtError, match="bad face corner at line 3"):
        crt.load_obj_native(str(tmp_path / "big.obj"))

"""Generate recorded/logcabin.npz: the reference's one end-to-end result that
can be re-run from its checkout.

The reference ships results/logcabin.bmp, rendered by its cuda_bvh on a
Kepler GPU with the flags of runLogcabin.sh (-f 16 -v 35 -P 15
-a 0.0001,0.0001,0.01 -p -4,2,-4 -w 1024 -h 1024 -R 0.5), from
objs/funyz/logcabin.obj and .mtl.  This stores that scene (read with
tinyobjloader's conventions, crt.data.load_obj), the flag values as the
reference's main.cpp parses them (vectors through stof, scalars through
stod) and the recorded image's pixels in the reference's bottom-up order.
It sits in its own folder: the fixtures beside this script all hold the
build, trace and image dumps that the parity tests iterate over.  The GPU
box has no reference checkout; this file travels instead.

Run (in a container with the reference checkout):
    python tests/golden/make_logcabin.py
"""
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "cuda-rt_gb300"))

from crt import data  # noqa: E402

sys.path.insert(0, ROOT)
from oracle.ref.build_ref import default_reference  # noqa: E402

REF = default_reference()


def read_recorded_bmp(path):
    """Pixels of a 24-bit BMP as written by the reference's writeBMP (whose
    bfSize field is 2 more than the file: it adds sizeof of its padded
    16-byte file-header struct), bottom-up rows, RGB."""
    raw = open(path, "rb").read()
    off = struct.unpack_from("<I", raw, 10)[0]
    _, w, h, _, bpp, comp = struct.unpack_from("<IiiHHI", raw, 14)
    assert bpp == 24 and comp == 0
    row = w * 3 + (-(w * 3) % 4)
    px = np.frombuffer(raw[off:off + row * h], np.uint8).reshape(h, row)[:, :w * 3].reshape(h, w, 3)
    return w, h, np.ascontiguousarray(px[..., ::-1].reshape(-1, 3))


def main():
    mesh = data.load_obj(os.path.join(REF, "objs", "funyz", "logcabin.obj"))
    w, h, rgb = read_recorded_bmp(os.path.join(REF, "results", "logcabin.bmp"))
    f = lambda *x: np.array([float(np.float32(v)) for v in x])  # noqa: E731  (stof)
    np.savez_compressed(
        os.path.join(HERE, "recorded", "logcabin.npz"), verts=mesh.verts, normals=mesh.normals, vidx=mesh.vidx,
        nidx=mesh.nidx, matid=mesh.matid, materials=mesh.materials, width=w, height=h, recorded_rgb=rgb,
        fov=35.0, fstop=16.0, focal_point=15.0, light_position=f(-4.0, 2.0, -4.0), light_color=f(1.0, 1.0, 1.0),
        light_radius=0.5, attenuation=f(0.0001, 0.0001, 0.01))
    print("recorded/logcabin.npz:", mesh.ntri, "triangles,", w, "x", h)


if __name__ == "__main__":
    main()

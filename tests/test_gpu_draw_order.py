"""The order of an area light's three draws (randVec3d, kernels/mrand.cu:
33-35, consumed by Light::getDirection, kernels/Light.cu:71-74).  The
reference builds a Vec3d from three randDouble calls whose evaluation order
C++ leaves to the compiler; the reference runs on the GPU, so its order is
the one nvcc gives that form.  The probe compiles the same form with the
library's flags and reports which component each draw lands in on the
device and on the host; the pixel kernels take the device order
(crt.LIGHT_DRAW_ORDER), and an area-light render equals the oracle's with
that order set."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import assert_equal

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _probe(tmp_path):
    from crt import build
    exe = str(tmp_path / "draw_order_probe")
    subprocess.check_call([build.nvcc(), *build.ARCH, "-O3", "-fmad=false",
                           os.path.join(HERE, "probes", "draw_order_probe.cu"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    dev = tuple(int(x) for x in re.search(r"device order: (\d) (\d) (\d)", r.stdout).groups())
    host = tuple(int(x) for x in re.search(r"host order: (\d) (\d) (\d)", r.stdout).groups())
    return dev, host


def test_kernels_take_nvcc_draw_order(cuda, tmp_path):
    import crt
    from crt import data
    from oracle.oracle import OracleScene
    dev, host = _probe(tmp_path)
    print(f"randVec3d draw order: device {dev}, host {host}")
    assert dev == crt.LIGHT_DRAW_ORDER, f"nvcc evaluates the draws in order {dev}"
    sc = data.config0(n=5000, width=64, height=48)
    light = data.Light(position=sc.light.position, radius=0.6)
    g = crt.Scene(sc.mesh).render(sc.camera, light, 64, 48, 6, aux=True)
    o = OracleScene(sc.mesh)
    assert o.lib.orc_set_light_draw_order(*dev) == 0
    try:
        r = o.render(sc.camera, light, 64, 48, spp=6, aux=True)
    finally:
        o.lib.orc_set_light_draw_order(*crt.LIGHT_DRAW_ORDER)
    assert_equal(g["shadow"], r["shadow"], "shadow")
    assert_equal(g["rgb8"], r["rgb"], "rgb8")
    assert np.array_equal(g["hit_id"], r["hit_id"])

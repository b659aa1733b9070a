"""The pixel kernel takes the thin-lens offset from sincos; the reference
calls cos and sin.  This compiles a probe with the library's flags and checks
that both give the same bits for every angle the mrand draw can produce."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_sincos_equals_sin_and_cos_for_every_lens_angle(cuda, tmp_path):
    from crt import build
    exe = str(tmp_path / "sincos_probe")
    subprocess.check_call([build.nvcc(), *build.ARCH, "-O3", "-fmad=false", os.path.join(HERE, "probes",
                                                                                          "sincos_probe.cu"),
                           "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "83886081 angles, 0 mismatches" in r.stdout, r.stdout

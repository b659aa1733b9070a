"""The command-line renderer's argument handling, on the CPU: every check
below runs before the CLI touches the GPU (usage, option and value errors,
the OBJ reader's errors), so it needs no device.  The renders themselves are
in test_gpu_cli.py."""
import subprocess

import pytest


@pytest.fixture(scope="module")
def cli(built):
    from crt import build
    return build.build_cli()


def run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=60)


def test_usage(cli):
    for args in ((), ("--help",)):
        r = run(cli, *args)
        assert r.returncode == 0 and "USAGE" in r.stdout, args


@pytest.mark.parametrize("args,message", [
    (("--bogus",), "bad option"),
    (("-x", "1"), "bad option"),
    (("-i",), "bad option"),                            # an option that needs a value, at the end
    (("-w", "zero"), "bad value"),
    (("-w", "0"), "bad value"),
    (("--height=-4",), "bad value"),
    (("--spp", "40000"), "bad value"),                  # above 2^15
    (("--depth", "9"), "bad value"),                    # above CRT_MAX_DEPTH
    (("--depth", "2x"), "bad value"),
    (("--seed", "-1"), "bad value"),
    (("--seed", "4294967296"), "bad value"),
    (("-p", "1,2"), "bad value"),                       # a vector needs three components
    (("-c", "1,,3"), "bad value"),
    (("-a", "a,b,c"), "bad value"),
    (("-f", "none"), "bad value"),
    (("-o", "x.bmp"), "input OBJ"),                     # -i is required
])
def test_rejected_arguments(cli, args, message):
    r = run(cli, *args)
    assert r.returncode == 1 and message in r.stderr, (args, r.stderr)


def test_reader_errors_come_before_the_device(cli, tmp_path):
    r = run(cli, "-i", str(tmp_path / "absent.obj"))
    assert r.returncode == 1 and "cannot open" in r.stderr
    (tmp_path / "nonormals.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    r = run(cli, "-i", str(tmp_path / "nonormals.obj"))
    assert r.returncode == 1 and "normal" in r.stderr
    (tmp_path / "bad.obj").write_text("v 0 0 0\nvn 0 0 1\nf 1//1 1//1 7//1\n")
    r = run(cli, "--input=" + str(tmp_path / "bad.obj"), "--spp=4", "-d", "0,-1,-1", "-n", "1", "-1", "1")
    assert r.returncode == 1 and "out of range" in r.stderr

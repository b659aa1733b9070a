"""bench.py's reference arm (CPU only: it times the reference's algorithm on
the host cores) prints the contract's JSON line, and the launch count the
GPU arm claims follows the build's kernels."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["unit"] == "Mrays/s" and line["steps"] == 1 and line["n_gpus"] == 1
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["value"] == line["value"] and cb["cores"] >= 1 and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_build_launch_count():
    import bench
    assert bench.build_launches(0) == 0
    assert bench.build_launches(1) == 7          # init, bounds, Morton, 3 look-back sort passes, refit
    assert bench.build_launches(512) == 8        # + split search; one refit block: no spanning-node pass
    assert bench.build_launches(513) == 9        # + the spanning-node pass
    assert bench.build_launches(1003520) == 7    # cooperative sort (123 tiles of 8192): one launch for 3 passes
    assert bench.build_launches(152 * 8192 + 1) == 9  # too many tiles to be resident: three look-back passes

import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "cuda-rt_gb300"))
sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def golden_mesh(z):
    from crt import data
    return data.Mesh(z["verts"], z["vidx"], z["normals"], z["nidx"], z["matid"], z["materials"])


def golden_camera_light(z):
    from crt import data
    c, L = z["camera"], z["light"]
    cam = data.Camera(fov=float(c[0]), focal_point=float(c[1]), fstop=float(c[2]), eye=tuple(c[3:6]))
    light = data.Light(position=tuple(L[0:3]), color=tuple(L[3:6]), radius=float(L[6]), constant_term=float(L[7]),
                       linear_term=float(L[8]), quadratic_term=float(L[9]))
    return cam, light


@pytest.fixture(scope="session")
def built():
    """Build libcrt.so and the oracle once per session."""
    import __graft_entry__
    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def cuda(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch


def assert_equal(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    bad = np.flatnonzero((a != b).reshape(len(a), -1).any(1)) if a.ndim else []
    assert len(bad) == 0, f"{what}: {len(bad)} mismatches, first at {bad[:5]}: {a[bad[:3]]} vs {b[bad[:3]]}"

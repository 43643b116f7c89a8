import json
import pathlib
import sys

import numpy as np
import pytest

REPO = pathlib.Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        have_gpu = torch.cuda.is_available()
    except Exception:
        have_gpu = False
    if have_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def pins():
    return np.load(GOLDEN / "ref_pins.npz")


@pytest.fixture(scope="session")
def ref_images():
    return np.load(GOLDEN / "ref_images.npz")


@pytest.fixture(scope="session")
def meta():
    return json.loads((GOLDEN / "ref_meta.json").read_text())


def lens_from_pins(pins, name):
    from ghostlight_gb300._abi import gl_surface
    raw = pins[name + "/lens"]
    n = raw.shape[0]
    arr = (gl_surface * n).from_buffer_copy(raw.tobytes())
    return list(arr)


LENS_NAMES = ["cfg1_double_gauss_12", "cfg2_wide_angle_24", "cfg4_anamorphic_18",
              "ref_DoubleGauss", "ref_hex_stop"]


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

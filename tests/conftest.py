import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path)")


def golden_cart_names():
    return sorted(os.path.basename(p)[5:-4] for p in glob.glob(os.path.join(GOLDEN, "cart_*.npz")))


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, f"cart_{name}.npz"))
    out = {k: d[k] for k in d.files}
    out["case"] = json.loads(str(out["case"]))
    return out


@pytest.fixture(scope="session")
def port_lib():
    from oracle import oracle
    oracle.build_port()
    return oracle.port_lib()

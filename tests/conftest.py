import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def golden_cases():
    import numpy as np

    d = os.path.join(ROOT, "tests", "golden")
    out = {}
    for f in sorted(os.listdir(d)):
        # the clipping cases (dist2mat_ref.npz holds another kernel's vectors)
        if f.endswith(".npz") and not f.endswith("_topo.npz") and not f.startswith("dist2mat"):
            out[f[:-4]] = dict(np.load(os.path.join(d, f)))
    # the reference's per-cell topology of each case's cells
    for name, case in out.items():
        t = os.path.join(d, name + "_topo.npz")
        if os.path.exists(t):
            case.update(dict(np.load(t)))
    return out

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built CUDA library")


GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_GRAPHS = ("grid12", "rgg", "chunglu")


def read_initf(path):
    import numpy as np
    return np.array([[float(a) for a in line.split()[:2]] for line in open(path)])


def load_golden(name):
    import numpy as np
    z = dict(np.load(os.path.join(GOLDEN, f"ref_{name}.npz")))
    z["init_xy"] = read_initf(os.path.join(GOLDEN, f"{name}.initf"))
    return z

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "kimera-rpgo_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def load_robot(name: str):
    from rpgo_gb300.graph import graph_from_g2o_arrays

    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return graph_from_g2o_arrays(z["vertex_keys"], z["vertex_vals"], z["edge_keys"], z["edge_vals"])


@pytest.fixture
def robot_a():
    return load_robot("robot_a")


@pytest.fixture
def robot_b():
    return load_robot("robot_b")

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a path)")


@pytest.fixture(scope="session")
def lib():
    """The in-tree native library, built on first use."""
    from maple3dmt_gb300 import _loader, build
    build.build_library()
    return _loader.load()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build_oracle()
    return oracle


def load_golden(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return d


@pytest.fixture(scope="session")
def golden_small():
    return load_golden("small_block")


@pytest.fixture(scope="session")
def golden_c1():
    return load_golden("halfspace_c1")


def leaves_from_golden(g):
    from maple3dmt_gb300.mesh import Leaves
    n = g["level"].shape[0]
    return Leaves(tuple(g["domain"]), int(g["min_level"]), int(g["max_level"]),
                  np.ascontiguousarray(g["level"], np.int32), np.zeros((n, 3), np.int32),
                  np.ascontiguousarray(g["cx"]), np.ascontiguousarray(g["cy"]),
                  np.ascontiguousarray(g["cz"]), np.ascontiguousarray(g["cell_type"], np.int32))


def rel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))

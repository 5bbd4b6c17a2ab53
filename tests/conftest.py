"""Shared pytest configuration: the ``gpu`` marker and fixture loaders."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name))


def unpack_sparse(d, name):
    """Dense compact array from the sparse (shape, idx, val) triple of a fixture."""
    shape = tuple(int(s) for s in d[f"{name}_shape"])
    out = np.zeros(int(np.prod(shape)), dtype=np.complex128)
    out[d[f"{name}_idx"]] = d[f"{name}_val"]
    return out.reshape(shape)


@pytest.fixture(scope="session")
def golden_hydro():
    return load_golden("reference_hydro.npz")


@pytest.fixture(scope="session")
def golden_cupy():
    return load_golden("reference_cupy.npz")


@pytest.fixture(scope="session")
def golden_tg64():
    return load_golden("reference_tg64.npz")


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))

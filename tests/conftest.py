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


# ---------------------------------------------------------------- GPU-side helpers
def full_to_compact(full, N):
    """Full complex fftn layout (C, N, N, N) -> compact Fourier coefficients (C, M, M, K+1)."""
    from oracle import tg_numpy as T
    K = T.dealias_cutoff(N)
    idx = T.kept_indices(N)
    return np.asarray(full)[:, idx][:, :, idx][:, :, :, : K + 1] / float(N) ** 3


def to_state(plan, c, batch_index=None):
    """Compact numpy coefficients (C, M, M, K+1) or (B, C, M, M, K+1) -> padded plan state."""
    import torch
    c = np.asarray(c)
    if c.ndim == 4:
        c = c[None]
    s = np.zeros(plan.state_shape, dtype=np.complex128)
    s[..., : c.shape[-1]] = c
    return torch.from_numpy(s).to(plan.complex_dtype).to(plan.device).contiguous()


def from_state(plan, s):
    """Plan state -> numpy (B, C, M, M, K+1) complex128 (padding dropped)."""
    return s[..., : plan.K + 1].to("cpu").numpy().astype(np.complex128)


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # noqa: BLE001
        return False

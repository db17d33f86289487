"""Shared test setup: markers, paths, seeded coefficient generators."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def degrees_so3(l_max):
    return np.concatenate([np.full((2 * l + 1) ** 2, l) for l in range(l_max + 1)])


def degrees_s2(l_max):
    return np.concatenate([np.full(2 * l + 1, l) for l in range(l_max + 1)])


def so3_coeffs(l_max, seed=0, complex_=True, decay="inv"):
    """Seeded F^l_mn ~ N(0,1)/(2l+1) (decay='inv') or N(0,1)(l+1)^-1.5 (decay='pow')."""
    rng = np.random.Generator(np.random.PCG64(seed))
    l = degrees_so3(l_max)
    s = 1.0 / (2 * l + 1) if decay == "inv" else (l + 1.0) ** -1.5
    re = rng.standard_normal(l.size) * s
    if not complex_:
        return re
    return re + 1j * rng.standard_normal(l.size) * s


def s2_coeffs(l_max, seed=0, complex_=True):
    rng = np.random.Generator(np.random.PCG64(seed))
    l = degrees_s2(l_max)
    re = rng.standard_normal(l.size) / (l + 1.0)
    if not complex_:
        return re
    return re + 1j * rng.standard_normal(l.size) / (l + 1.0)


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gblib():
    """The CUDA library, built in-tree for sm_103a."""
    from fftso3_gb300 import build as b
    b.build()
    from fftso3_gb300 import _lib
    return _lib


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False

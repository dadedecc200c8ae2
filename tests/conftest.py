"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; everything else
runs on the CPU (oracle, host logic, library load / symbol checks)."""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np
import pytest

REPO = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    """The CPU FP64 oracle (test infrastructure)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    from oracle_py import Oracle  # noqa: E402
    return Oracle


@pytest.fixture(scope="session")
def capi():
    from cuda_sto_pf_gb300 import build, capi as c
    build.build()
    c.load()
    return c


def params_for(capi, name="c2.params", n=32, **over):
    p = capi.load_params_file(os.path.join(GOLDEN, name))
    p.Nx = p.Ny = p.Nz = n
    for k, v in over.items():
        if isinstance(getattr(p, k), ctypes.Array):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, k, v)
    capi.finalize(p)
    return p


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))

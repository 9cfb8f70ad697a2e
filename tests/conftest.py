"""Shared test configuration: the ``gpu`` marker and fixture loaders."""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


def load_case(name: str) -> dict:
    with np.load(GOLDEN / f"ref_{name}.npz") as z:
        return {k: z[k] for k in z.files}


def csr_from(d: dict, prefix: str):
    from scipy import sparse

    n = len(d[f"{prefix}_indptr"]) - 1
    return sparse.csc_matrix((d[f"{prefix}_data"], d[f"{prefix}_indices"], d[f"{prefix}_indptr"]), shape=(n, n))


CASES = ["square", "cubetria", "ico3", "deformed3", "kuhn5"]


@pytest.fixture(scope="session")
def cuda_ok():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lapy_gb300 import _lib

    _lib.lib()
    return True

"""Shared pytest setup: the `gpu` marker, the repo on sys.path, and helpers."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libccgpu.so")


@pytest.fixture(scope="session")
def built():
    """Build the native libraries in-tree once per session."""
    import __graft_entry__ as ge
    ge.build()
    return True


@pytest.fixture(scope="session")
def cuda(built):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")


def csr_from_rows(rows, id_bytes=4, num_parts=1):
    """StaticGraph from explicit adjacency rows (kept as given: self-loops and
    duplicate entries stay)."""
    from components_gb300 import StaticGraph
    rp = np.zeros(len(rows) + 1, np.uint64)
    for i, r in enumerate(rows):
        rp[i + 1] = rp[i] + len(r)
    col = np.array([w for r in rows for w in r], np.uint32 if id_bytes == 4 else np.uint64)
    return StaticGraph(rp, col, num_parts)

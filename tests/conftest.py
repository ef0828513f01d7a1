"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on a CPU-only host."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    """Builds (incrementally) and loads libnanogi.so."""
    from nanogi_gb300.build import build_library

    build_library()
    import nanogi_gb300 as ng

    return ng.load_library()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle.oracle import lib

    return lib()


@pytest.fixture(scope="session")
def cornell(tmp_path_factory):
    """The Cornell-box workload on disk plus its in-memory description."""
    from nanogi_gb300 import scenegen

    desc = scenegen.cornell_box()
    d = tmp_path_factory.mktemp("cornell")
    path = scenegen.write_scene(desc, d)
    return desc, path


def rel_rmse(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.sqrt(((a - b) ** 2).sum() / max((b ** 2).sum(), 1e-300)))

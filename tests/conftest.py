import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "graph-utils_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def pytest_collection_modifyitems(config, items):
    # keep tests/test_zz_* last even when selected by marker
    items.sort(key=lambda it: os.path.basename(str(it.fspath)).startswith("test_zz_"))


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle once per session (incremental)."""
    import build as gu_build  # graph-utils_gb300/build.py
    gu_build.build_library()
    gu_build.build_oracle()


def golden_names(prefix="graph_"):
    return sorted(os.path.basename(p)[len(prefix):-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def load_golden(name, prefix="graph_"):
    return dict(np.load(os.path.join(GOLDEN, f"{prefix}{name}.npz")))


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False

import contextlib
import os
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(GOLDEN / name, allow_pickle=False)
    return load


@pytest.fixture(scope="session")
def gpu_ctx():
    from graada3d_gb300 import Context
    ctx = Context(0)
    yield ctx
    ctx.close()


@contextlib.contextmanager
def cg_path(mode: str):
    """Selects the CG loop inside the block: "1" the persistent launch for every
    stored G, "0" the graph-replayed iteration (GRADA_CG_FUSED)."""
    old = os.environ.get("GRADA_CG_FUSED")
    os.environ["GRADA_CG_FUSED"] = mode
    try:
        yield
    finally:
        if old is None:
            os.environ.pop("GRADA_CG_FUSED", None)
        else:
            os.environ["GRADA_CG_FUSED"] = old

import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


@pytest.fixture(scope="session")
def oracle_lib():
    """The oracle's C restatement (built in place if missing)."""
    import oracle

    if not os.path.exists(oracle._PORT_SO):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j4"], check=True,
                       stdout=subprocess.DEVNULL)
    return oracle


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


def golden_matrix(g, name):
    from combblas_gb300.generators import CSC

    shape = g[f"in/{name}/shape"]
    vals = g[f"in/{name}/values"] if f"in/{name}/values" in g.files else None
    return CSC(int(shape[0]), int(shape[1]), g[f"in/{name}/colptr"], g[f"in/{name}/rowidx"], vals)


@pytest.fixture(scope="session")
def gpu_ctx():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from combblas_gb300 import local

    return local.default_context(0)

import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def emfa_lib():
    """Build (if stale) and load libemfa_cuda.so -- no GPU needed to load."""
    from emfa_gb300 import build
    build.build()
    from emfa_gb300 import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx(emfa_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from emfa_gb300 import api
    c = api.Context(0)
    yield c
    c.close()


def load_golden(name):
    import numpy as np
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))
    import ast
    d["meta"] = ast.literal_eval(str(d["meta"]))
    return d

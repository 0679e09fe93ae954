import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402
from oracle import oracle as oracle_mod  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libbhgpu kernels)")


def _ensure_built():
    pkg = __graft_entry__.PKG
    if not os.path.exists(os.path.join(pkg, "libbhgpu.so")) or not os.path.exists(oracle_mod.RESTATEMENT_LIB):
        __graft_entry__.build()


@pytest.fixture(scope="session")
def bh():
    _ensure_built()
    mod = __graft_entry__.package()
    mod.load()
    return mod


@pytest.fixture(scope="session")
def orc():
    _ensure_built()
    return oracle_mod.Restatement()


@pytest.fixture(scope="session")
def ref():
    if not os.path.exists(oracle_mod.REF_LIB):
        from oracle import build_oracle

        if build_oracle.build_ref() is None:
            pytest.skip("reference checkout not available: REF-LITERAL cannot be built here")
    return oracle_mod.RefLiteral()


def golden(name):
    return np.load(os.path.join(GOLDEN, name))

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libugpu.so")


@pytest.fixture(scope="session")
def ctx():
    """A device context on cuda:0 (builds libugpu.so in-tree first if it is missing)."""
    from utopia_gb300 import _abi, build

    if not os.path.exists(_abi.LIB_PATH):
        build.build()
    import utopia_gb300 as U

    c = U.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


def load_golden_mat(npz, prefix):
    from utopia_gb300.problems import CSR

    shape = npz[prefix + "_shape"]
    return CSR(int(shape[0]), int(shape[1]), npz[prefix + "_rowptr"], npz[prefix + "_colidx"], npz[prefix + "_values"])


@pytest.fixture(scope="session")
def laplace_hierarchy():
    """The reference's 4-level 2D fixture (utopia/data/laplace/matrices_for_petsc)."""
    d = np.load(os.path.join(GOLDEN, "laplace_hierarchy.npz"))
    A = load_golden_mat(d, "A")
    Is = [load_golden_mat(d, f"I{k}") for k in (1, 2, 3)]
    return A, Is, d["rhs"].copy()


@pytest.fixture(scope="session")
def mg_two_level():
    d = np.load(os.path.join(GOLDEN, "mg_two_level.npz"))
    return load_golden_mat(d, "A"), [load_golden_mat(d, "I")], d["rhs"].copy()

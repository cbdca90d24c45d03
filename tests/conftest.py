import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and liboofem_gb300.so")


def load_golden(name: str) -> dict:
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


# LinearStatic goldens solved with the direct solver (the _ic / _ilu / _void cases are
# CG runs to 1e-10 and have tests of their own)
LINEAR_CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                      if "mises" not in p and "idm" not in p and not p.endswith(("_ic.npz", "_ilu.npz", "_void.npz")))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def native_lib():
    from oofem_gb300 import build, native
    build.build()
    return native

import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pagerank-cuda-dynamic_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# The reference's checkout, for the CPU tests that compile against its
# headers (PRX_REFERENCE_DIR, else where it is mounted beside this checkout
# for tests); those tests skip where it is absent.
REFERENCE_DIR = os.environ.get("PRX_REFERENCE_DIR") or "/root/reference"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases():
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def ctx():
    import pagerank_gb300 as pg
    c = pg.Context(0)
    yield c
    c.close()

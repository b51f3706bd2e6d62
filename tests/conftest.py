import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native():
    """The native library, built in-tree (incremental) and loaded."""
    from dist_mem_gapbs_gb300 import _build
    _build.build()
    from dist_mem_gapbs_gb300 import gbbfs
    gbbfs.lib()
    return gbbfs


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_small():
    return dict(np.load(os.path.join(GOLDEN_DIR, "golden_small.npz")))


def config_args(flags):
    """(scale, degree, uniform) of a -u/-g/-k flag list."""
    scale, degree, uniform = None, 16, False
    it = iter(flags)
    for f in it:
        if f == "-u":
            scale, uniform = int(next(it)), True
        elif f == "-g":
            scale = int(next(it))
        elif f == "-k":
            degree = int(next(it))
    return scale, degree, uniform

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


def _batch_keys(native, off, nbr, g):
    """The batching key of every vertex (gbbfs_msbfs_order), restated: depth
    from the highest-degree vertex (lowest id among ties; 255 = unreached),
    then 255 - the quarter-octave of the sum of the neighbours' degrees (over
    the first 256 neighbours, scaled by deg // 256, for larger degrees)."""
    deg = np.diff(off).astype(np.int64)
    hd = native.DOBFS(g, int(np.argmax(deg)), depth=True)[1]
    hd = np.where(hd < 0, 255, np.minimum(hd, 254)).astype(np.int64)
    take = np.minimum(deg, 256)
    csum = np.concatenate([[0], np.cumsum(deg[nbr])])
    s = csum[off[:-1] + take] - csum[off[:-1]]
    big = deg > take
    s[big] = s[big] * deg[big] // take[big]
    q = np.zeros(len(deg), np.int64)
    for v in np.nonzero(s)[0]:
        t = int(s[v]) << 2
        b = t.bit_length()
        q[v] = min(255, 4 * b + ((t >> (b - 3)) & 3))
    return (hd << 8) | (255 - q)


@pytest.fixture(scope="session")
def batch_keys():
    return _batch_keys

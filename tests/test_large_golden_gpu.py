"""Parity on the measured configurations: Kronecker-22, -24 and -26 and
uniform-26 (degree 16), each with the reference's 64 SourcePicker sources.

tests/golden/golden_large.json holds what the reference itself produced for
them (gapbs-verify's Builder, SourcePicker and DOBFS, compiled from source,
driven by oracle/ref_driver.cc in its fixture mode): the SHA-256 of the CSR
offsets and neighbours, the source sequence, and per source the DOBFS step
trace, the reached count and degree sum, and the SHA-256 of the depth array
its parent tree implies.

Here the graph is rebuilt through the product (the host generator, then the
CSR built in HBM by gbbfs_graph_create_from_edges, as the benchmark builds
it) and every source is searched through the C ABI.  Depths must hash to the
reference's, the step trace must equal the reference's line for line, and
the parent tree must be consistent with the depths (every parent one level
up).  The edge check of the full verifier runs on the smallest graph, where
the serial verifier is quick."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, config_args

pytestmark = pytest.mark.gpu

LARGE = ["g22", "g24", "u26", "g26"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def golden_large():
    with open(os.path.join(GOLDEN_DIR, "golden_large.json")) as f:
        return json.load(f)


def tree_matches_depth(parent, depth, source):
    """parent[source] == source, unreached <=> parent -1, and every other
    reached vertex's parent sits one level above it."""
    if parent[source] != source or depth[source] != 0:
        return False
    reached = depth >= 0
    if not np.array_equal(reached, parent >= 0):
        return False
    v = np.nonzero(reached)[0]
    v = v[v != source]
    return bool(np.all(depth[parent[v]] == depth[v] - 1))


@pytest.mark.parametrize("name", LARGE)
def test_reference_fixture(native, oracle, golden_large, name):
    gd = golden_large[name]
    scale, degree, uniform = config_args(gd["flags"])
    el = native.generate_edges(scale, degree, uniform)
    g = native.Graph.from_edges(el)
    del el
    try:
        assert g.n == gd["num_nodes"] and g.m == gd["num_edges_directed"]
        off, nbr = g.csr()
        assert sha(off) == gd["offsets_sha256"]
        assert sha(nbr) == gd["neigh_sha256"]
        if name != "g22":
            del nbr                       # 8.4 GB of host memory at scale 26
        assert [int(s) for s in native.pick_sources(off, len(gd["sources"]))] == gd["sources"]
        deg = np.diff(off)
        parent = np.empty(g.n, np.int32)
        depth = np.empty(g.n, np.int32)
        for i, t in enumerate(gd["trials"]):
            src = t["source"]
            _, _, st = native.DOBFS(g, src, depth=True, stats=True, parent_out=parent,
                                    depth_out=depth)
            assert [list(x) for x in st.trace] == t["trace"], (name, src)
            assert sha(depth) == t["depth_sha256"], (name, src)
            assert int(depth.max()) == t["max_depth"]
            assert st.reached == t["reached"]
            assert int(deg[parent >= 0].sum()) == t["reached_degree_sum"]
            assert tree_matches_depth(parent, depth, src), (name, src)
            if name == "g22" and i < 4:
                ok, why = oracle.verify(off, nbr, src, parent)
                assert ok, why
    finally:
        g.close()

"""Pins to fixtures the reference itself produced (no GPU needed).

* Graph files: every file under tests/golden/io/ (edge lists, DIMACS, METIS,
  Matrix Market, a serialized graph) read by gbbfs_read_graph gives the CSR
  the reference's Reader + Builder built from it (golden_io.json, recorded by
  tests/golden/make_golden.py --io through the reference's own
  Builder::MakeGraph with -f).
* BC's BFS phase: the oracle's serial restatement (orc_bc_bfs) gives, for
  every recorded source, the depths, path counts, successor bits and level
  sizes of the reference's PBFS (golden_bc.json, gapbs-verify/bc.cc:51-92).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, config_args

IO_DIR = os.path.join(GOLDEN_DIR, "io")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _load(name):
    with open(os.path.join(GOLDEN_DIR, name)) as f:
        return json.load(f)


IO = _load("golden_io.json")
BC = _load("golden_bc.json")


@pytest.mark.parametrize("name", sorted(IO))
def test_reader_matches_reference(native, name):
    gd = IO[name]
    off, nbr = native.make_graph(filename=os.path.join(IO_DIR, name),
                                 symmetrize=gd["symmetrize"])
    assert len(off) - 1 == gd["num_nodes"] and len(nbr) == gd["num_edges_directed"]
    assert sha(off) == gd["offsets_sha256"]
    assert sha(nbr) == gd["neigh_sha256"]


def test_serialized_graph_is_the_generated_one(native, golden):
    """The .sg fixture was written by this library from the Kronecker-10
    graph; the reference read it back (golden_io.json) to the CSR the
    reference itself generates for -g 10 (golden.json)."""
    assert IO["g10.sg"]["offsets_sha256"] == golden["g10"]["offsets_sha256"]
    assert IO["g10.sg"]["neigh_sha256"] == golden["g10"]["neigh_sha256"]


def bc_digest(sigma, dep, succ, starts, m):
    bits = np.frombuffer(np.ascontiguousarray(succ).tobytes(), np.uint8)[:(m + 7) // 8]
    return dict(depth_sha256=sha(dep.astype(np.int32)),
                path_counts_sha256=sha(sigma.astype(np.uint64)),
                succ_bits_sha256=sha(bits), level_sizes=[int(x) for x in np.diff(starts)],
                reached=int(starts[-1] - starts[0]))


@pytest.mark.parametrize("name", sorted(BC))
def test_bc_oracle_matches_reference(oracle, name):
    gd = BC[name]
    off, nbr = oracle.build_synthetic(*config_args(gd["flags"]))
    for t in gd["trials"]:
        assert t["counts_exact"]
        sigma, dep, succ, order, starts = oracle.bc_bfs(off, nbr, t["source"])
        d = bc_digest(sigma, dep, succ, starts, len(nbr))
        for k in ("depth_sha256", "path_counts_sha256", "succ_bits_sha256", "level_sizes",
                  "reached"):
            assert d[k] == t[k], (name, t["source"], k)

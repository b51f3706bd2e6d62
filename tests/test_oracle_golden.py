"""The oracle restatement, pinned against fixtures made by the reference itself.

tests/golden/golden.json comes from the reference's own gapbs-verify BFS
compiled from its sources (tests/golden/make_golden.py).  Every check here is
CPU-only.
"""
import hashlib

import numpy as np
import pytest

from conftest import config_args

QUICK = ["u10", "g10", "u15", "g15", "g16k8", "u16k4"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", QUICK + ["g18"])
def test_oracle_graph_matches_reference(oracle, golden, name):
    g = golden[name]
    off, nbr = oracle.build_synthetic(*config_args(g["flags"]))
    assert len(off) - 1 == g["num_nodes"]
    assert len(nbr) == g["num_edges_directed"]
    assert sha(off) == g["offsets_sha256"]
    assert sha(nbr) == g["neigh_sha256"]


@pytest.mark.parametrize("name", QUICK)
def test_oracle_sources_match_reference(oracle, golden, name):
    g = golden[name]
    off, _ = oracle.build_synthetic(*config_args(g["flags"]))
    assert [int(x) for x in oracle.source_picker(off, 16)] == g["sources16"]


@pytest.mark.parametrize("name", QUICK + ["g18"])
@pytest.mark.parametrize("threads", [1, 4])
def test_oracle_dobfs_matches_reference(oracle, golden, name, threads):
    g = golden[name]
    off, nbr = oracle.build_synthetic(*config_args(g["flags"]))
    deg = np.diff(off)
    for t in g["trials"]:
        parent, trace, _, _ = oracle.dobfs(off, nbr, t["source"], threads=threads,
                                           want_steps=False)
        assert [list(x) for x in trace] == t["trace"]
        assert int((parent >= 0).sum()) == t["reached"]
        assert int(deg[parent >= 0].sum()) == t["reached_degree_sum"]
        ok, why = oracle.verify(off, nbr, t["source"], parent)
        assert ok, why
        assert sha(oracle.depth(off, nbr, t["source"])) == t["depth_sha256"]


def test_oracle_small_depths(oracle, golden, golden_small):
    for name in ("u10", "g10"):
        off = golden_small[name + "_offsets"]
        nbr = golden_small[name + "_neigh"]
        for t in golden[name]["trials"]:
            d = oracle.depth(off, nbr, t["source"])
            assert np.array_equal(d, golden_small["%s_depth_%d" % (name, t["source"])])


def test_verifier_catches_planted_mistakes(oracle, golden_small):
    """Mistakes are planted in a copy of the oracle's own output, on the CPU."""
    off = golden_small["g10_offsets"]
    nbr = golden_small["g10_neigh"]
    src = 204
    parent, _, _, _ = oracle.dobfs(off, nbr, src)
    assert oracle.verify(off, nbr, src, parent) == (True, 0)
    depth = oracle.depth(off, nbr, src)
    # source not its own parent
    bad = parent.copy()
    bad[src] = int(nbr[off[src]])
    assert oracle.verify(off, nbr, src, bad) == (False, 1)
    # parent that is not a neighbour
    v = int(np.nonzero(depth == 2)[0][0])
    nonnb = [u for u in range(len(off) - 1) if u not in set(nbr[off[v]:off[v + 1]].tolist())
             and u != v]
    bad = parent.copy()
    bad[v] = nonnb[0]
    assert oracle.verify(off, nbr, src, bad) == (False, 3)
    # neighbour at the wrong depth
    nb = nbr[off[v]:off[v + 1]]
    same = [int(u) for u in nb if depth[u] == depth[v]]
    if same:
        bad = parent.copy()
        bad[v] = same[0]
        assert oracle.verify(off, nbr, src, bad) == (False, 2)
    # reachable vertex reported unreachable
    bad = parent.copy()
    bad[v] = -1
    assert oracle.verify(off, nbr, src, bad) == (False, 4)


def test_alg_bytes_model(oracle, golden):
    """Byte model: InitParent 12n, then the per-step terms (serial replay)."""
    off, nbr = oracle.build_synthetic(10, 16, True)
    n = len(off) - 1
    _, trace, st, _ = oracle.dobfs(off, nbr, 204)
    b = 12 * n
    prev = 1
    for r in st["records"]:
        if r["kind"] == "td":
            assert r["frontier"] == prev
            b += 20 * r["frontier"] + 8 * r["edges"] + 8 * r["claimed"]
        elif r["kind"] == "bu":
            b += 4 * n + n // 4 + 8 * r["unvisited"] + 4 * r["edges"] + 4 * r["claimed"]
        elif r["kind"] == "e":
            b += 4 * r["frontier"] + n // 8
        else:
            b += n // 8 + 4 * r["claimed"]
        prev = r["claimed"] if r["kind"] != "e" else r["frontier"]
    assert b == st["alg_bytes"]


def test_reference_sources_are_found_by_override(tmp_path, monkeypatch):
    """oracle/build.py looks for the reference's gapbs-verify/ sources in
    GAPBS_REF_DIR first, then in the staged copy; a directory without them is
    passed over."""
    from oracle import build as B
    (tmp_path / "gapbs-verify").mkdir()
    monkeypatch.setenv("GAPBS_REF_DIR", str(tmp_path))
    assert B.ref_dir() != str(tmp_path)          # no bfs.cc yet
    (tmp_path / "gapbs-verify" / "bfs.cc").write_text("// stand-in\n")
    assert B.ref_dir() == str(tmp_path)

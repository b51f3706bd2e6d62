"""Parity of the CUDA BFS (through the C ABI) with the oracle and the golden
fixtures the reference produced.  Depths must match bit for bit, the step
trace (td/e/bu/c with counts) must equal the reference's, bottom-up parents
must equal the oracle's (they are deterministic: first frontier neighbour in
sorted order), and every parent tree must pass the BFSVerifier restatement."""
import hashlib
import os

import numpy as np
import pytest

from conftest import config_args

pytestmark = pytest.mark.gpu

QUICK = ["u10", "g10", "u15", "g15", "g16k8", "u16k4", "g18"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def check_against_oracle(native, oracle, off, nbr, g, src, alpha=15, beta=18):
    parent, depth, st = native.DOBFS(g, src, alpha=alpha, beta=beta, depth=True, stats=True,
                                     instrument=True)
    opar, otrace, ost, _ = oracle.dobfs(off, nbr, src, alpha=alpha, beta=beta)
    odepth = oracle.depth(off, nbr, src)
    assert np.array_equal(depth, odepth)
    assert st.trace == otrace
    ok, why = oracle.verify(off, nbr, src, parent)
    assert ok, why
    assert st.reached == int((odepth >= 0).sum())
    # bottom-up parents are deterministic
    bu_levels = [s["level"] for s in st.steps if s["kind"] == "bu"]
    if bu_levels:
        mask = np.isin(depth, bu_levels)
        assert np.array_equal(parent[mask], opar[mask])
    # per-step counts of the byte model, and the model total
    rec = [r for r in ost["records"]]
    assert [s["count"] for s in st.steps] == [
        r["claimed"] if r["kind"] != "e" else r["frontier"] for r in rec]
    for s, r in zip(st.steps, rec):
        if s["kind"] in ("td", "bu"):
            assert s["edges"] == r["edges"], (s, r)
        if s["kind"] == "bu":
            assert s["unvisited"] == r["unvisited"]
    assert st.alg_bytes == ost["alg_bytes"]
    # the host-stepped driver runs the same kernels and decisions
    p2, d2, st2 = native.DOBFS(g, src, alpha=alpha, beta=beta, depth=True, stats=True,
                               instrument=True, stepped=True)
    assert np.array_equal(d2, depth)
    assert st2.trace == st.trace
    assert st2.alg_bytes == st.alg_bytes
    assert all(s["seconds"] >= 0 for s in st2.steps)
    for x in (st, st2):
        assert 0 <= x.init_seconds < 1.0
        assert all(0 <= s["seconds"] < 1.0 for s in x.steps)
    return parent, depth, st


@pytest.mark.parametrize("name", QUICK)
def test_golden_graphs(native, oracle, golden, name):
    gd = golden[name]
    off, nbr = native.make_graph(*config_args(gd["flags"]))
    with native.Graph(off, nbr) as g:
        for t in gd["trials"]:
            parent, depth, st = native.DOBFS(g, t["source"], depth=True, stats=True)
            assert [list(x) for x in st.trace] == t["trace"]
            assert sha(depth) == t["depth_sha256"]
            assert int((parent >= 0).sum()) == t["reached"]
            ok, why = oracle.verify(off, nbr, t["source"], parent)
            assert ok, why


def test_golden_small_exact(native, oracle, golden, golden_small):
    for name in ("u10", "g10"):
        off = golden_small[name + "_offsets"]
        nbr = golden_small[name + "_neigh"]
        with native.Graph(off, nbr) as g:
            for t in golden[name]["trials"]:
                _, depth = native.DOBFS(g, t["source"], depth=True)
                assert np.array_equal(depth, golden_small["%s_depth_%d" % (name, t["source"])])


@pytest.mark.parametrize("name", ["u15", "g15", "g18"])
def test_counts_and_bytes_match_oracle(native, oracle, golden, name):
    off, nbr = native.make_graph(*config_args(golden[name]["flags"]))
    with native.Graph(off, nbr) as g:
        for t in golden[name]["trials"][:4]:
            check_against_oracle(native, oracle, off, nbr, g, t["source"])


@pytest.mark.parametrize("alpha,beta", [(1, 18), (2, 2), (15, 1), (1000, 18), (15, 1000),
                                        (4, 50)])
def test_direction_parameters(native, oracle, alpha, beta):
    off, nbr = native.make_graph(14, 16, False)
    with native.Graph(off, nbr) as g:
        for src in native.pick_sources(off, 3):
            check_against_oracle(native, oracle, off, nbr, g, int(src), alpha, beta)


def _graph_from_edges(native, edges, n=None):
    return native.build_csr(np.asarray(edges, np.int32).reshape(-1, 2),
                            num_nodes=-1 if n is None else n)


def _cases():
    rng = np.random.default_rng(11)
    path = [[i, i + 1] for i in range(999)]
    star = [[0, i] for i in range(1, 5000)]
    two = [[i, i + 1] for i in range(99)] + [[200 + i, 201 + i] for i in range(99)]
    k64 = [[i, j] for i in range(64) for j in range(i + 1, 64)]
    iso = [[0, 1], [1, 2], [5, 6], [40, 41], [41, 42], [42, 43]]   # 3,4,7..39 isolated
    ragged = rng.integers(0, 997, size=(3000, 2)).tolist()          # n not a multiple of 32
    loops = [[i, i] for i in range(50)] + [[i, (i * 7) % 50] for i in range(50)] * 3
    tree = [[i, (i - 1) // 3] for i in range(1, 3000)]
    hub = [[0, i] for i in range(1, 70000)] + rng.integers(1, 70000, size=(20000, 2)).tolist()
    return {"path": (path, None), "star": (star, None), "two_components": (two, None),
            "k64": (k64, None), "isolated": (iso, 64), "ragged": (ragged, 997),
            "loops_dups": (loops, None), "tree": (tree, None), "hub": (hub, None)}


@pytest.mark.parametrize("case", list(_cases()))
def test_handmade_graphs(native, oracle, case):
    edges, n = _cases()[case]
    off, nbr = _graph_from_edges(native, edges, n)
    with native.Graph(off, nbr) as g:
        deg = np.diff(off)
        cand = [v for v in (0, 1, 5, len(off) - 2, int(np.argmax(deg))) if deg[v] > 0]
        for src in cand:
            check_against_oracle(native, oracle, off, nbr, g, src)
        for alpha, beta in ((1, 1), (2, 100)):
            check_against_oracle(native, oracle, off, nbr, g, cand[0], alpha, beta)


def test_isolated_source_and_single_vertex(native, oracle):
    off, nbr = _graph_from_edges(native, [[1, 2]], 8)
    with native.Graph(off, nbr) as g:
        parent, depth = native.DOBFS(g, 5, depth=True)
        exp = np.full(8, -1, np.int32)
        exp[5] = 5
        assert np.array_equal(parent, exp)
        exp[5] = 0
        assert np.array_equal(depth, exp)
    off = np.zeros(2, np.int64)
    with native.Graph(off, np.zeros(0, np.int32)) as g:
        parent, st = native.DOBFS(g, 0, stats=True)
        assert list(parent) == [0]
        assert 0 <= st.init_seconds < 1.0   # first search on a fresh handle


def test_bad_source_rejected(native):
    off, nbr = native.make_graph(10, 16, True)
    with native.Graph(off, nbr) as g:
        for bad in (-1, len(off) - 1, 1 << 30):
            with pytest.raises(native.GbbfsError) as e:
                native.DOBFS(g, bad)
            assert e.value.status == native.ERR_ARG


def test_repeated_searches_reuse_state(native, oracle):
    off, nbr = native.make_graph(16, 16, False)
    with native.Graph(off, nbr) as g:
        srcs = native.pick_sources(off, 6)
        first = {}
        for s in srcs:
            first[int(s)] = native.DOBFS(g, int(s), depth=True)[1].copy()
        for s in srcs[::-1]:
            d = native.DOBFS(g, int(s), depth=True)[1]
            assert np.array_equal(d, first[int(s)])
            assert np.array_equal(d, oracle.depth(off, nbr, int(s)))
        # results left on the device, read back later
        native.bfs_device(g, int(srcs[0]), want_depth=True)
        p = np.empty(len(off) - 1, np.int32)
        d = np.empty(len(off) - 1, np.int32)
        native.results(g, p, d)
        assert np.array_equal(d, first[int(srcs[0])])
        native.bfs_device(g, int(srcs[1]))
        with pytest.raises(native.GbbfsError) as e:
            native.results(g, p, d)      # depth was not kept by that search
        assert e.value.status == native.ERR_STATE


def test_many_searches_pipelined(native, oracle):
    """gbbfs_bfs_many: the trial loop in one call, each parent array copied
    out while the next search runs.  Every row is a valid BFS tree of its own
    source (rows in source order), and one shared output keeps the last."""
    off, nbr = native.make_graph(16, 16, False)
    with native.Graph(off, nbr) as g:
        srcs = native.pick_sources(off, 7)
        out = np.full((len(srcs), g.n), -7, np.int32)
        native.bfs_many(g, srcs, out)
        for i, s in enumerate(srcs):
            ok, why = oracle.verify(off, nbr, int(s), out[i])
            assert ok, (i, why)
            assert out[i][int(s)] == int(s)
        one = np.full(g.n, -7, np.int32)
        native.bfs_many(g, srcs[::-1], one)
        ok, why = oracle.verify(off, nbr, int(srcs[0]), one)
        assert ok, why
        last = np.empty(g.n, np.int32)
        native.results(g, last, None)         # the handle's result: the last search
        assert np.array_equal(last, one)
        for i in range(2):                    # fewer searches than parent arrays
            native.bfs_many(g, srcs[i:i + 1], one)
            assert oracle.verify(off, nbr, int(srcs[i]), one)[0]
        native.bfs_many(g, srcs[:0], one)
        with pytest.raises(native.GbbfsError):
            native.bfs_many(g, np.array([srcs[0], g.n + 2], np.int32),
                            np.empty((2, g.n), np.int32))


def test_offset64_path(native, oracle, golden, monkeypatch):
    """The uint64-offset kernels (graphs with >= 2^32 directed edges), forced
    onto small graphs."""
    monkeypatch.setenv("GBBFS_FORCE_OFF64", "1")
    for name in ("u15", "g15"):
        gd = golden[name]
        off, nbr = native.make_graph(*config_args(gd["flags"]))
        with native.Graph(off, nbr) as g:
            for t in gd["trials"][:3]:
                parent, depth, st = native.DOBFS(g, t["source"], depth=True, stats=True)
                assert [list(x) for x in st.trace] == t["trace"]
                assert sha(depth) == t["depth_sha256"]


def test_large_kron_properties(native, oracle):
    """Scale-21 Kronecker: exact depths against the serial oracle for a few
    sources, and the verifier on every tree."""
    off, nbr = native.make_graph(21, 16, False)
    with native.Graph(off, nbr) as g:
        for src in native.pick_sources(off, 3):
            parent, depth, st = native.DOBFS(g, int(src), depth=True, stats=True)
            assert np.array_equal(depth, oracle.depth(off, nbr, int(src)))
            assert oracle.verify(off, nbr, int(src), parent)[0]
            _, otrace, _, _ = oracle.dobfs(off, nbr, int(src), threads=8, want_steps=False)
            assert st.trace == otrace

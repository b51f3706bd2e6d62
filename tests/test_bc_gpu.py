"""BC's BFS phase on the GPU (gbbfs_bc_bfs) against the oracle's serial
restatement (gapbs-verify/bc.cc:51-92): path counts, depths and the
successor bitmap bit for bit, the same level boundaries and the same vertex
set in every level.  And against the reference's PBFS itself: the digests it
recorded in tests/golden/golden_bc.json."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, config_args
from test_reference_pins import bc_digest

pytestmark = pytest.mark.gpu


def check(native, oracle, off, nbr, g, s):
    sig, dep, succ, order, starts = native.bc_bfs(g, int(s))
    osig, odep, osucc, oorder, ostarts = oracle.bc_bfs(off, nbr, int(s))
    assert np.array_equal(dep, odep)
    assert np.array_equal(sig, osig)
    assert np.array_equal(succ, osucc)
    assert np.array_equal(starts, ostarts)
    for d in range(len(starts) - 1):
        a = np.sort(order[starts[d]:starts[d + 1]])
        b = np.sort(oorder[ostarts[d]:ostarts[d + 1]])
        assert np.array_equal(a, b), d
    return sig, dep, succ, order, starts


@pytest.mark.parametrize("scale,uniform", [(12, False), (12, True), (16, False), (16, True)])
def test_generated_graphs(native, oracle, scale, uniform):
    off, nbr = native.make_graph(scale, 16, uniform)
    with native.Graph(off, nbr) as g:
        for s in native.pick_sources(off, 5):
            check(native, oracle, off, nbr, g, s)


def test_handmade_and_edges_cases(native, oracle):
    # square 0-1-3-2-0, a pendant 4 on 3, an isolated 5, a hub 6 joined to
    # 7..5006 and to 0
    edges = [[0, 1], [0, 2], [1, 3], [2, 3], [3, 4], [6, 0]] + [[6, 7 + i] for i in range(5000)]
    off, nbr = native.build_csr(np.array(edges, np.int32), num_nodes=5007)
    with native.Graph(off, nbr) as g:
        for s in (0, 3, 4, 6, 100):
            check(native, oracle, off, nbr, g, s)
        sig, dep, succ, order, starts = check(native, oracle, off, nbr, g, 5)   # isolated
        assert list(order) == [5] and list(starts) == [0, 1] and sig[5] == 1
        with pytest.raises(native.GbbfsError):
            native.bc_bfs(g, len(off) + 3)


def test_path_counts_wrap(native, oracle):
    """A chain of 70 diamonds doubles the path count 70 times: counts wrap
    modulo 2^64 exactly as the reference's unsigned adds."""
    edges, v = [], 0
    for _ in range(70):
        edges += [[v, v + 1], [v, v + 2], [v + 1, v + 3], [v + 2, v + 3]]
        v += 3
    off, nbr = native.build_csr(np.array(edges, np.int32))
    with native.Graph(off, nbr) as g:
        sig, dep, *_ = check(native, oracle, off, nbr, g, 0)
        assert int(sig[3 * 63]) == 1 << 63 and int(sig[3 * 64]) == 0


def test_offset64_path(native, oracle, monkeypatch):
    monkeypatch.setenv("GBBFS_FORCE_OFF64", "1")
    off, nbr = native.make_graph(14, 16, False)
    with native.Graph(off, nbr) as g:
        for s in native.pick_sources(off, 3):
            check(native, oracle, off, nbr, g, s)


@pytest.mark.parametrize("scale,uniform,k", [(12, False, 16), (12, True, 16), (15, False, 8)])
def test_brandes_scores(native, oracle, scale, uniform, k):
    """Normalized scores within the reference verifier's tolerance (1e-6) of
    the exact (double) Brandes sums.  The reference's own float accumulation
    strays up to ~1.5e-6 from them at this size, so it is not the yardstick."""
    off, nbr = native.make_graph(scale, 16, uniform)
    srcs = native.pick_sources(off, k)
    with native.Graph(off, nbr) as g:
        got = native.bc(g, srcs)
        again = native.bc(g, srcs)
    want = oracle.bc(off, nbr, srcs, precise=True)
    assert np.array_equal(got, again)                 # deterministic
    assert float(np.max(np.abs(got - want))) < 1e-6
    assert got.max() == 1.0


def test_brandes_handmade(native, oracle):
    edges = [[0, 1], [0, 2], [1, 3], [2, 3], [3, 4], [6, 0]] + [[6, 7 + i] for i in range(300)]
    off, nbr = native.build_csr(np.array(edges, np.int32), num_nodes=400)
    srcs = np.array([0, 4, 6, 9, 399], np.int32)
    with native.Graph(off, nbr) as g:
        got = native.bc(g, srcs)
        with pytest.raises(native.GbbfsError):
            native.bc(g, np.array([0, 1000], np.int32))
    assert float(np.max(np.abs(got - oracle.bc(off, nbr, srcs, precise=True)))) < 1e-6


def test_bc_cli(native, capsys):
    from dist_mem_gapbs_gb300 import bc_cli
    assert bc_cli.main(["-g", "11", "-n", "3"]) == 0
    out = capsys.readouterr().out
    assert out.count("source: ") == 3 and "Brandes over 3 sources" in out
    assert out.strip().splitlines()[-5].endswith(":1")      # the top score is the maximum


def test_reference_pbfs_fixture(native):
    """Depths, path counts, successor bits and level sizes equal those of the
    reference's own PBFS for every recorded source."""
    with open(os.path.join(GOLDEN_DIR, "golden_bc.json")) as f:
        fx = json.load(f)
    for name, gd in sorted(fx.items()):
        off, nbr = native.make_graph(*config_args(gd["flags"]))
        with native.Graph(off, nbr) as g:
            for t in gd["trials"]:
                sig, dep, succ, order, starts = native.bc_bfs(g, t["source"])
                d = bc_digest(sig, dep, succ, starts, g.m)
                for k in ("depth_sha256", "path_counts_sha256", "succ_bits_sha256",
                          "level_sizes", "reached"):
                    assert d[k] == t[k], (name, t["source"], k)

"""The oracle's BC BFS phase (gapbs-verify/bc.cc:51-92) against a plain
Python statement of what it computes: BFS depths, shortest-path counts
(mod 2^64), and successor bits for the edges that go one level down."""
import numpy as np
import pytest


def python_bc_bfs(off, nbr, source):
    n = len(off) - 1
    depth = np.full(n, -1, np.int64)
    depth[source] = 0
    sigma = [0] * n
    sigma[source] = 1
    frontier = [source]
    levels = [[source]]
    while frontier:
        nxt = []
        for u in frontier:
            for v in nbr[off[u]:off[u + 1]]:
                if depth[v] == -1:
                    depth[v] = depth[u] + 1
                    nxt.append(int(v))
        for u in frontier:
            for v in nbr[off[u]:off[u + 1]]:
                if depth[v] == depth[u] + 1:
                    sigma[v] = (sigma[v] + sigma[u]) % (1 << 64)
        frontier = nxt
        if nxt:
            levels.append(nxt)
    succ = np.zeros((len(nbr) + 31) // 32, np.uint32)
    for u in range(n):
        for e in range(off[u], off[u + 1]):
            if depth[u] >= 0 and depth[nbr[e]] == depth[u] + 1:
                succ[e >> 5] |= np.uint32(1 << (e & 31))
    return np.array(sigma, np.uint64), depth.astype(np.int32), succ, levels


@pytest.mark.parametrize("scale,uniform", [(8, False), (8, True), (10, False)])
def test_bc_bfs_oracle_matches_definition(oracle, scale, uniform):
    off, nbr = oracle.build_synthetic(scale, 8, uniform)
    for s in oracle.source_picker(off, 4):
        sig, dep, succ, order, starts = oracle.bc_bfs(off, nbr, int(s))
        psig, pdep, psucc, plevels = python_bc_bfs(off, nbr, int(s))
        assert np.array_equal(dep, pdep)
        assert np.array_equal(sig, psig)
        assert np.array_equal(succ, psucc)
        assert len(starts) == len(plevels) + 1
        for d, lv in enumerate(plevels):
            assert sorted(order[starts[d]:starts[d + 1]]) == sorted(lv)
        assert np.array_equal(dep, oracle.depth(off, nbr, int(s)))


def test_bc_bfs_oracle_handmade(oracle):
    # square 0-1-3-2-0 plus a pendant 4 on 3 and an isolated 5
    off = np.array([0, 2, 4, 6, 9, 10, 10], np.int64)
    nbr = np.array([1, 2, 0, 3, 0, 3, 1, 2, 4, 3], np.int32)
    sig, dep, succ, order, starts = oracle.bc_bfs(off, nbr, 0)
    assert list(dep) == [0, 1, 1, 2, 3, -1]
    assert list(sig) == [1, 1, 1, 2, 2, 0]
    assert int(succ[0]) == (1 << 0) | (1 << 1) | (1 << 3) | (1 << 5) | (1 << 8)
    assert list(starts) == [0, 1, 3, 4, 5]


def python_brandes(off, nbr, sources):
    n = len(off) - 1
    scores = np.zeros(n, np.float64)
    for s in sources:
        sigma, depth, succ, levels = python_bc_bfs(off, nbr, int(s))
        delta = np.zeros(n, np.float64)
        for lv in reversed(levels):
            for u in lv:
                acc = 0.0
                for e in range(off[u], off[u + 1]):
                    v = nbr[e]
                    if depth[v] == depth[u] + 1:
                        acc += float(sigma[u]) / float(sigma[v]) * (1.0 + delta[v])
                delta[u] = acc
                scores[u] += acc
    return scores / scores.max()


@pytest.mark.parametrize("scale,uniform", [(8, False), (9, True)])
def test_brandes_oracle_matches_definition(oracle, scale, uniform):
    off, nbr = oracle.build_synthetic(scale, 8, uniform)
    srcs = oracle.source_picker(off, 6)
    want = python_brandes(off, nbr, srcs)
    assert np.max(np.abs(oracle.bc(off, nbr, srcs, precise=True) - want)) < 1e-6
    assert np.max(np.abs(oracle.bc(off, nbr, srcs) - want)) < 1e-6

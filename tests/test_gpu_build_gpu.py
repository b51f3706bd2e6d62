"""The CSR built on the GPU (gbbfs_graph_create_from_edges) equals the host
builder's (gbbfs_build_csr, pinned to the reference's Builder by the golden
fixtures) byte for byte, and searches on it match the oracle."""
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def same_csr(native, el, num_nodes=-1):
    host_off, host_nbr = native.build_csr(el, num_nodes)
    with native.Graph.from_edges(el, num_nodes) as g:
        off, nbr = g.csr()
        assert g.n == len(host_off) - 1 and g.m == len(host_nbr)
    assert np.array_equal(off, host_off)
    assert np.array_equal(nbr, host_nbr)
    return off, nbr


@pytest.mark.parametrize("scale,uniform", [(10, True), (10, False), (14, False), (16, True),
                                           (17, False)])
def test_generated_graphs(native, scale, uniform):
    el = native.generate_edges(scale, 16, uniform)
    off, nbr = same_csr(native, el)
    moff, mnbr = native.make_graph(scale, 16, uniform)
    assert np.array_equal(off, moff) and np.array_equal(nbr, mnbr)


def test_handmade_edges(native):
    el = np.array([[0, 1], [1, 0], [1, 1], [2, 3], [3, 2], [2, 3], [4, 4], [0, 5],
                   [5, 0], [7, 2]], np.int32)
    off, nbr = same_csr(native, el)
    assert list(off) == [0, 2, 3, 5, 6, 6, 7, 7, 8]        # 4 has only a self-loop
    assert list(nbr[off[2]:off[3]]) == [3, 7]
    same_csr(native, el, num_nodes=12)                      # isolated tail vertices
    same_csr(native, el[:1])
    same_csr(native, np.zeros((0, 2), np.int32), num_nodes=5)
    same_csr(native, np.zeros((0, 2), np.int32))
    # every vertex of a clique with repeats, in scrambled order
    rng = np.random.default_rng(5)
    pairs = np.array([[i, j] for i in range(40) for j in range(40)] * 3, np.int32)
    same_csr(native, pairs[rng.permutation(len(pairs))])


def test_random_multigraphs(native):
    rng = np.random.default_rng(11)
    for n, e in [(1000, 50000), (3, 1000), (100000, 300000), (70000, 2000)]:
        el = rng.integers(0, n, size=(e, 2)).astype(np.int32)
        same_csr(native, el)
        same_csr(native, el, num_nodes=n + 17)


def test_bad_ids_rejected(native):
    el = np.array([[0, 1], [2, 9]], np.int32)
    with pytest.raises(native.GbbfsError) as e:
        native.Graph.from_edges(el, num_nodes=5)
    assert e.value.status == native.ERR_ARG
    with pytest.raises(native.GbbfsError) as e:
        native.Graph.from_edges(np.array([[0, -3]], np.int32))
    assert e.value.status == native.ERR_ARG


def test_offset64_path(native, monkeypatch):
    monkeypatch.setenv("GBBFS_FORCE_OFF64", "1")
    el = native.generate_edges(12, 16, False)
    same_csr(native, el)


def test_search_on_gpu_built_graph(native, oracle):
    el = native.generate_edges(16, 16, False)
    off, nbr = native.build_csr(el)
    with native.Graph.from_edges(el) as g:
        for s in native.pick_sources(off, 4):
            parent, depth = native.DOBFS(g, int(s), depth=True)
            assert np.array_equal(depth, oracle.depth(off, nbr, int(s)))
            ok, why = oracle.verify(off, nbr, int(s), parent)
            assert ok, why
        d8 = native.msbfs(g, native.pick_sources(off, 40), 4)
        for i, s in enumerate(native.pick_sources(off, 40)[:5]):
            assert np.array_equal(d8[i], oracle.depth(off, nbr, int(s)))


def test_scale20_hash(native):
    el = native.generate_edges(20, 16, False)
    host_off, host_nbr = native.build_csr(el)
    with native.Graph.from_edges(el) as g:
        off, nbr = g.csr()
    h = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    assert h(off) == h(host_off) and h(nbr) == h(host_nbr)

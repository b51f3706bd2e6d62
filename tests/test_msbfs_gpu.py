"""Batched multi-source BFS: every row must equal the single-source depths
(which are pinned to the reference by test_bfs_gpu), bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def single_depths(native, g, sources):
    return np.stack([native.DOBFS(g, int(s), depth=True)[1] for s in sources])


def as_int32(d):
    d = d.astype(np.int32)
    d[d == 255] = -1
    return d


@pytest.mark.parametrize("lanes,batch,alpha", [(64, 8, 15), (32, 4, 2), (64, 16, 200),
                                               (32, 8, 6), (64, 4, 1), (128, 8, 15),
                                               (128, 4, 2), (128, 16, 200), (256, 8, 15),
                                               (256, 4, 2), (256, 16, 200)])
def test_msbfs_matches_single_source(native, lanes, batch, alpha):
    off, nbr = native.make_graph(16, 16, False)
    with native.Graph(off, nbr) as g:
        srcs = native.pick_sources(off, 100)
        ref = single_depths(native, g, srcs)
        native.msbfs_set_config(g, lanes, batch, alpha)
        assert native.msbfs_get_config(g) == dict(lanes=lanes, batch=batch, alpha=alpha)
        d8, st = native.msbfs(g, srcs, 1, stats=True)
        assert st.batches == (100 + lanes - 1) // lanes
        assert np.array_equal(as_int32(d8), ref)
        d32 = native.msbfs(g, srcs, 4)
        assert np.array_equal(d32, ref)


@pytest.mark.parametrize("scale,uniform,lanes", [(15, True, 64), (18, False, 64),
                                                 (15, True, 128), (18, False, 128),
                                                 (15, True, 256), (18, False, 256)])
def test_msbfs_graphs(native, scale, uniform, lanes):
    off, nbr = native.make_graph(scale, 16, uniform)
    with native.Graph(off, nbr) as g:
        native.msbfs_set_config(g, lanes, 8, 15)
        srcs = native.pick_sources(off, 300)
        ref = single_depths(native, g, srcs)
        assert np.array_equal(native.msbfs(g, srcs, 4), ref)
        # fewer sources than lanes, duplicate sources, any order
        sub = np.array([srcs[3], srcs[3], srcs[0], srcs[7]], np.int32)
        got = native.msbfs(g, sub, 4)
        assert np.array_equal(got, ref[[3, 3, 0, 7]])


def test_msbfs_handmade(native):
    edges = np.array([[i, i + 1] for i in range(299)] +      # path: depth up to 299
                     [[400 + i, 401 + i] for i in range(50)] + [[500, 501]], np.int32)
    off, nbr = native.build_csr(edges, num_nodes=520)
    with native.Graph(off, nbr) as g:
        srcs = np.array([0, 150, 299, 400, 510, 425, 500], np.int32)   # 510 is isolated
        ref = single_depths(native, g, srcs)
        assert np.array_equal(native.msbfs(g, srcs, 4), ref)
        # depths above 254 do not fit uint8: refused, not wrapped
        with pytest.raises(native.GbbfsError) as e:
            native.msbfs(g, srcs, 1)
        assert e.value.status == native.ERR_ARG
        ok = np.array([150, 400, 510], np.int32)
        assert np.array_equal(as_int32(native.msbfs(g, ok, 1)), ref[[1, 3, 4]])


@pytest.mark.parametrize("alpha,lanes", [(1, 64), (15, 64), (100000, 64), (1, 128),
                                         (100000, 128), (1, 256), (100000, 256)])
def test_msbfs_hubs(native, alpha, lanes):
    """Vertices above the hub degree are cut into work chunks in both directions."""
    rng = np.random.default_rng(3)
    edges = np.concatenate([
        np.stack([np.zeros(9000, np.int32), np.arange(1, 9001, dtype=np.int32)], 1),
        np.stack([np.full(5000, 9001, np.int32), rng.integers(0, 20000, 5000)], 1),
        rng.integers(0, 20000, size=(30000, 2))]).astype(np.int32)
    off, nbr = native.build_csr(edges)
    with native.Graph(off, nbr) as g:
        deg = np.diff(off)
        srcs = np.array([0, 9001, int(np.argmax(deg[1:]) + 1)] +
                        list(native.pick_sources(off, 40)), np.int32)
        ref = single_depths(native, g, srcs)
        native.msbfs_set_config(g, lanes, 8, alpha)
        assert np.array_equal(native.msbfs(g, srcs, 4), ref)
        assert np.array_equal(as_int32(native.msbfs(g, srcs, 1)), ref)


def test_msbfs_device_and_autotune(native):
    off, nbr = native.make_graph(17, 16, False)
    with native.Graph(off, nbr) as g:
        srcs = native.pick_sources(off, 64)
        best = native.msbfs_autotune(g, srcs, 1)
        assert best["lanes"] in (32, 64, 128, 256) and best["batch"] in (4, 8, 16)
        assert native.msbfs_get_config(g) == best
        ref = single_depths(native, g, srcs)
        assert np.array_equal(as_int32(native.msbfs(g, srcs, 1)), ref)
        ptr, st = native.msbfs_device(g, srcs[:best["lanes"]], 1)
        assert ptr and st.batches == 1
        with pytest.raises(native.GbbfsError):
            native.msbfs_device(g, srcs[:10].tolist() + [len(off) + 5], 1)


def test_msbfs_cli(native, capsys):
    from dist_mem_gapbs_gb300 import msbfs_cli
    assert msbfs_cli.main(["-g", "12", "-n", "40", "--lanes", "32", "--levels"]) == 0
    out = capsys.readouterr().out
    assert out.count("batch ") == 2 and "queries/s" in out and "level  1" in out
    assert msbfs_cli.main(["-g", "12", "-n", "300", "--lanes", "256"]) == 0
    out = capsys.readouterr().out
    assert out.count("batch ") == 2 and "batch 1: 44 sources" in out


def test_msbfs_order(native, batch_keys):
    """Batching order: stable sort by (depth from the highest-degree vertex,
    neighbours' degree sum highest first), keys restated in conftest."""
    off, nbr = native.make_graph(15, 16, False)
    with native.Graph(off, nbr) as g:
        assert np.diff(off).max() > 256             # the sampled-sum path is covered
        key = batch_keys(native, off, nbr, g)
        srcs = native.pick_sources(off, 500)
        srcs = np.concatenate([srcs, srcs[:7]])      # repeats keep their order
        order = native.msbfs_order(g, srcs)
        assert np.array_equal(order, np.argsort(key[srcs], kind="stable"))
        assert len(native.msbfs_order(g, srcs[:0])) == 0
        with pytest.raises(native.GbbfsError):
            native.msbfs_order(g, [0, len(off) + 3])
        # rows of a multi-batch call land at the callers' positions
        native.msbfs_set_config(g, 32, 8, 15)
        ref = single_depths(native, g, srcs[:80])
        assert np.array_equal(native.msbfs(g, srcs[:80], 4), ref)


def test_msbfs_rows_equal_reference_fixture(native, golden):
    """Every row of a batch over the reference's recorded sources hashes to the
    depth array the reference's DOBFS implies (golden.json, Kronecker-18; and
    golden_large.json, Kronecker-22 with all 64 sources)."""
    import hashlib
    import json
    import os
    from conftest import GOLDEN_DIR, config_args
    with open(os.path.join(GOLDEN_DIR, "golden_large.json")) as f:
        large = json.load(f)
    for gd in (golden["g18"], large["g22"]):
        srcs = np.array([t["source"] for t in gd["trials"]], np.int32)
        el = native.generate_edges(*config_args(gd["flags"]))
        with native.Graph.from_edges(el) as g:
            rows = native.msbfs(g, srcs, 1)
            for row, t in zip(rows, gd["trials"]):
                d = as_int32(row)
                assert hashlib.sha256(d.tobytes()).hexdigest() == t["depth_sha256"], t["source"]


def test_msbfs_rows_equal_oracle(native, oracle):
    """16 rows of a 256-lane batch against the oracle's serial BFS depths."""
    off, nbr = native.make_graph(17, 16, False)
    with native.Graph(off, nbr) as g:
        native.msbfs_set_config(g, 256, 8, 15)
        srcs = native.pick_sources(off, 256)
        rows = native.msbfs(g, srcs, 4)
        for i in range(0, 256, 16):
            assert np.array_equal(rows[i], oracle.depth(off, nbr, int(srcs[i]))), i

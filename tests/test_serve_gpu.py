"""Query server: every result must be the same alone and in a mix of
concurrent queries on several resident graphs, and equal to the single-source
search (pinned to the reference by test_bfs_gpu)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def u8(depth32):
    d = depth32.astype(np.int64)
    d[d < 0] = 255
    return d.astype(np.uint8)


@pytest.fixture(scope="module")
def pool(native):
    specs = [(12, 16, False), (12, 16, True), (14, 8, False)]
    graphs = []
    for sc, k, uni in specs:
        off, nbr = native.make_graph(sc, k, uni)
        graphs.append((off, native.Graph(off, nbr)))
    yield graphs
    for _, g in graphs:
        g.close()


def expected(native, pool):
    exp = {}
    for gid, (off, g) in enumerate(pool):
        for s in native.pick_sources(off, 40):
            d = u8(native.DOBFS(g, int(s), depth=True)[1])
            exp[(gid, int(s))] = d
    return exp


def run_queries(native, server, queries, n_of, with_rows):
    rows = {}
    for i, (gid, s) in enumerate(queries):
        out = np.empty(n_of[gid], np.uint8) if with_rows else None
        t = server.submit(gid, s, out)
        rows[t] = (gid, s, out)
    server.drain()
    res = []
    while True:
        got = server.poll(4096)
        if not got:
            break
        res += got
    assert len(res) == len(queries)
    return res, rows


@pytest.mark.parametrize("mode", [0, 1])
def test_alone_and_mixed(native, pool, mode):
    exp = expected(native, pool)
    n_of = [g.n for _, g in pool]
    keys = list(exp)
    with native.Server(mode=mode) as srv:
        ids = [srv.add_graph(g) for _, g in pool]
        assert ids == [0, 1, 2]
        # alone: one query at a time
        alone = {}
        for key in keys[::7]:
            res, rows = run_queries(native, srv, [key], n_of, True)
            r = res[0]
            assert r["status"] == 0 and r["batch_size"] == 1
            alone[key] = (r["checksum"], rows[r["ticket"]][2].copy())
        # mixed: every query of every graph, shuffled, repeats included
        rng = np.random.default_rng(9)
        mix = [keys[i] for i in rng.permutation(len(keys))] + keys[:25]
        res, rows = run_queries(native, srv, mix, n_of, True)
        batched = 0
        for r in res:
            key = (r["graph_id"], r["source"])
            row = rows[r["ticket"]][2]
            assert r["status"] == 0
            assert np.array_equal(row, exp[key])
            assert r["checksum"] == native.depth_checksum(exp[key])
            assert r["reached"] == int((exp[key] != 255).sum())
            assert r["max_depth"] == int(exp[key][exp[key] != 255].max())
            assert r["submit_s"] <= r["start_s"] <= r["done_s"]
            if key in alone:
                assert alone[key][0] == r["checksum"]
                assert np.array_equal(alone[key][1], row)
            batched = max(batched, r["batch_size"])
        if mode == 0:
            assert batched > 1      # queries really shared batches
        else:
            assert batched == 1


def test_admission_budget(native, pool):
    """A budget that holds one graph's search state at a time: graphs take
    turns, every answer still exact."""
    exp = expected(native, pool)
    n_of = [g.n for _, g in pool]
    budget = max(native.msbfs_state_bytes(g.n, g.m, 1) for _, g in pool)
    with native.Server(mode=0, hbm_budget_bytes=budget) as srv:
        for _, g in pool:
            srv.add_graph(g)
        keys = list(exp)
        res, _ = run_queries(native, srv, keys + keys[::-1], n_of, False)
        for r in res:
            assert r["status"] == 0
            assert r["checksum"] == native.depth_checksum(exp[(r["graph_id"], r["source"])])


@pytest.mark.parametrize("max_batch,order", [(256, 0), (128, 1), (128, 0)])
def test_full_width_batches(native, pool, max_batch, order):
    """More queries on one graph than two batches hold: both batch buffers run
    full batches (256 lanes: the widest word), every digest exact."""
    off, g = pool[2]
    srcs = [int(s) for s in native.pick_sources(off, 40)]
    exp = {s: u8(native.DOBFS(g, s, depth=True)[1]) for s in srcs}
    picks = np.array([srcs[i % len(srcs)] for i in range(2 * max_batch + 150)], np.int32)
    with native.Server(mode=0, max_batch=max_batch, order=order) as srv:
        srv.add_graph(g)
        srv.submit(0, srcs[0])                  # admission first
        srv.drain()
        srv.poll(16)
        # one burst: the batcher sees every query before it fills lanes
        srv.submit_many(np.zeros(len(picks), np.int32), picks)
        srv.drain()
        res = srv.poll(4096)
        assert len(res) == len(picks)
        assert max(r["batch_size"] for r in res) == max_batch
        for r in res:
            assert r["status"] == 0
            assert r["checksum"] == native.depth_checksum(exp[r["source"]])


def test_grouped_batches(native, pool, batch_keys):
    """With more queries waiting than a batch holds, grouped batches hold
    sources of closer batching keys than arrival-order batches, the oldest
    query goes in the first batch, and every digest is exact."""
    off, g = pool[0]
    key = batch_keys(native, off, g.csr()[1], g)
    srcs = [int(s) for s in native.pick_sources(off, 40)]
    exp = {s: u8(native.DOBFS(g, s, depth=True)[1]) for s in srcs}
    rng = np.random.default_rng(5)
    keys = [(0, srcs[i]) for i in rng.integers(len(srcs), size=600)]
    spread = {}
    for order in (0, 1):
        with native.Server(mode=0, max_batch=32, order=order) as srv:
            srv.add_graph(g)
            srv.submit(0, srcs[0])          # admission (and the batching keys) first
            srv.drain()
            srv.poll(16)
            tickets = srv.submit_many([k[0] for k in keys], [k[1] for k in keys])
            srv.drain()
            res = []
            while True:
                got = srv.poll(4096)
                if not got:
                    break
                res += got
            assert len(res) == len(keys)
            for r in res:
                assert r["status"] == 0
                assert r["checksum"] == native.depth_checksum(exp[r["source"]])
            first = min(res, key=lambda r: r["ticket"])
            assert first["ticket"] == tickets[0]
            assert first["start_s"] == min(r["start_s"] for r in res)
            batches = {}
            for r in res:
                batches.setdefault(r["start_s"], []).append(key[r["source"]])
            spread[order] = np.mean([max(b) - min(b) for b in batches.values()])
    assert spread[0] < spread[1]


def test_submit_many(native, pool):
    """A burst queued in one call: tickets in order, every digest exact."""
    exp = expected(native, pool)
    keys = list(exp) * 2
    with native.Server(mode=0) as srv:
        for _, g in pool:
            srv.add_graph(g)
        tickets = srv.submit_many([k[0] for k in keys], [k[1] for k in keys])
        assert tickets == sorted(tickets) and len(set(tickets)) == len(keys)
        srv.drain()
        res = []
        while True:
            got = srv.poll(4096)
            if not got:
                break
            res += got
        assert len(res) == len(keys)
        for r in res:
            assert r["status"] == 0
            assert r["checksum"] == native.depth_checksum(exp[(r["graph_id"], r["source"])])
        with pytest.raises(native.GbbfsError):
            srv.submit_many([0, 9], [1, 1])


def test_server_rejects(native, pool):
    with native.Server() as srv:
        gid = srv.add_graph(pool[0][1])
        with pytest.raises(native.GbbfsError):
            srv.submit(gid, pool[0][1].n + 3)
        with pytest.raises(native.GbbfsError):
            srv.submit(gid + 5, 0)
        srv.submit(gid, int(native.pick_sources(pool[0][0], 1)[0]))
        with pytest.raises(native.GbbfsError) as e:
            srv.add_graph(pool[1][1])
        assert e.value.status == native.ERR_STATE
        srv.drain()


@pytest.mark.parametrize("batches_only", [0, 1])
def test_plain_or_batch_per_launch(native, pool, batches_only):
    """Launches of few queries may run as plain searches (once the graph's
    costs are measured), bursts as batches; rows and digests are exact
    either way, and batches_only keeps every launch a batch.  (On graphs
    of a few thousand vertices a batch's kernel is as cheap as one plain
    search, so the graph here is Kronecker-16.)"""
    off, nbr = native.make_graph(16, 16, False)
    g = native.Graph(off, nbr)
    srcs = [int(s) for s in native.pick_sources(off, 40)]
    exp = {s: u8(native.DOBFS(g, s, depth=True)[1]) for s in srcs}
    with g, native.Server(mode=0, batches_only=batches_only) as srv:
        srv.add_graph(g)
        res, rows = [], {}
        for rnd in range(6):                      # one query at a time
            s = srcs[rnd]
            out = np.empty(g.n, np.uint8)
            rows[srv.submit(0, s, out)] = (s, out)
            srv.drain()
            res += srv.poll(16)
        tickets = srv.submit_many([0] * 300, [srcs[i % 40] for i in range(300)])
        srv.drain()
        while True:
            got = srv.poll(4096)
            if not got:
                break
            res += got
        assert len(res) == 306
        for r in res:
            assert r["status"] == 0
            assert r["checksum"] == native.depth_checksum(exp[r["source"]])
        for t, (s, out) in rows.items():
            assert np.array_equal(out, exp[s])
        plain = [r for r in res if r["plain"]]
        if batches_only:
            assert not plain
        else:
            assert plain and all(r["batch_size"] < 256 for r in plain)
        assert max(r["batch_size"] for r in res) > 32


def test_batches_of_two_graphs_overlap_on_the_device(native):
    """With the SMs split among the graphs (grid_policy 1), the batches of two
    graphs run on the GPU at the same time: some pair of their device-clock
    intervals overlaps.  Every result still equals the single-source search."""
    specs = [(18, False), (17, True)]
    graphs = []
    try:
        for sc, uni in specs:
            graphs.append(native.Graph.from_edges(native.generate_edges(sc, 16, uni)))
        srcs = [native.pick_sources(g.offsets, 64) for g in graphs]
        with native.Server(mode=0, batches_only=1, max_batch=32, grid_policy=1) as srv:
            for g in graphs:
                srv.add_graph(g)
            gids = np.repeat(np.arange(2, dtype=np.int32), 512)
            picks = np.concatenate([srcs[i][np.arange(512) % 64] for i in range(2)])
            order = np.random.default_rng(3).permutation(len(gids))
            srv.submit_many(gids[order], picks[order])
            srv.drain()
            res = srv.poll(4096)
        assert len(res) == 1024 and all(r["status"] == 0 for r in res)
        iv = [sorted({(r["device_begin_ns"], r["device_end_ns"]) for r in res
                      if r["graph_id"] == gid}) for gid in range(2)]
        assert all(len(x) >= 2 and all(b > a > 0 for a, b in x) for x in iv)
        overlaps = sum(1 for a0, a1 in iv[0] for b0, b1 in iv[1] if a0 < b1 and b0 < a1)
        assert overlaps > 0, iv
        for gid, g in enumerate(graphs):
            for s in srcs[gid][:8]:
                d = u8(native.DOBFS(g, int(s), depth=True)[1])
                want = native.depth_checksum(d)
                got = {r["checksum"] for r in res if r["graph_id"] == gid and r["source"] == s}
                assert got == {want}
    finally:
        for g in graphs:
            g.close()

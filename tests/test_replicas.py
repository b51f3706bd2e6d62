"""Multi-GPU runs of bench.py are replicas: each rank searches its own slice of
the SourcePicker sequence on its own copy of the graph, and only the final
timings are combined.  This covers that plumbing with two gloo ranks on CPU
(the search itself is replaced by fixed per-search times)."""
import os
import socket

import pytest

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    all_sources = list(range(100, 100 + 8 * world))
    mine = bench.replica_sources(all_sources, rank, world, 8)
    edges = [2000 * (s - 99) for s in mine]
    secs = [1e-3 * (rank + 1)] * len(mine)
    value = bench.hmean_gteps(edges, secs)
    elapsed = sum(secs)
    t = torch.tensor([value, elapsed], dtype=torch.float64)
    allv = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(allv, t)
    combined, t_max = bench.combine_replicas([(float(x[0]), float(x[1])) for x in allv])
    q.put((rank, mine, value, elapsed, combined, t_max))
    dist.destroy_process_group()


def test_two_replicas_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    (r0, s0, v0, t0, c0, m0), (r1, s1, v1, t1, c1, m1) = out
    assert s0 == list(range(100, 108)) and s1 == list(range(108, 116))   # disjoint slices
    assert c0 == pytest.approx(c1) and m0 == m1 == max(t0, t1)
    # rank 1 is twice as slow: the job value counts each rank for its busy share
    assert c0 == pytest.approx(v0 * t0 / m0 + v1 * t1 / m1)


def test_single_rank_value_is_its_hmean():
    v, t = bench.combine_replicas([(123.0, 4.0)])
    assert v == 123.0 and t == 4.0
    assert bench.hmean_gteps([2e9, 4e9], [1.0, 1.0]) == pytest.approx(1.0 / ((1 / 1.0 + 1 / 2.0) / 2))

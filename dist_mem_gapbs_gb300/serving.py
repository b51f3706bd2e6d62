"""Open-loop load generation for the query server.

Queries (graph, source) arrive as a Poisson process of a given rate (seeded
mt19937-style reproducibility through numpy's PCG64 with a fixed seed); the
client submits each at its arrival time on the server clock and collects the
results.  Latency is done - arrival; throughput is completed queries over the
span from the first arrival to the last completion.
"""
import time

import numpy as np

from . import gbbfs


def poisson_schedule(rate_qps, duration_s, n_graphs, sources_per_graph, seed=27491095,
                     weights=None):
    """Arrival times and (graph, source index) of an open-loop query stream."""
    rng = np.random.default_rng(seed)
    count = max(1, int(rate_qps * duration_s))
    gaps = rng.exponential(1.0 / rate_qps, size=count)
    times = np.cumsum(gaps)
    p = None if weights is None else np.asarray(weights, float) / np.sum(weights)
    graphs = rng.choice(n_graphs, size=count, p=p)
    picks = rng.integers(0, sources_per_graph, size=count)
    return times, graphs, picks


def run_open_loop(server, sources, rate_qps, duration_s, seed=27491095, weights=None,
                  timeout_s=120.0):
    """Drive `server` with Poisson arrivals; sources[g] lists graph g's sources.

    Returns a dict with p50/p99/mean latency (ms), offered and achieved qps,
    mean batch size and the per-query results.
    """
    n_graphs = len(sources)
    per = min(len(s) for s in sources)
    times, graphs, picks = poisson_schedule(rate_qps, duration_s, n_graphs, per, seed, weights)
    t0 = server.clock() + 0.05
    arrival = {}
    results = []
    i = 0
    count = len(times)
    deadline = time.time() + duration_s + timeout_s
    while len(results) < count:
        now = server.clock()
        while i < count and t0 + times[i] <= now:
            g = int(graphs[i])
            tk = server.submit(g, int(sources[g][picks[i]]))
            arrival[tk] = t0 + times[i]
            i += 1
        got = server.poll(4096, wait_us=0 if i < count else 2000)
        results.extend(got)
        if time.time() > deadline:
            raise TimeoutError("server did not finish the open-loop run")
    lat = np.array([r["done_s"] - arrival[r["ticket"]] for r in results]) * 1e3
    span = max(r["done_s"] for r in results) - t0
    bad = sum(1 for r in results if r["status"] != gbbfs.OK)
    return dict(queries=count, offered_qps=rate_qps, achieved_qps=count / span,
                p50_ms=float(np.percentile(lat, 50)), p99_ms=float(np.percentile(lat, 99)),
                mean_ms=float(lat.mean()),
                mean_batch=float(np.mean([r["batch_size"] for r in results])),
                errors=bad, results=results)

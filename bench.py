"""Benchmark of the GB300 direction-optimizing BFS (GTEPS, harmonic mean over sources).

One step = one direction-optimizing BFS from each of the workload's sources
(the reference's SourcePicker sequence, -n 64), on a synthetic graph built
exactly as the reference builds it.  The graph (CSR in HBM) is far larger
than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--graph g22|g26|u26|...]
    python bench.py --impl reference ...   # the reference's CPU path, same metric

Multi-GPU runs are replicas (weak scaling): each rank owns its own slice of the
source sequence and its own copy of the graph; nothing is exchanged but the
final timings.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRAPHS = {
    # name: (scale, degree, uniform)
    "g20": (20, 16, False), "g22": (22, 16, False), "g24": (24, 16, False),
    "g26": (26, 16, False), "u22": (22, 16, True), "u26": (26, 16, True),
}


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbbfs", choices=["gbbfs", "reference"])
    ap.add_argument("--graph", default="g26", choices=sorted(GRAPHS))
    ap.add_argument("--sources", type=int, default=64)
    ap.add_argument("--cpu-budget-s", type=float, default=20.0,
                    help="bound on the CPU-baseline sample")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched and serving measurements")
    return ap.parse_args(argv)


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_sources(all_sources, rank, world, per_rank):
    """Rank r's sources: the r-th block of `per_rank` picks of the sequence."""
    return all_sources[rank * per_rank:(rank + 1) * per_rank]


def combine_replicas(per_rank):
    """Whole-job value from per-rank (hmean GTEPS, timed seconds) pairs.

    Each replica contributes its own harmonic-mean rate for the fraction of
    the job's wall time (max over ranks) it was busy; at N=1 this is the
    rank's harmonic mean.
    """
    t_max = max(t for _, t in per_rank)
    return sum(v * (t / t_max) for v, t in per_rank), t_max


def hmean_gteps(edges, seconds):
    """Harmonic mean over searches of (edges / 2) / t."""
    inv = sum(t / (e / 2.0) for e, t in zip(edges, seconds) if e > 0)
    cnt = sum(1 for e in edges if e > 0)
    return (cnt / inv) * 1e-9 if inv > 0 else 0.0


# ---------------------------------------------------------------------------
# clocks during the timed region

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.skip = 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return self
        # nvidia-smi takes a while to start: the timed region opens once its
        # first sample is in (at most a few seconds' wait); only samples taken
        # after that are summarised.
        t_end = time.time() + 5.0
        while not self.lines and time.time() < t_end and self.proc.poll() is None:
            time.sleep(0.01)
        self.skip = len(self.lines)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[self.skip:]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for name, val in zip(names, f[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------

def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def step_alg_bytes(n, step, prev_count):
    """Algorithmic bytes of one step (the byte model of the BFS path)."""
    k = step["kind"]
    if k == "td":
        return 20 * prev_count + 8 * step["edges"] + 8 * step["count"]
    if k == "bu":
        return 4 * n + n // 4 + 8 * step["unvisited"] + 4 * step["edges"] + 4 * step["count"]
    if k == "e":
        return 4 * step["count"] + n // 8
    return n // 8 + 4 * step["count"]


def step_layout_bytes(n, step, prev_count):
    """Bytes one step must move between HBM and the SMs with this library's
    layout (the frontier bitmaps, 8 MB at scale 26, stay in L2 and are not
    counted): uint32 offsets, 32-bit bitmaps swept instead of a parent sweep,
    parents written once per claim."""
    W4 = 4 * ((n + 31) // 32)                  # one bitmap, in bytes
    k, cnt = step["kind"], step["count"]
    if k == "td":
        b = 12 * prev_count + 4 * step["edges"] + 4 * cnt + 16 * cnt
        if step["edges"] > (n >> 3):           # k_tdb + sweep: claim bitmap swept
            b += 2 * W4
        return b
    if k == "bu":
        return 2 * W4 + 4 * min(cnt, W4 // 4) + 4 * step["unvisited"] + 4 * step["edges"] + 4 * cnt
    if k == "e":
        return 4 * cnt
    return W4 + 16 * cnt


def count_launches(step_lists, n):
    """Kernels the searches launched: init, per step a decide and the step
    kernel (a top-down step over more than n/8 frontier edges runs as two:
    claims, sweep), and the final decide that ends the loop."""
    return sum(2 + sum(3 if (x["kind"] == "td" and x["edges"] > (n >> 3)) else 2
                       for x in steps) for steps in step_lists)


def init_layout_bytes(n):
    """k_init: the -1 fill of parent (4 bytes per vertex slot), the iso
    bitmap read, visited and the first frontier bitmap written."""
    W = (n + 31) // 32
    return 4 * 32 * W + 3 * 4 * W


def load_fixture(graph):
    """The reference's own results for this workload (tests/golden/golden_large.json),
    or None when the workload has no fixture."""
    p = os.path.join(ROOT, "tests", "golden", "golden_large.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f).get(graph)


def check_parity(gbbfs, g, sources, fixture):
    """Outside the timed region: every timed source searched once more through
    the C ABI, its step trace and the SHA-256 of its depth array compared with
    the reference's (DOBFS of gapbs-verify, recorded in the fixture)."""
    import hashlib
    if fixture is None:
        return {"fixture": None, "ok": None}
    by_src = {t["source"]: t for t in fixture["trials"]}
    depth = np.empty(g.n, np.int32)
    parent = np.empty(g.n, np.int32)
    checked = trace_eq = depth_eq = 0
    missing = 0
    for s in sources:
        t = by_src.get(int(s))
        if t is None:
            missing += 1
            continue
        _, _, st = gbbfs.DOBFS(g, int(s), depth=True, stats=True, parent_out=parent,
                               depth_out=depth)
        checked += 1
        trace_eq += [list(x) for x in st.trace] == t["trace"]
        depth_eq += hashlib.sha256(depth.tobytes()).hexdigest() == t["depth_sha256"]
    ok = checked > 0 and trace_eq == checked and depth_eq == checked
    return {"fixture": "tests/golden/golden_large.json:%s (reference gapbs-verify DOBFS)"
                       % fixture["flags"], "sources_checked": checked,
            "trace_equal": trace_eq, "depth_sha256_equal": depth_eq,
            "sources_without_fixture": missing, "ok": ok}


def load_traffic(graph, kernel):
    """DRAM bytes per launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(graph, {}).get(kernel)


def cpu_port_sample(off, nbr, sources, budget_s, threads):
    """The oracle port of the reference's OpenMP DOBFS on the host cores."""
    from oracle import oracle as O
    deg = np.diff(off)
    edges, secs = [], []
    t0 = time.time()
    for s in sources:
        parent, _, _, t = O.dobfs(off, nbr, int(s), threads=threads, want_steps=False)
        edges.append(int(deg[parent >= 0].sum()))
        secs.append(t)
        if time.time() - t0 > budget_s:
            break
    return edges, secs


def reference_binary():
    """oracle/_ref/gapbs_ref when it was compiled on this host from the
    reference's own gapbs-verify/bfs.cc (and runs here), else None."""
    from oracle import build as obuild
    exe = os.path.join(obuild.REF_OUT, "gapbs_ref")
    if not os.path.exists(exe):
        return None
    try:
        subprocess.run([exe], capture_output=True, timeout=30)
    except (OSError, subprocess.SubprocessError):
        return None
    return exe


def run_reference_binary(args, exe):
    """The reference's own DOBFS (gapbs-verify/bfs.cc:122-173), built from its
    sources, on every host core: one process builds the graph with the
    reference's Builder, then times (W + K) x per-step searches cycling over the
    workload's SourcePicker picks (oracle/ref_driver.cc, time mode)."""
    scale, degree, uniform = GRAPHS[args.graph]
    threads = os.cpu_count() or 1
    per_step = max(1, min(args.sources, 16 if scale >= 25 else args.sources))
    flags = ["-u" if uniform else "-g", str(scale), "-k", str(degree),
             "-n", str((args.warmup + args.steps) * per_step)]
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    t0 = time.time()
    r = subprocess.run([exe, "time", str(args.sources)] + flags, capture_output=True,
                       text=True, env=env, check=True)
    wall = time.time() - t0
    n = m = None
    trials = []
    for line in r.stdout.splitlines():
        f = line.split()
        if line.startswith("Graph has"):
            n, m = int(f[2]), 2 * int(f[5])
        elif f and f[0] == "trial":
            trials.append((int(f[1]), float(f[2]), int(f[3])))
    timed = trials[args.warmup * per_step:]
    edges = [e for _, _, e in timed]
    secs = [t for _, t, _ in timed]
    value = hmean_gteps(edges, secs)
    step_ms = [1e3 * sum(secs[k * per_step:(k + 1) * per_step]) for k in range(args.steps)]
    sample = ("%d of the %d SourcePicker sources per step (cycling) on %s; gapbs-verify DOBFS "
              "compiled from the reference's sources (g++ -O3 -fopenmp), %d threads; "
              "process wall %.0f s incl. the reference's graph build" %
              (per_step, args.sources, args.graph, threads, wall))
    line = {
        "impl": "reference", "metric": "GTEPS (harmonic mean over sources)", "value": value,
        "unit": "GTEPS", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sum(step_ms) / len(step_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": workload_config(args, n, m),
        "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "reference",
                         "sample": sample},
        "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    exe = reference_binary()
    if exe is not None:
        return run_reference_binary(args, exe)
    from oracle import oracle as O
    scale, degree, uniform = GRAPHS[args.graph]
    off, nbr = O.build_synthetic(scale, degree, uniform)
    sources = O.source_picker(off, args.sources)
    threads = os.cpu_count() or 1
    per_step = max(1, min(args.sources, 16 if scale >= 25 else args.sources))
    deg = np.diff(off)
    reached = {}
    for _ in range(args.warmup):
        for s in sources[:per_step]:
            parent, _, _, _ = O.dobfs(off, nbr, int(s), threads=threads, want_steps=False)
            reached[int(s)] = int(deg[parent >= 0].sum())
    edges, secs, step_times = [], [], []
    for k in range(args.steps):
        t0 = time.perf_counter()
        chunk = [sources[(k * per_step + i) % len(sources)] for i in range(per_step)]
        for s in chunk:
            parent, _, _, t = O.dobfs(off, nbr, int(s), threads=threads, want_steps=False)
            edges.append(int(deg[parent >= 0].sum()))
            secs.append(t)
        step_times.append(time.perf_counter() - t0)
    value = hmean_gteps(edges, secs)
    sample = "%d of the %d sources per step on %s (n=%d, m_dir=%d)" % (
        per_step, args.sources, args.graph, len(off) - 1, len(nbr))
    line = {
        "impl": "reference", "metric": "GTEPS (harmonic mean over sources)", "value": value,
        "unit": "GTEPS", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(step_times) / len(step_times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": workload_config(args, len(off) - 1, len(nbr)),
        "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def workload_config(args, n, m):
    scale, degree, uniform = GRAPHS[args.graph]
    return {"workload": "%s-%d degree %d direction-optimizing BFS, %d SourcePicker sources"
                        % ("uniform" if uniform else "kronecker", scale, degree, args.sources),
            "graph": args.graph, "num_nodes": n, "num_edges_directed": m,
            "alpha": 15, "beta": 18, "sources_per_step": args.sources,
            "parallelism": "replicas" if args.gpus > 1 else "single-gpu",
            "l2": "inputs larger than L2: CSR %.2f GB" % ((4 * m + 8 * (n + 1)) / 1e9)}


def run_gbbfs(args):
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
    else:
        tdist = None
        torch.cuda.set_device(0)
    from dist_mem_gapbs_gb300 import _build, gbbfs
    _build.build()
    scale, degree, uniform = GRAPHS[args.graph]
    t0 = time.time()
    # The reference's generator on the host, the CSR built in HBM
    # (gbbfs_graph_create_from_edges), the host copy read back for the CPU arm.
    el = gbbfs.generate_edges(scale, degree, uniform)
    gen_s = time.time() - t0
    g = gbbfs.Graph.from_edges(el)
    del el
    off, nbr = g.csr()
    build_s = time.time() - t0
    n, m = len(off) - 1, len(nbr)
    all_sources = gbbfs.pick_sources(off, args.sources * world)
    sources = [int(s) for s in replica_sources(all_sources, rank, world, args.sources)]
    deg = np.diff(off)

    # Untimed instrumented pass: per-source reached edges and per-step byte counts.
    info = {}
    for s in sources:
        st = gbbfs.bfs_device(g, s, stats=True, instrument=True)
        parent = np.empty(n, np.int32)
        gbbfs.results(g, parent)
        info[s] = dict(edges=int(deg[parent >= 0].sum()), steps=st.steps)

    def one_step(record, stepped=False):
        for s in sources:
            st = gbbfs.bfs_device(g, s, stats=True, stepped=stepped)
            if record is not None:
                record.append((s, st))

    for _ in range(args.warmup):
        one_step(None)

    # Timed region: every search is one CUDA graph launch (device-resident
    # control loop); per-search device time from CUDA events around it.
    records = []
    if tdist is not None:
        tdist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            one_step(records)
        torch.cuda.synchronize()
        elapsed = time.perf_counter() - t0
    if tdist is not None:
        tdist.barrier()
    edges = [info[s]["edges"] for s, _ in records]
    secs = [st.device_ms * 1e-3 for _, st in records]
    my_value = hmean_gteps(edges, secs)
    busy = sum(secs)
    launches = count_launches([st.steps for _, st in records], n)

    # Kernel shares and the roofline of the dominant kernel: the same searches
    # once more, host-stepped, with CUDA events around every step kernel on
    # the library's stream.
    kind_time = {"init": 0.0, "td": 0.0, "bu": 0.0, "e": 0.0, "c": 0.0}
    kind_bytes = {"init": 0, "td": 0, "bu": 0, "e": 0, "c": 0}
    kind_layout = {"init": 0, "td": 0, "bu": 0, "e": 0, "c": 0}
    kind_launch = {"init": 0, "td": 0, "bu": 0, "e": 0, "c": 0}
    stepped = []
    one_step(stepped, stepped=True)
    for s, st in stepped:
        kind_time["init"] += st.init_seconds
        kind_bytes["init"] += 12 * n
        kind_layout["init"] += init_layout_bytes(n)
        kind_launch["init"] += 1
        prev = 1
        for step, ref in zip(st.steps, info[s]["steps"]):
            kind_time[step["kind"]] += step["seconds"]
            kind_bytes[step["kind"]] += step_alg_bytes(n, ref, prev)
            kind_layout[step["kind"]] += step_layout_bytes(n, ref, prev)
            kind_launch[step["kind"]] += 1
            prev = ref["count"]
    kernel_names = {"init": "k_init", "td": "k_td", "bu": "k_bu", "e": "k_q2b", "c": "k_b2q"}
    dom = max(kind_time, key=lambda k: kind_time[k])
    peak, peak_kind = measured_peaks()
    achieved = kind_bytes[dom] / kind_time[dom] / 1e9 if kind_time[dom] > 0 else 0.0
    traffic = load_traffic(args.graph, kernel_names[dom])

    # End to end through the public call: each step is one gbbfs_bfs_many
    # call over all the sources, the sources in and every search's parent
    # array back in pinned host memory (each copy runs while the next search
    # does).  Same warm-up and step count as the device-timed loop; each
    # search is charged an equal share of the steps' wall time.
    pinned = torch.empty(n, dtype=torch.int32, pin_memory=True)
    host_parent = pinned.numpy()
    for _ in range(args.warmup):
        gbbfs.bfs_many(g, sources, host_parent)
    t1 = time.perf_counter()
    for _ in range(args.steps):
        gbbfs.bfs_many(g, sources, host_parent)
    e2e_wall = time.perf_counter() - t1
    e2e_edges = [info[s]["edges"] for s in sources] * args.steps
    e2e_secs = [e2e_wall / len(e2e_edges)] * len(e2e_edges)
    e2e_value = hmean_gteps(e2e_edges, e2e_secs)

    parity = None
    if rank == 0:
        fx = load_fixture(args.graph)
        if fx is not None and (fx["num_nodes"] != n or fx["num_edges_directed"] != m):
            fx = None
        parity = check_parity(gbbfs, g, sources, fx)

    if tdist is not None:
        t = torch.tensor([my_value, elapsed, e2e_value], dtype=torch.float64, device="cuda")
        allv = [torch.zeros_like(t) for _ in range(world)]
        tdist.all_gather(allv, t)
        per_rank = [(float(x[0]), float(x[1])) for x in allv]
        value, t_max = combine_replicas(per_rank)
        e2e_total, _ = combine_replicas([(float(x[2]), float(x[1])) for x in allv])
    else:
        value, t_max = my_value, elapsed
        e2e_total = e2e_value

    if rank == 0:
        cpu = None
        threads = os.cpu_count() or 1
        c_edges, c_secs = cpu_port_sample(off, nbr, sources, args.cpu_budget_s, threads)
        cpu = {"value": hmean_gteps(c_edges, c_secs), "unit": "GTEPS", "cores": threads,
               "kind": "port",
               "sample": "%d sources of the workload, oracle port of the reference's OpenMP "
                         "DOBFS" % len(c_secs)}
        share = {k: kind_time[k] / max(1e-12, sum(kind_time.values())) for k in kind_time}
        t_all = sum(kind_time.values())
        searches = max(1, len(stepped))

        def frac_of(bytes_total, t):
            return bytes_total / t / 1e9 / peak if t > 0 else 0.0
        whole = {
            "note": "all step kernels of the host-stepped pass: bytes / device time",
            "device_ms_per_search": 1e3 * t_all / searches,
            "model_bytes_per_search": sum(kind_bytes.values()) / searches,
            "model_frac": frac_of(sum(kind_bytes.values()), t_all),
            "layout_bytes_per_search": sum(kind_layout.values()) / searches,
            "layout_frac": frac_of(sum(kind_layout.values()), t_all),
            "per_kernel_layout_frac": {kernel_names[k]: frac_of(kind_layout[k], kind_time[k])
                                       for k in kind_time if kind_time[k] > 0},
        }
        line = {
            "metric": "GTEPS (harmonic mean over sources)", "value": value, "unit": "GTEPS",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": workload_config(args, n, m),
            "roofline": {"bound": "hbm", "kernel": kernel_names[dom], "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_kind, "traffic": traffic,
                         "alg_bytes_per_launch": kind_bytes[dom] / max(1, kind_launch[dom]),
                         "launch_ms": 1e3 * kind_time[dom] / max(1, kind_launch[dom])},
            "kernel_share": share,
            "whole_search_roofline": whole,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_total, "unit": "GTEPS", "h2d_bytes_per_step": 4 * len(sources),
                    "d2h_bytes_per_step": 4 * n * len(sources)},
            "gpu_launches": launches,
            "clocks": clocks.summary(),
            "device_busy_s": busy, "graph_build_s": build_s, "graph_generate_s": gen_s,
            "parity": parity,
        }
    bc_line = None
    if rank == 0 and world == 1 and not args.no_extras:
        try:
            bc_line = run_bc(gbbfs, g, sources[:5], deg)
        except Exception as exc:  # reported, never hides the main line
            bc_line = {"error": "%s: %s" % (type(exc).__name__, exc)}
    g.close()
    del off, nbr
    if rank == 0:
        if bc_line is not None:
            line["bc_bfs_phase"] = bc_line
        if world == 1 and not args.no_extras:
            # The metric's other two parts: batched queries/s and served p50/p99.
            for key, fn in (("batched", run_batched), ("serving", run_serving)):
                try:
                    line[key] = fn(gbbfs)
                except Exception as exc:  # reported, never hides the main line
                    line[key] = {"error": "%s: %s" % (type(exc).__name__, exc)}
        print(json.dumps(line))
    if tdist is not None:
        tdist.destroy_process_group()
    if rank == 0 and parity is not None and parity.get("ok") is False:
        print("bench: depths or step traces differ from the reference's", file=sys.stderr)
        return 1
    return 0


def run_bc(gbbfs, g, sources, deg):
    """BC's BFS phase (gbbfs_bc_bfs) on the metric's graph: wall time per
    source with the path counts, depths, successor bitmap and level order
    copied to host memory."""
    gbbfs.bc_bfs(g, sources[0])                            # state allocated
    ms, rate = [], []
    for s in sources[1:]:
        t = time.perf_counter()
        _, _, _, order, starts = gbbfs.bc_bfs(g, s)
        dt = time.perf_counter() - t
        ms.append(dt * 1e3)
        rate.append(float(deg[order].sum()) / dt / 1e9)
    t = time.perf_counter()
    gbbfs.bc(g, sources[1:])                                # Brandes: BFS phase + dependencies
    brandes_ms = (time.perf_counter() - t) * 1e3 / len(sources[1:])
    return {"sources": len(ms), "ms_per_source": float(np.mean(ms)),
            "edges_per_s_g": float(np.mean(rate)), "levels": int(len(starts) - 1),
            "includes": "device->host copies of all four results",
            "brandes_ms_per_source": brandes_ms}


def check_batched_rows(gbbfs, g, batched, lanes):
    """Outside the timed region: every batch run again with its rows left in
    HBM, each row digested on the device (sum over v of (d[v] + 1) * (v + 1) *
    0x9E3779B97F4A7C15 mod 2^64, d = 255 where unreached), and compared with
    the same digest of the single-source search from that row's source."""
    import torch
    n = g.n
    k64 = 0x9E3779B97F4A7C15 - (1 << 64)
    w = torch.arange(1, n + 1, dtype=torch.int64, device="cuda") * k64

    def digest(d):                       # d: int64 depth with 255 for unreached
        return int(((d + 1) * w).sum().item())

    ok = checked = 0
    for b in range(0, len(batched), lanes):
        srcs = batched[b:b + lanes]
        ptr, _ = gbbfs.msbfs_device(g, srcs, 1)
        rows = torch.as_tensor(gbbfs.DeviceArray(ptr, (len(srcs), n), "|u1"), device="cuda")
        got = [digest(rows[i].to(torch.int64)) for i in range(len(srcs))]
        for i, s in enumerate(srcs):
            gbbfs.bfs_device(g, int(s), want_depth=True)
            _, dptr = gbbfs.result_device_ptrs(g)
            d = torch.as_tensor(gbbfs.DeviceArray(dptr, (n,), "<i4"), device="cuda")
            d = torch.where(d < 0, 255, d).to(torch.int64)
            checked += 1
            ok += digest(d) == got[i]
    return ok, checked


def run_batched(gbbfs, scale=24, queries=4096, plain_sample=256):
    """Batched multi-source BFS on Kronecker-24: queries/s for 4096 sources
    against back-to-back plain single-source launches, rows spot-checked."""
    with gbbfs.Graph.from_edges(gbbfs.generate_edges(scale, 16, False)) as g:
        off = g.offsets
        srcs = gbbfs.pick_sources(off, queries)
        for s in srcs[:8]:
            gbbfs.bfs_device(g, int(s))
        plain_ms = []
        for s in srcs[:plain_sample]:
            plain_ms.append(gbbfs.bfs_device(g, int(s), stats=True).device_ms)
        plain_qps = 1e3 / np.mean(plain_ms)
        t0 = time.time()
        best = gbbfs.msbfs_autotune(g, srcs[:512], 1)     # two batches of 256 at every width
        tune_s = time.time() - t0
        lanes = best["lanes"]
        # The batching order (one single-source search on first use, then a
        # host sort), timed and charged to the batched side.
        t0 = time.perf_counter()
        batched = srcs[gbbfs.msbfs_order(g, srcs)]
        order_ms = (time.perf_counter() - t0) * 1e3
        gbbfs.msbfs_device(g, batched[:lanes], 1)          # warm
        dev_ms = td_ms = bu_ms = 0.0
        for b in range(0, queries, lanes):
            _, st = gbbfs.msbfs_device(g, batched[b:b + lanes], 1)
            dev_ms += st.device_ms
            td_ms += st.td_ms
            bu_ms += st.bu_ms
        # the same sources in the order given (no batching order)
        fifo_ms = 0.0
        for b in range(0, queries, lanes):
            fifo_ms += gbbfs.msbfs_device(g, srcs[b:b + lanes], 1)[1].device_ms
        rows_ok, rows_checked = check_batched_rows(gbbfs, g, batched, lanes)
        if rows_ok != rows_checked:
            raise AssertionError("%d of %d batched depth rows differ from the single-source "
                                 "search" % (rows_checked - rows_ok, rows_checked))
        # a few rows against the oracle's serial BFS as well
        from oracle import oracle as O
        last = batched[queries - 2:queries]
        rows = gbbfs.msbfs(g, last, 4)
        _, nbr_h = g.csr()
        for i in range(len(last)):
            if not np.array_equal(rows[i], O.depth(off, nbr_h, int(last[i]))):
                raise AssertionError("batched depths differ from the oracle")
        del nbr_h
        # with the depth rows streamed to host memory, batch by batch
        import torch
        pinned = torch.empty((lanes, g.n), dtype=torch.uint8, pin_memory=True).numpy()
        t0 = time.time()
        for b in range(0, min(queries, 16 * lanes), lanes):
            gbbfs.msbfs(g, batched[b:b + lanes], 1, out=pinned)
        host_qps = min(queries, 16 * lanes) / (time.time() - t0)
        qps = queries / ((dev_ms + order_ms) * 1e-3)
        return {"workload": "kronecker-%d degree 16, %d sources" % (scale, queries),
                "queries_per_s": qps, "plain_queries_per_s": plain_qps,
                "ratio_vs_plain": qps / plain_qps, "with_host_rows_queries_per_s": host_qps,
                "queries_per_s_in_given_order": queries / (fifo_ms * 1e-3),
                "order_ms": order_ms,
                "config": best, "autotune_s": tune_s, "device_ms": dev_ms,
                "td_ms": td_ms, "bu_ms": bu_ms, "rows_checked": rows_checked,
                "rows_equal": rows_ok, "oracle_rows_checked": 2,
                "rows_check": "every row's depth digest (on the device) against the digest of "
                              "the single-source search from its source"}


def batch_overlap(results):
    """Share of the time some batch kernel ran during which two or more did
    (from the batch kernels' own device-clock stamps in the results)."""
    iv = sorted({(r["device_begin_ns"], r["device_end_ns"]) for r in results
                 if r["device_begin_ns"]})
    ev = sorted([(a, 1) for a, _ in iv] + [(b, -1) for _, b in iv])
    cur, last, busy, multi = 0, None, 0, 0
    for t, d in ev:
        if last is not None and cur > 0:
            busy += t - last
            if cur > 1:
                multi += t - last
        cur += d
        last = t
    return multi / busy if busy else 0.0


def run_serving(gbbfs, rates=(1000, 5000, 10000, 20000), duration_s=2.0, burst=4096):
    """Query server over the 8-graph pool: saturation throughput batched vs
    plain per-query launches, and p50/p99 latency under Poisson arrivals."""
    from dist_mem_gapbs_gb300 import serving
    pool = [(16, False), (18, False), (20, False), (22, False), (24, False), (25, False),
            (20, True), (23, True)]
    graphs, sources = [], []
    t0 = time.time()
    for sc, uni in pool:
        g = gbbfs.Graph.from_edges(gbbfs.generate_edges(sc, 16, uni))
        graphs.append(g)
        sources.append([int(s) for s in gbbfs.pick_sources(g.offsets, 256)])
    build_s = time.time() - t0
    out = {"pool": ["%s%d" % ("u" if u else "g", s) for s, u in pool], "build_s": build_s}
    try:
        for mode, order, name in ((gbbfs.Server.BATCHED, gbbfs.Server.GROUPED, "batched"),
                                  (gbbfs.Server.BATCHED, gbbfs.Server.ARRIVAL,
                                   "batched_arrival_order"),
                                  (gbbfs.Server.PLAIN, gbbfs.Server.ARRIVAL, "plain")):
            with gbbfs.Server(mode=mode, order=order) as srv:
                for g in graphs:
                    srv.add_graph(g)
                # warm every graph once
                for gid in range(len(graphs)):
                    srv.submit(gid, sources[gid][0])
                srv.drain()
                srv.poll(4096)
                # saturation: a burst of queries spread over the pool, handed
                # to the server in one call
                rng = np.random.default_rng(7)
                gids = rng.integers(len(graphs), size=burst)
                picks = rng.integers(256, size=burst)
                srcs = [sources[int(gg)][int(pp)] for gg, pp in zip(gids, picks)]
                t_start = srv.clock()
                srv.submit_many(gids, srcs)
                srv.drain()
                res = srv.poll(burst + 16)
                span = max(r["done_s"] for r in res) - t_start
                out[name + "_saturation_qps"] = burst / span
                if name == "batched":
                    out["latency"] = []
                    for rate in rates:
                        r = serving.run_open_loop(srv, sources, rate, duration_s)
                        res = r.pop("results")
                        r["batch_overlap"] = batch_overlap(res)
                        r["p50_ms_by_graph"] = [
                            float(np.percentile([x["done_s"] - x["submit_s"] for x in res
                                                 if x["graph_id"] == gid], 50) * 1e3)
                            for gid in range(len(graphs))]
                        out["latency"].append(r)
        out["ratio_vs_plain"] = out["batched_saturation_qps"] / out["plain_saturation_qps"]
        out["saturation_vs_50k_offered"] = out["batched_saturation_qps"] / 50000.0
        out["policy"] = "every batch spans the whole GPU, one batch per graph in flight"
        # The same pool with the SMs split among the graphs (grid_policy 1):
        # batches of different graphs run side by side.
        with gbbfs.Server(mode=gbbfs.Server.BATCHED, grid_policy=1) as srv:
            for g in graphs:
                srv.add_graph(g)
            for gid in range(len(graphs)):
                srv.submit(gid, sources[gid][0])
            srv.drain()
            srv.poll(4096)
            out["split_sms_latency"] = []
            for rate in rates[1:3]:
                r = serving.run_open_loop(srv, sources, rate, duration_s)
                res = r.pop("results")
                r["batch_overlap"] = batch_overlap(res)
                out["split_sms_latency"].append(r)
    finally:
        for g in graphs:
            g.close()
    return out


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        return run_reference(args)
    return run_gbbfs(args)


if __name__ == "__main__":
    sys.exit(main())

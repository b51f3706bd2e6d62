"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own gapbs-verify BFS, compiled from its sources by
oracle/build.py into oracle/_ref/gapbs_ref, on the reference's synthetic
graphs, and records:

* the graph: num_nodes, num_edges_directed and SHA-256 of the int64 offsets
  and int32 neighbour arrays that Builder::MakeGraph builds;
* the SourcePicker sequence (first 16 picks);
* per source (the first TRIALS picks): the reference's DOBFS step trace
  (PrintStep kinds and counts, times dropped), the number of reached
  vertices, the summed degree of reached vertices and the SHA-256 of the
  depth array implied by the reference's parent tree;
* for the two 1024-vertex graphs, the full depth arrays (golden_small.npz).

The large configurations the GPU is measured on (Kronecker-22/24/26 and
uniform-26, 64 SourcePicker sources each) go to golden_large.json through the
reference driver's (oracle/ref_driver.cc) "fixture" mode: one reference graph
build per configuration, the hashes computed inside that program, so no
multi-GB array is written out.  The
same fields are recorded (the depth hash is over the depth the reference's
parent tree implies).

Two more fixture files pin the rows around the search:

* golden_bc.json: BC's BFS phase, the reference's PBFS (gapbs-verify/bc.cc:51-92,
  driven by oracle/ref_bc_driver.cc): per source the SHA-256 of the depths, of
  the path counts (as uint64, exact below 2^53) and of the successor bits,
  and the level sizes;
* golden_io.json: the graph files under tests/golden/io/ (edge lists, DIMACS,
  Matrix Market, METIS and a serialized graph, all made here from seeded
  random graphs), each read by the reference's Reader through Builder (-f,
  with -s where the format needs it), with the SHA-256 of the CSR it builds.

Run it where a copy of the reference sources is present (not on the GPU host):
    python tests/golden/make_golden.py            # small fixtures
    python tests/golden/make_golden.py --large    # golden_large.json (~40 min, ~40 GB RAM)
    python tests/golden/make_golden.py --bc       # golden_bc.json
    python tests/golden/make_golden.py --io       # tests/golden/io/ and golden_io.json
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle import oracle as O  # noqa: E402

CONFIGS = [
    ("u10", ["-u", "10"]),
    ("g10", ["-g", "10"]),
    ("u15", ["-u", "15"]),
    ("g15", ["-g", "15"]),
    ("g16k8", ["-g", "16", "-k", "8"]),
    ("u16k4", ["-u", "16", "-k", "4"]),
    ("g18", ["-g", "18"]),
]
TRIALS = 8

LARGE_CONFIGS = [
    ("g22", ["-g", "22"]),
    ("g24", ["-g", "24"]),
    ("u26", ["-u", "26"]),
    ("g26", ["-g", "26"]),
]
LARGE_TRIALS = 64


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def depth_from_parent(parent, source):
    """BFS depth of every vertex in the tree `parent` (-1 where unreached)."""
    n = len(parent)
    depth = np.full(n, -1, dtype=np.int32)
    depth[source] = 0
    has = parent >= 0
    has[source] = False
    while True:
        todo = has & (depth < 0)
        if not todo.any():
            break
        idx = np.nonzero(todo)[0]
        pd = depth[parent[idx]]
        ok = pd >= 0
        if not ok.any():
            raise RuntimeError("parent tree has a cycle or a dangling vertex")
        depth[idx[ok]] = pd[ok] + 1
    return depth


def main():
    obuild.build_ref()
    if not O.ref_available():
        raise SystemExit("reference sources not present: cannot regenerate fixtures")
    out = {}
    small = {}
    for name, flags in CONFIGS:
        with tempfile.TemporaryDirectory() as d:
            off, nbr = O.ref_graph(flags, d)
            srcs = [int(x) for x in O.ref_run("sources", d + "/s", flags + ["-n", "16"]).split()
                    if x.lstrip("-").isdigit()]
            stdout = O.ref_run("bfs", d + "/p", flags + ["-n", str(TRIALS)], threads=4)
            runs = O.parse_trace(stdout)
            par = np.fromfile(d + "/p.par", dtype=np.int32).reshape(TRIALS, -1)
        deg = np.diff(off)
        per = []
        for i, (s, trace) in enumerate(runs):
            dep = depth_from_parent(par[i], s)
            per.append(dict(source=s, trace=[[k, c] for k, c in trace],
                            reached=int((par[i] >= 0).sum()),
                            reached_degree_sum=int(deg[par[i] >= 0].sum()),
                            depth_sha256=sha(dep), max_depth=int(dep.max())))
            if len(off) - 1 <= 1024:
                small["%s_depth_%d" % (name, s)] = dep
        out[name] = dict(flags=flags, num_nodes=int(len(off) - 1),
                         num_edges_directed=int(len(nbr)),
                         offsets_sha256=sha(off), neigh_sha256=sha(nbr),
                         sources16=srcs[-16:], trials=per)
        if len(off) - 1 <= 1024:
            small[name + "_offsets"] = off
            small[name + "_neigh"] = nbr
        print(name, out[name]["num_nodes"], out[name]["num_edges_directed"])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **small)


def parse_fixture(stdout):
    """graph line, source list and per-trial records of ref_driver's fixture mode."""
    graph, sources, trials, trace = None, None, [], None
    for line in stdout.splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "graph":
            graph = dict(num_nodes=int(f[1]), num_edges_directed=int(f[2]),
                         offsets_sha256=f[3], neigh_sha256=f[4])
        elif f[0] == "sources":
            sources = [int(x) for x in f[1:]]
        elif f[0] == "Source:":
            trace = []
        elif f[0] in ("td", "bu") and trace is not None:
            trace.append([f[0], int(f[1])])
        elif f[0] in ("e", "c") and trace is not None:
            trace.append([f[0], 0])
        elif f[0] == "result":
            trials.append(dict(source=int(f[1]), reached=int(f[2]),
                               reached_degree_sum=int(f[3]), max_depth=int(f[4]),
                               depth_sha256=f[5], trace=trace))
            trace = None
    return graph, sources, trials


def main_large(names=None):
    obuild.build_ref()
    if not O.ref_available():
        raise SystemExit("reference sources not present: cannot regenerate fixtures")
    path = os.path.join(HERE, "golden_large.json")
    out = {}
    if os.path.exists(path):
        with open(path) as f:
            out = json.load(f)
    for name, flags in LARGE_CONFIGS:
        if names and name not in names:
            continue
        with tempfile.TemporaryDirectory() as d:
            stdout = O.ref_run("fixture", d + "/f", flags + ["-n", str(LARGE_TRIALS)])
        graph, sources, trials = parse_fixture(stdout)
        assert len(trials) == LARGE_TRIALS and sources == [t["source"] for t in trials]
        out[name] = dict(flags=flags, sources=sources, trials=trials, **graph)
        print(name, graph["num_nodes"], graph["num_edges_directed"], flush=True)
        with open(path, "w") as f:
            json.dump(out, f, indent=1, sort_keys=True)


BC_CONFIGS = [
    ("g10", ["-g", "10"]),
    ("u12", ["-u", "12"]),
    ("g14k8", ["-g", "14", "-k", "8"]),
    ("g16", ["-g", "16"]),
]
BC_TRIALS = 8


def main_bc():
    obuild.build_ref()
    exe = os.path.join(obuild.REF_OUT, "gapbs_ref_bc")
    if not os.path.exists(exe):
        raise SystemExit("reference sources not present: cannot regenerate fixtures")
    out = {}
    for name, flags in BC_CONFIGS:
        r = subprocess.run([exe] + flags + ["-n", str(BC_TRIALS)], capture_output=True,
                           text=True, check=True)
        trials = []
        for line in r.stdout.splitlines():
            f = line.split()
            if f and f[0] == "bcbfs":
                trials.append(dict(source=int(f[1]), reached=int(f[2]), levels=int(f[3]),
                                   counts_exact=bool(int(f[4])), depth_sha256=f[5],
                                   path_counts_sha256=f[6], succ_bits_sha256=f[7],
                                   level_sizes=[int(x) for x in f[8].split(",")]))
        assert len(trials) == BC_TRIALS
        out[name] = dict(flags=flags, trials=trials)
        print(name, [t["source"] for t in trials])
    with open(os.path.join(HERE, "golden_bc.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


IO_DIR = os.path.join(HERE, "io")


def write_io_inputs():
    """Small graph files in every format the reference's Reader takes, from a
    seeded random multigraph (duplicates, self-loops, an isolated vertex)."""
    rng = np.random.default_rng(20240611)
    n = 300
    el = rng.integers(0, n, size=(1500, 2))
    el = el[(el[:, 0] != 150) & (el[:, 1] != 150)]                 # 150 is isolated
    el = np.concatenate([el, el[:40], [[7, 7], [8, 8]], [[n - 1, 3]]])
    w = rng.integers(1, 100, size=len(el))
    os.makedirs(IO_DIR, exist_ok=True)
    files = {}

    def put(name, text):
        with open(os.path.join(IO_DIR, name), "w") as fh:
            fh.write(text)
        files[name] = None

    put("er.el", "".join("%d %d\n" % (u, v) for u, v in el))
    put("er.wel", "".join("%d %d %d\n" % (u, v, x) for (u, v), x in zip(el, w)))
    put("er.gr", "c seeded random multigraph\np sp %d %d\n" % (n, len(el)) +
        "".join("a %d %d %d\n" % (u + 1, v + 1, x) for (u, v), x in zip(el, w)))
    put("er_general.mtx", "%%%%MatrixMarket matrix coordinate pattern general\n"
        "%% seeded random multigraph\n%d %d %d\n" % (n, n, len(el)) +
        "".join("%d %d\n" % (u + 1, v + 1) for u, v in el))
    lower = np.stack([el.max(1), el.min(1)], 1)
    put("er_sym.mtx", "%%%%MatrixMarket matrix coordinate real symmetric\n%d %d %d\n"
        % (n, n, len(lower)) + "".join("%d %d %.3f\n" % (u + 1, v + 1, x / 7.0)
                                        for (u, v), x in zip(lower, w)))
    # METIS: each undirected edge on both endpoints' lines, 1-based, no self-loops
    adj = [set() for _ in range(n)]
    for u, v in el:
        if u != v:
            adj[u].add(v)
            adj[v].add(u)
    # Every adjacency line ends in a space: the reference's METIS reader
    # (gapbs-verify/reader.h:128-131) drops a line's last entry when no
    # whitespace follows it, and these files are meant to be read whole.
    lines = ["% seeded random graph", "%d %d" % (n, sum(len(a) for a in adj) // 2)]
    for u in range(n):
        order = sorted(adj[u], key=lambda x: (x * 7919) % n)
        lines.append("".join("%d " % (v + 1) for v in order))
        if u == 17:
            lines.append("% a comment between two vertices")
    put("er.graph", "\n".join(lines) + "\n")
    # METIS with edge weights (fmt 1): "neighbour weight" pairs
    lines = ["%d %d 1" % (n, sum(len(a) for a in adj) // 2)]
    for u in range(n):
        lines.append("".join("%d %d " % (v + 1, 1 + (u * v) % 9) for v in sorted(adj[u])))
    put("er_w.graph", "\n".join(lines) + "\n")
    # a serialized graph written by this library: the Kronecker-10 graph
    from dist_mem_gapbs_gb300 import _build, gbbfs
    _build.build()
    off, nbr = gbbfs.make_graph(10, 16, False)
    gbbfs.write_sg(os.path.join(IO_DIR, "g10.sg"), off, nbr)
    files["g10.sg"] = None
    return sorted(files)


IO_FLAGS = {".el": ["-s"], ".wel": ["-s"], ".gr": ["-s"], ".graph": [], ".sg": []}


def main_io():
    obuild.build_ref()
    if not O.ref_available():
        raise SystemExit("reference sources not present: cannot regenerate fixtures")
    out = {}
    for name in write_io_inputs():
        suffix = os.path.splitext(name)[1]
        flags = ["-f", os.path.join(IO_DIR, name)]
        flags += ["-s"] if name == "er_general.mtx" else IO_FLAGS.get(suffix, [])
        with tempfile.TemporaryDirectory() as d:
            off, nbr = O.ref_graph(flags, d)
        out[name] = dict(symmetrize="-s" in flags, num_nodes=int(len(off) - 1),
                         num_edges_directed=int(len(nbr)), offsets_sha256=sha(off),
                         neigh_sha256=sha(nbr))
        print(name, out[name]["num_nodes"], out[name]["num_edges_directed"])
    with open(os.path.join(HERE, "golden_io.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)


if __name__ == "__main__":
    if "--bc" in sys.argv:
        main_bc()
    elif "--io" in sys.argv:
        main_io()
    elif "--large" in sys.argv:
        main_large([a for a in sys.argv[1:] if not a.startswith("--")])
    else:
        main()

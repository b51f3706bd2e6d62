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

Run it where the reference checkout exists (not on the GPU host):
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
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


if __name__ == "__main__":
    main()

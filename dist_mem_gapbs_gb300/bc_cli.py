"""Betweenness centrality from the command line (the reference's BC binary,
src/bc.cc:106-171, 252-282, on the GPU).

    python -m dist_mem_gapbs_gb300.bc_cli -g 24 -n 4

Builds the reference's synthetic graph (edge list from the host generator,
CSR built on the GPU), picks -n sources with SourcePicker, times the BFS
phase of each source (gbbfs_bc_bfs, results copied to the host), then runs
Brandes over all of them (gbbfs_bc) and prints the top scores as the
reference's PrintTopScores does (vertex:score, highest first).
"""
import argparse
import sys
import time

import numpy as np

from dist_mem_gapbs_gb300 import gbbfs


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    kind = ap.add_mutually_exclusive_group(required=True)
    kind.add_argument("-g", type=int, help="Kronecker (R-MAT) graph of 2^scale vertices")
    kind.add_argument("-u", type=int, help="uniform random graph of 2^scale vertices")
    ap.add_argument("-k", type=int, default=16, help="average degree")
    ap.add_argument("-n", type=int, default=4, help="sources (iterations)")
    a = ap.parse_args(argv)
    scale, uniform = (a.g, False) if a.g is not None else (a.u, True)
    with gbbfs.Graph.from_edges(gbbfs.generate_edges(scale, a.k, uniform)) as g:
        print("Graph has %d nodes and %d undirected edges" % (g.n, g.m // 2))
        srcs = gbbfs.pick_sources(g.offsets, a.n)
        for s in srcs:
            t = time.perf_counter()
            _, _, _, order, starts = gbbfs.bc_bfs(g, int(s))
            print("source: %d  BFS phase %.3f ms, %d levels, %d reached" % (
                s, (time.perf_counter() - t) * 1e3, len(starts) - 1, len(order)))
        t = time.perf_counter()
        scores = gbbfs.bc(g, srcs)
        print("Brandes over %d sources: %.3f ms" % (len(srcs), (time.perf_counter() - t) * 1e3))
        top = np.argsort(-scores, kind="stable")[:5]
        for v in top:
            print("%d:%g" % (v, scores[v]))
    return 0


if __name__ == "__main__":
    sys.exit(main())

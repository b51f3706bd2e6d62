"""Batched multi-source BFS from the command line.

    python -m dist_mem_gapbs_gb300.msbfs_cli -g 24 -n 512 --levels

Builds the reference's synthetic graph (-g/-u <scale>, -k <degree>; edge
list from the host generator, CSR built on the GPU), picks -n sources with
the reference's SourcePicker, runs them in batches of --lanes sources
through gbbfs_msbfs_device (in gbbfs_msbfs_order's order unless
--given-order) and prints each batch's device time and phase shares,
optionally its per-level times, and the queries/s of all batches.
"""
import argparse
import sys

from dist_mem_gapbs_gb300 import gbbfs


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    kind = ap.add_mutually_exclusive_group(required=True)
    kind.add_argument("-g", type=int, help="Kronecker (R-MAT) graph of 2^scale vertices")
    kind.add_argument("-u", type=int, help="uniform random graph of 2^scale vertices")
    ap.add_argument("-k", type=int, default=16, help="average degree")
    ap.add_argument("-n", type=int, default=256, help="sources")
    ap.add_argument("--lanes", type=int, default=256, choices=(32, 64, 128, 256))
    ap.add_argument("--batch", type=int, default=8, choices=(4, 8, 16))
    ap.add_argument("--alpha", type=int, default=15)
    ap.add_argument("--depth-bytes", type=int, default=1, choices=(1, 4))
    ap.add_argument("--levels", action="store_true", help="print per-level times")
    ap.add_argument("--given-order", action="store_true",
                    help="batch the sources in SourcePicker order")
    a = ap.parse_args(argv)
    scale, uniform = (a.g, False) if a.g is not None else (a.u, True)
    with gbbfs.Graph.from_edges(gbbfs.generate_edges(scale, a.k, uniform)) as g:
        print("Graph has %d nodes and %d undirected edges" % (g.n, g.m // 2))
        srcs = gbbfs.pick_sources(g.offsets, a.n)
        if not a.given_order:
            srcs = srcs[gbbfs.msbfs_order(g, srcs)]
        gbbfs.msbfs_set_config(g, a.lanes, a.batch, a.alpha)
        total_ms = 0.0
        for b in range(0, a.n, a.lanes):
            _, st = gbbfs.msbfs_device(g, srcs[b:b + a.lanes], a.depth_bytes)
            total_ms += st.device_ms
            print("batch %d: %d sources, %.3f ms, %d levels, phases %s" % (
                b // a.lanes, len(srcs[b:b + a.lanes]), st.device_ms, st.levels, st.phases()))
            if a.levels:
                for lvl, ms, f, e, bu in st.per_level():
                    print("  level %2d %s %8.3f ms  frontier %10d  degree sum %12d" % (
                        lvl, "BU" if bu else "TD", ms, f, e))
        print("queries/s: %.1f" % (a.n / (total_ms * 1e-3)))
    return 0


if __name__ == "__main__":
    sys.exit(main())

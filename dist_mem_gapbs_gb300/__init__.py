"""GB300-native direction-optimizing BFS (the DMM-GAPBS BFS hot path).

The compute path is the native library ``_lib/libgbbfs.so`` (hand-written
CUDA for sm_103a behind the C ABI of ``include/gbbfs.h``); this package is the
Python mirror of that interface.  Build it with ``__graft_entry__.build()`` or
``python -m dist_mem_gapbs_gb300._build``.
"""
from .gbbfs import (DOBFS, Graph, GbbfsError, SearchStats, SourcePicker, bfs_device,
                    build_csr, make_graph, pick_sources, results, write_bfs_output, write_sg)

__all__ = ["DOBFS", "Graph", "GbbfsError", "SearchStats", "SourcePicker", "bfs_device",
           "build_csr", "make_graph", "pick_sources", "results", "write_bfs_output", "write_sg"]

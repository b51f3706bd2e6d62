"""Python mirror of the reference's BFS interface over the C ABI (include/gbbfs.h).

Names follow the reference so that tests read like its own usage:

* :func:`make_graph` — ``Builder(cli).MakeGraph()`` for ``-g/-u <scale> -k <degree>``
  or ``-f <file>`` (src/builder.h:314-338);
* :class:`Graph` — the CSR graph, resident in HBM (src/graph.h ``CSRGraph``);
* :class:`SourcePicker` — ``SourcePicker::PickNext`` (src/benchmark.h:49-88);
* :func:`DOBFS` — the direction-optimizing BFS kernel functor
  (src/bfs.cc:142-188);
* :func:`write_bfs_output` — the ``bfs_output.txt`` writer (src/bfs.cc:213-235).

The native library is required: there is no CPU fallback, and every call
raises :class:`GbbfsError` with the library's status when it fails.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgbbfs.so")
CLI_PATH = os.path.join(_HERE, "_lib", "bfs_gpu")

OK, ERR_ARG, ERR_NOMEM, ERR_CUDA, ERR_TIMEOUT, ERR_BOUNDS, ERR_STATE, ERR_IO = range(8)
STEP_TD, STEP_E, STEP_BU, STEP_C = 1, 2, 3, 4
STEP_NAME = {STEP_TD: "td", STEP_E: "e", STEP_BU: "bu", STEP_C: "c"}

# Every symbol include/gbbfs.h declares (the tests check the library exports them).
EXPORTS = (
    "gbbfs_graph_create", "gbbfs_graph_create_from_edges", "gbbfs_graph_csr",
    "gbbfs_graph_destroy", "gbbfs_graph_info", "gbbfs_bfs",
    "gbbfs_bfs_many", "gbbfs_bc_bfs", "gbbfs_bc",
    "gbbfs_bfs_device", "gbbfs_results", "gbbfs_result_device_ptrs", "gbbfs_strerror",
    "gbbfs_last_error", "gbbfs_generate", "gbbfs_free_host", "gbbfs_generate_edges",
    "gbbfs_build_csr", "gbbfs_read_graph", "gbbfs_write_sg", "gbbfs_pick_sources",
    "gbbfs_append_bfs_output", "gbbfs_msbfs", "gbbfs_msbfs_device", "gbbfs_msbfs_set_config",
    "gbbfs_msbfs_get_config", "gbbfs_msbfs_autotune", "gbbfs_msbfs_state_bytes",
    "gbbfs_msbfs_order", "gbbfs_server_open",
    "gbbfs_server_add_graph", "gbbfs_server_submit", "gbbfs_server_submit_many",
    "gbbfs_server_poll", "gbbfs_server_drain",
    "gbbfs_server_clock", "gbbfs_server_close", "gbbfs_bfs_noalloc",
)


class GbbfsError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        detail = ""
        if _lib is not None:
            detail = _lib.gbbfs_last_error().decode()
            name = _lib.gbbfs_strerror(status).decode()
        else:
            name = str(status)
        super().__init__("%s: %s%s" % (what, name, (" (%s)" % detail) if detail else ""))


class Step(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("level", ctypes.c_int32),
                ("count", ctypes.c_int64), ("edges", ctypes.c_int64),
                ("unvisited", ctypes.c_int64), ("seconds", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("steps", ctypes.POINTER(Step)), ("max_steps", ctypes.c_int32),
                ("instrument", ctypes.c_int32), ("stepped", ctypes.c_int32),
                ("num_steps", ctypes.c_int32),
                ("levels", ctypes.c_int32), ("device_ms", ctypes.c_double),
                ("init_seconds", ctypes.c_double), ("reached", ctypes.c_int64),
                ("alg_bytes", ctypes.c_int64)]


class MsConfig(ctypes.Structure):
    _fields_ = [("lanes", ctypes.c_int32), ("batch", ctypes.c_int32), ("alpha", ctypes.c_int32)]

    def as_dict(self):
        return dict(lanes=self.lanes, batch=self.batch, alpha=self.alpha)


class MsStats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("batches", ctypes.c_int32),
                ("levels", ctypes.c_int32), ("lanes", ctypes.c_int32),
                ("batch", ctypes.c_int32), ("alpha", ctypes.c_int32),
                ("td_levels", ctypes.c_int32), ("bu_levels", ctypes.c_int32),
                ("pad", ctypes.c_int32), ("td_ms", ctypes.c_double), ("bu_ms", ctypes.c_double),
                ("phase_share", ctypes.c_double * 8),
                ("level_ms", ctypes.c_double * 32), ("level_frontier", ctypes.c_double * 32),
                ("level_edges", ctypes.c_double * 32), ("level_bu", ctypes.c_int32 * 32)]

    PHASES = ("top_down", "bu_small", "bu_mid", "write", "hub", "clear", "install", "barrier")

    def phases(self):
        return {k: round(self.phase_share[i], 4) for i, k in enumerate(self.PHASES)}

    def per_level(self):
        """[(level, ms, frontier vertices, frontier degree sum, bottom-up
        batches)] summed over the batches of the call."""
        top = min(self.levels, 31)
        return [(l, self.level_ms[l], self.level_frontier[l], self.level_edges[l],
                 self.level_bu[l]) for l in range(1, top + 1)]


_lib = None


def lib():
    """Load libgbbfs.so (built in-tree by __graft_entry__.build())."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libgbbfs.so is not built (%s); run __graft_entry__.build()"
                              % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        P, i64, i32, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int
        PP = ctypes.POINTER(ctypes.c_void_p)
        sig = {
            "gbbfs_graph_create": (I, [P, P, i64, i64, PP]),
            "gbbfs_graph_destroy": (I, [P]),
            "gbbfs_graph_create_from_edges": (I, [P, i64, i64, PP]),
            "gbbfs_graph_csr": (I, [P, P, P]),
            "gbbfs_graph_info": (I, [P, P, P, P]),
            "gbbfs_bfs": (I, [P, i32, I, I, P, P, P]),
            "gbbfs_bfs_many": (I, [P, P, i64, I, I, P, P]),
            "gbbfs_bc_bfs": (I, [P, i32, P, P, P, P, P, P]),
            "gbbfs_bc": (I, [P, P, i64, P]),
            "gbbfs_bfs_device": (I, [P, i32, I, I, I, P]),
            "gbbfs_results": (I, [P, P, P]),
            "gbbfs_result_device_ptrs": (I, [P, PP, PP]),
            "gbbfs_strerror": (ctypes.c_char_p, [I]),
            "gbbfs_last_error": (ctypes.c_char_p, []),
            "gbbfs_generate": (I, [I, I, I, PP, PP, P, P]),
            "gbbfs_free_host": (None, [P]),
            "gbbfs_generate_edges": (I, [I, I, I, PP, P]),
            "gbbfs_build_csr": (I, [P, i64, i64, PP, PP, P, P]),
            "gbbfs_read_graph": (I, [ctypes.c_char_p, I, PP, PP, P, P]),
            "gbbfs_write_sg": (I, [ctypes.c_char_p, P, P, i64, i64]),
            "gbbfs_pick_sources": (I, [P, i64, i64, I, P]),
            "gbbfs_append_bfs_output": (I, [ctypes.c_char_p, P, i64]),
            "gbbfs_msbfs": (I, [P, P, i64, I, P, P]),
            "gbbfs_msbfs_device": (I, [P, P, i64, I, PP, P]),
            "gbbfs_msbfs_set_config": (I, [P, P]),
            "gbbfs_msbfs_get_config": (I, [P, P]),
            "gbbfs_msbfs_autotune": (I, [P, P, i64, I, P]),
            "gbbfs_msbfs_state_bytes": (i64, [i64, i64, I]),
            "gbbfs_msbfs_order": (I, [P, P, i64, P]),
            "gbbfs_server_open": (I, [P, PP]),
            "gbbfs_server_add_graph": (I, [P, P, P]),
            "gbbfs_server_submit": (I, [P, i32, i32, P, P]),
            "gbbfs_server_submit_many": (I, [P, i64, P, P, P, P]),
            "gbbfs_server_poll": (I, [P, P, i32, P, i32]),
            "gbbfs_server_drain": (I, [P, i32]),
            "gbbfs_server_clock": (ctypes.c_double, [P]),
            "gbbfs_server_close": (I, [P]),
            "gbbfs_bfs_noalloc": (I, [P, P, i64, i64, i32, I, I, P, P, P]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _check(rc, what):
    if rc != OK:
        raise GbbfsError(rc, what)


def _take_csr(po, pn, n, m):
    L = lib()
    off = np.ctypeslib.as_array(ctypes.cast(po, ctypes.POINTER(ctypes.c_int64)),
                                shape=(n + 1,)).copy()
    nbr = np.ctypeslib.as_array(ctypes.cast(pn, ctypes.POINTER(ctypes.c_int32)),
                                shape=(max(m, 1),))[:m].copy()
    L.gbbfs_free_host(po)
    L.gbbfs_free_host(pn)
    return off, nbr


def make_graph(scale=None, degree=16, uniform=False, filename=None, symmetrize=False):
    """Host CSR (offsets int64[n+1], neigh int32[m]) as Builder::MakeGraph builds it."""
    L = lib()
    po, pn = ctypes.c_void_p(), ctypes.c_void_p()
    n, m = ctypes.c_int64(), ctypes.c_int64()
    if filename is not None:
        rc = L.gbbfs_read_graph(os.fsencode(filename), 1 if symmetrize else 0, ctypes.byref(po),
                                ctypes.byref(pn), ctypes.byref(n), ctypes.byref(m))
    else:
        rc = L.gbbfs_generate(int(scale), int(degree), 1 if uniform else 0, ctypes.byref(po),
                              ctypes.byref(pn), ctypes.byref(n), ctypes.byref(m))
    _check(rc, "make_graph")
    return _take_csr(po, pn, n.value, m.value)


def build_csr(edges, num_nodes=-1):
    """Symmetrized, squished CSR of an (E, 2) int32 edge list."""
    L = lib()
    el = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
    po, pn = ctypes.c_void_p(), ctypes.c_void_p()
    n, m = ctypes.c_int64(), ctypes.c_int64()
    _check(L.gbbfs_build_csr(_p(el), len(el), int(num_nodes), ctypes.byref(po), ctypes.byref(pn),
                             ctypes.byref(n), ctypes.byref(m)), "build_csr")
    return _take_csr(po, pn, n.value, m.value)


def generate_edges(scale, degree=16, uniform=False):
    """The generator's (E, 2) int32 edge list for -g/-u <scale> -k <degree>
    (src/generator.h), before the CSR is built."""
    L = lib()
    pe, e = ctypes.c_void_p(), ctypes.c_int64()
    _check(L.gbbfs_generate_edges(int(scale), int(degree), 1 if uniform else 0, ctypes.byref(pe),
                                  ctypes.byref(e)), "generate_edges")
    try:
        arr = np.ctypeslib.as_array(ctypes.cast(pe, ctypes.POINTER(ctypes.c_int32)),
                                    shape=(max(e.value, 1) * 2,))[:2 * e.value].copy()
    finally:
        L.gbbfs_free_host(pe)
    return arr.reshape(-1, 2)


def write_sg(path, offsets, neigh):
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    nbr = np.ascontiguousarray(neigh, dtype=np.int32)
    _check(lib().gbbfs_write_sg(os.fsencode(path), _p(off), _p(nbr), len(off) - 1, len(nbr)),
           "write_sg")


class SourcePicker:
    """SourcePicker (src/benchmark.h:49-88): the same sequence of sources."""

    def __init__(self, offsets, given_source=-1):
        self._off = np.ascontiguousarray(offsets, dtype=np.int64)
        self._given = int(given_source)
        self._taken = 0

    def take(self, count):
        """The next `count` picks, as int32 array."""
        total = self._taken + count
        out = np.empty(max(total, 1), dtype=np.int32)
        _check(lib().gbbfs_pick_sources(_p(self._off), len(self._off) - 1, self._given,
                                        total, _p(out)), "pick_sources")
        self._taken = total
        return out[total - count:total]

    def PickNext(self):
        return int(self.take(1)[0])


def pick_sources(offsets, count, given=-1):
    return SourcePicker(offsets, given).take(count)


class Graph:
    """A CSR graph resident in HBM (one gbbfs_graph handle)."""

    def __init__(self, offsets, neigh):
        L = lib()
        self._off = np.ascontiguousarray(offsets, dtype=np.int64)
        nbr = np.ascontiguousarray(neigh, dtype=np.int32)
        self.n = len(self._off) - 1
        self.m = len(nbr)
        h = ctypes.c_void_p()
        _check(L.gbbfs_graph_create(_p(self._off), _p(nbr) if self.m else None, self.n, self.m,
                                    ctypes.byref(h)), "graph_create")
        self._h = h

    @classmethod
    def from_edges(cls, edges, num_nodes=-1):
        """The graph of an (E, 2) int32 edge list, its CSR built on the GPU
        (gbbfs_graph_create_from_edges)."""
        L = lib()
        el = np.ascontiguousarray(edges, dtype=np.int32).reshape(-1, 2)
        h = ctypes.c_void_p()
        _check(L.gbbfs_graph_create_from_edges(_p(el) if len(el) else None, len(el),
                                               int(num_nodes), ctypes.byref(h)),
               "graph_create_from_edges")
        self = cls.__new__(cls)
        self._h = h
        n, m = ctypes.c_int64(), ctypes.c_int64()
        _check(L.gbbfs_graph_info(h, ctypes.byref(n), ctypes.byref(m), None), "graph_info")
        self.n, self.m = n.value, m.value
        self._off = np.empty(self.n + 1, np.int64)
        _check(L.gbbfs_graph_csr(h, _p(self._off), None), "graph_csr")
        return self

    def csr(self):
        """The handle's CSR copied back: (offsets int64[n+1], neigh int32[m])."""
        off = np.empty(self.n + 1, np.int64)
        nbr = np.empty(self.m, np.int32)
        _check(lib().gbbfs_graph_csr(self.handle, _p(off), _p(nbr) if self.m else None),
               "graph_csr")
        return off, nbr

    @property
    def handle(self):
        if self._h is None:
            raise GbbfsError(ERR_STATE, "graph closed")
        return self._h

    @property
    def offsets(self):
        """The CSR offsets (host copy, int64[n+1])."""
        return self._off

    def num_nodes(self):
        return self.n

    def num_edges_directed(self):
        return self.m

    def num_edges(self):
        return self.m // 2

    def out_degree(self, v):
        return int(self._off[v + 1] - self._off[v])

    def device_bytes(self):
        b = ctypes.c_int64()
        _check(lib().gbbfs_graph_info(self.handle, None, None, ctypes.byref(b)), "graph_info")
        return b.value

    def close(self):
        if getattr(self, "_h", None) is not None:
            lib().gbbfs_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class SearchStats:
    """Result of the stats block of one search."""

    def __init__(self, st, steps):
        self.device_ms = st.device_ms
        self.init_seconds = st.init_seconds
        self.levels = st.levels
        self.reached = st.reached
        self.alg_bytes = st.alg_bytes
        k = min(st.num_steps, st.max_steps)
        self.steps = [dict(kind=STEP_NAME[steps[i].kind], level=steps[i].level,
                           count=steps[i].count, edges=steps[i].edges,
                           unvisited=steps[i].unvisited, seconds=steps[i].seconds)
                      for i in range(k)]

    @property
    def trace(self):
        """(kind, count) pairs as the reference's PrintStep lines carry them."""
        return [(s["kind"], s["count"] if s["kind"] in ("td", "bu") else 0) for s in self.steps]


def _stats_block(instrument, stepped=False, max_steps=4096):
    steps = (Step * max_steps)()
    st = Stats()
    st.steps = ctypes.cast(steps, ctypes.POINTER(Step))
    st.max_steps = max_steps
    st.instrument = 1 if instrument else 0
    st.stepped = 1 if stepped else 0
    return st, steps


def DOBFS(g, source, alpha=15, beta=18, depth=False, stats=False, instrument=False,
          stepped=False, parent_out=None, depth_out=None):
    """One direction-optimizing BFS; returns parent (and depth, stats on request).

    parent uses the reference's output encoding: parent[source] == source and
    -1 for vertices the search did not reach.
    """
    parent = parent_out if parent_out is not None else np.empty(g.n, dtype=np.int32)
    dep = None
    if depth:
        dep = depth_out if depth_out is not None else np.empty(g.n, dtype=np.int32)
    st, steps = (_stats_block(instrument, stepped) if (stats or instrument or stepped)
                 else (None, None))
    _check(lib().gbbfs_bfs(g.handle, int(source), int(alpha), int(beta), _p(parent), _p(dep),
                           ctypes.byref(st) if st is not None else None), "bfs")
    out = [parent]
    if depth:
        out.append(dep)
    if st is not None:
        out.append(SearchStats(st, steps))
    return out[0] if len(out) == 1 else tuple(out)


def bfs_many(g, sources, out, alpha=15, beta=18):
    """Searches from every source back to back, each parent array copied to
    host memory while the next search runs.  `out` is a (k, n) int32 array
    (row i for sources[i]) or one n-entry array that every search overwrites
    in turn (the last source's parents remain)."""
    src = np.ascontiguousarray(sources, dtype=np.int32)
    k = len(src)
    if out.dtype != np.int32 or not out.flags["C_CONTIGUOUS"]:
        raise ValueError("out must be a contiguous int32 array")
    if out.ndim == 2:
        if out.shape != (k, g.n):
            raise ValueError("out must be (len(sources), n)")
        ptrs = (ctypes.c_void_p * max(k, 1))(*[out[i].ctypes.data for i in range(k)])
    else:
        if out.shape != (g.n,):
            raise ValueError("out must have n entries")
        ptrs = (ctypes.c_void_p * max(k, 1))(*([out.ctypes.data] * k))
    _check(lib().gbbfs_bfs_many(g.handle, _p(src), k, int(alpha), int(beta), ptrs, None),
           "bfs_many")
    return out


def bc_bfs(g, source):
    """BC's BFS phase (src/bc.cc:55-102): (path counts uint64[n], depth
    int32[n], successor bitmap uint32[(m+31)//32], reached vertices in level
    order int32, level starts int64[levels + 1])."""
    n, m = g.n, g.m
    sigma = np.empty(n, np.uint64)
    dep = np.empty(n, np.int32)
    succ = np.empty(max(1, (m + 31) // 32), np.uint32)
    order = np.empty(max(n, 1), np.int32)
    starts = np.empty(n + 1, np.int64)
    levels = ctypes.c_int32()
    _check(lib().gbbfs_bc_bfs(g.handle, int(source), _p(sigma), _p(dep), _p(succ), _p(order),
                              _p(starts), ctypes.byref(levels)), "bc_bfs")
    lv = levels.value
    return sigma, dep, succ[:(m + 31) // 32], order[:int(starts[lv])], starts[:lv + 1]


def bc(g, sources):
    """Approximate betweenness centrality over `sources` (Brandes,
    src/bc.cc:106-171): float32[n] scores divided by their maximum."""
    src = np.ascontiguousarray(sources, dtype=np.int32)
    scores = np.empty(g.n, np.float32)
    _check(lib().gbbfs_bc(g.handle, _p(src), len(src), _p(scores)), "bc")
    return scores


def bfs_device(g, source, alpha=15, beta=18, want_depth=False, stats=False, instrument=False,
               stepped=False):
    """The search with results left in HBM; returns SearchStats or None."""
    st, steps = (_stats_block(instrument, stepped) if (stats or instrument or stepped)
                 else (None, None))
    _check(lib().gbbfs_bfs_device(g.handle, int(source), int(alpha), int(beta),
                                  1 if want_depth else 0,
                                  ctypes.byref(st) if st is not None else None), "bfs_device")
    return SearchStats(st, steps) if st is not None else None


def results(g, parent_out=None, depth_out=None):
    _check(lib().gbbfs_results(g.handle, _p(parent_out), _p(depth_out)), "results")


def result_device_ptrs(g):
    """Device addresses (parent, depth) of the handle's last search; depth is
    None unless that search kept depths."""
    pp, dp = ctypes.c_void_p(), ctypes.c_void_p()
    _check(lib().gbbfs_result_device_ptrs(g.handle, ctypes.byref(pp), ctypes.byref(dp)),
           "result_device_ptrs")
    return pp.value, dp.value


class DeviceArray:
    """A device buffer of this library seen through __cuda_array_interface__
    (so torch.as_tensor(..., device="cuda") can read it without a copy)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (int(ptr), False), "version": 3,
                                         "strides": None}


def write_bfs_output(path, parent):
    p = np.ascontiguousarray(parent, dtype=np.int32)
    _check(lib().gbbfs_append_bfs_output(os.fsencode(path), _p(p), len(p)), "append_bfs_output")


# ---------------------------------------------------------------------------
# Batched multi-source BFS.

def msbfs(g, sources, depth_bytes=1, out=None, stats=False):
    """Depths from many sources: array (k, n), uint8 (255 = unreached) or
    int32 (-1 = unreached).  Row s equals DOBFS(g, sources[s]) depths."""
    src = np.ascontiguousarray(sources, dtype=np.int32)
    dt = np.uint8 if depth_bytes == 1 else np.int32
    if out is None:
        out = np.empty((len(src), g.n), dtype=dt)
    st = MsStats()
    _check(lib().gbbfs_msbfs(g.handle, _p(src), len(src), int(depth_bytes), _p(out),
                             ctypes.byref(st)), "msbfs")
    return (out, st) if stats else out


def msbfs_device(g, sources, depth_bytes=1):
    """One batch with results left in HBM; returns (device pointer, stats)."""
    src = np.ascontiguousarray(sources, dtype=np.int32)
    ptr = ctypes.c_void_p()
    st = MsStats()
    _check(lib().gbbfs_msbfs_device(g.handle, _p(src), len(src), int(depth_bytes),
                                    ctypes.byref(ptr), ctypes.byref(st)), "msbfs_device")
    return ptr.value, st


def msbfs_order(g, sources):
    """Indices of `sources` in the order to batch them (gbbfs_msbfs_order)."""
    src = np.ascontiguousarray(sources, dtype=np.int32)
    order = np.empty(len(src), np.int32)
    _check(lib().gbbfs_msbfs_order(g.handle, _p(src), len(src), _p(order)), "msbfs_order")
    return order


def msbfs_set_config(g, lanes=256, batch=8, alpha=15):
    c = MsConfig(lanes, batch, alpha)
    _check(lib().gbbfs_msbfs_set_config(g.handle, ctypes.byref(c)), "msbfs_set_config")


def msbfs_get_config(g):
    c = MsConfig()
    _check(lib().gbbfs_msbfs_get_config(g.handle, ctypes.byref(c)), "msbfs_get_config")
    return c.as_dict()


def msbfs_state_bytes(n, m_dir, depth_bytes=1):
    """HBM bytes the batched search state of a graph with n vertices and
    m_dir directed edges takes."""
    r = lib().gbbfs_msbfs_state_bytes(int(n), int(m_dir), int(depth_bytes))
    if r < 0:
        raise ValueError("bad arguments to msbfs_state_bytes")
    return r


def msbfs_autotune(g, sample, depth_bytes=1):
    src = np.ascontiguousarray(sample, dtype=np.int32)
    c = MsConfig()
    _check(lib().gbbfs_msbfs_autotune(g.handle, _p(src), len(src), int(depth_bytes),
                                      ctypes.byref(c)), "msbfs_autotune")
    return c.as_dict()


# ---------------------------------------------------------------------------
# Query server.

class ServerConfig(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("max_batch", ctypes.c_int32),
                ("hbm_budget_bytes", ctypes.c_int64), ("hbm_reserve_bytes", ctypes.c_int64),
                ("order", ctypes.c_int32), ("batches_only", ctypes.c_int32),
                ("grid_policy", ctypes.c_int32), ("max_inflight", ctypes.c_int32),
                ("priorities", ctypes.c_int32)]


class Result(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_uint64), ("graph_id", ctypes.c_int32),
                ("source", ctypes.c_int32), ("status", ctypes.c_int32),
                ("batch_size", ctypes.c_int32), ("submit_s", ctypes.c_double),
                ("start_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("checksum", ctypes.c_uint64), ("reached", ctypes.c_int64),
                ("max_depth", ctypes.c_int32), ("plain", ctypes.c_int32),
                ("device_begin_ns", ctypes.c_uint64), ("device_end_ns", ctypes.c_uint64)]


def depth_checksum(depth_u8):
    """Host restatement of the server's digest of a uint8 depth row."""
    d = np.asarray(depth_u8, dtype=np.uint64)
    v = np.arange(1, len(d) + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        mix = v * np.uint64(0x9E3779B97F4A7C15)
        return int(np.sum((d + np.uint64(1)) * mix, dtype=np.uint64))


class Server:
    """(graph, source) queries answered as they arrive (see include/gbbfs.h)."""

    PLAIN = 1
    BATCHED = 0

    GROUPED = 0
    ARRIVAL = 1

    def __init__(self, mode=0, max_batch=256, hbm_budget_bytes=0, hbm_reserve_bytes=0, order=0,
                 batches_only=0, grid_policy=0, max_inflight=0, priorities=0):
        cfg = ServerConfig(mode, max_batch, hbm_budget_bytes, hbm_reserve_bytes, order,
                           batches_only, grid_policy, max_inflight, priorities)
        h = ctypes.c_void_p()
        _check(lib().gbbfs_server_open(ctypes.byref(cfg), ctypes.byref(h)), "server_open")
        self._h = h
        self._graphs = []
        self._keep = {}

    def add_graph(self, g):
        gid = ctypes.c_int32()
        _check(lib().gbbfs_server_add_graph(self._h, g.handle, ctypes.byref(gid)), "add_graph")
        self._graphs.append(g)
        return gid.value

    def submit(self, graph_id, source, out=None):
        t = ctypes.c_uint64()
        _check(lib().gbbfs_server_submit(self._h, int(graph_id), int(source), _p(out),
                                         ctypes.byref(t)), "server_submit")
        if out is not None:
            self._keep[t.value] = out
        return t.value

    def submit_many(self, graph_ids, sources):
        """Queue a burst of (graph, source) queries at once (digests only);
        returns their tickets."""
        gids = np.ascontiguousarray(graph_ids, dtype=np.int32)
        src = np.ascontiguousarray(sources, dtype=np.int32)
        if gids.shape != src.shape:
            raise ValueError("graph_ids and sources differ in length")
        t = np.empty(len(src), np.uint64)
        _check(lib().gbbfs_server_submit_many(self._h, len(src), _p(gids), _p(src), None,
                                              _p(t)), "server_submit_many")
        return [int(x) for x in t]

    def poll(self, max_results=1024, wait_us=0):
        buf = (Result * max_results)()
        cnt = ctypes.c_int32()
        _check(lib().gbbfs_server_poll(self._h, buf, max_results, ctypes.byref(cnt),
                                       int(wait_us)), "server_poll")
        out = []
        for i in range(cnt.value):
            r = buf[i]
            self._keep.pop(r.ticket, None)
            out.append(dict(ticket=r.ticket, graph_id=r.graph_id, source=r.source,
                            status=r.status, batch_size=r.batch_size, submit_s=r.submit_s,
                            start_s=r.start_s, done_s=r.done_s, checksum=r.checksum,
                            reached=r.reached, max_depth=r.max_depth, plain=r.plain,
                            device_begin_ns=r.device_begin_ns,
                            device_end_ns=r.device_end_ns))
        return out

    def drain(self, timeout_ms=600000):
        _check(lib().gbbfs_server_drain(self._h, int(timeout_ms)), "server_drain")

    def clock(self):
        return lib().gbbfs_server_clock(self._h)

    def close(self):
        if getattr(self, "_h", None) is not None:
            lib().gbbfs_server_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

"""ctypes front end of the oracle library (test infrastructure, not product code).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.  It restates the reference's CPU BFS path (gapbs-verify/bfs.cc,
builder.h, generator.h, benchmark.h) and serves as the checker of the CUDA
path; see oracle/gapbs_oracle.cc for the line-by-line citations.
"""
import ctypes
import os
import subprocess

import numpy as np

from . import build as _build

TD, E, BU, C = 1, 2, 3, 4
KIND_NAME = {TD: "td", E: "e", BU: "bu", C: "c"}


class OrcStep(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int64), ("frontier", ctypes.c_int64),
                ("edges", ctypes.c_int64), ("claimed", ctypes.c_int64),
                ("unvisited", ctypes.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.orc_build_synthetic.restype = i64
        L.orc_build_synthetic.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(P), ctypes.POINTER(P)]
        L.orc_free.argtypes = [P]
        L.orc_source_picker.argtypes = [P, i64, i64, ctypes.c_int, P]
        L.orc_dobfs.restype = ctypes.c_int
        L.orc_dobfs.argtypes = [P, P, i64, ctypes.c_int32, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int, P, P, ctypes.c_int, P,
                                ctypes.POINTER(ctypes.c_double)]
        L.orc_depth.argtypes = [P, P, i64, ctypes.c_int32, P]
        L.orc_verify.restype = ctypes.c_int
        L.orc_verify.argtypes = [P, P, i64, ctypes.c_int32, P, ctypes.POINTER(ctypes.c_int)]
        L.orc_alg_bytes.restype = i64
        L.orc_alg_bytes.argtypes = [i64, P, ctypes.c_int]
        L.orc_bc.argtypes = [P, P, i64, P, i64, ctypes.c_int, P]
        L.orc_bc_bfs.restype = ctypes.c_int32
        L.orc_bc_bfs.argtypes = [P, P, i64, ctypes.c_int32, P, P, P, P, P]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def build_synthetic(scale, degree=16, uniform=False):
    """Symmetrized synthetic CSR exactly as the reference Builder makes it.

    Returns (offsets int64[n+1], neigh int32[m]).
    """
    L = lib()
    po, pn = ctypes.c_void_p(), ctypes.c_void_p()
    n = L.orc_build_synthetic(int(scale), int(degree), 1 if uniform else 0,
                              ctypes.byref(po), ctypes.byref(pn))
    off = np.ctypeslib.as_array(ctypes.cast(po, ctypes.POINTER(ctypes.c_int64)),
                                shape=(n + 1,)).copy()
    m = int(off[-1])
    nbr = np.ctypeslib.as_array(ctypes.cast(pn, ctypes.POINTER(ctypes.c_int32)),
                                shape=(max(m, 1),))[:m].copy()
    L.orc_free(po)
    L.orc_free(pn)
    return off, nbr


def source_picker(off, count, given=-1):
    off = np.ascontiguousarray(off, dtype=np.int64)
    out = np.empty(count, dtype=np.int32)
    lib().orc_source_picker(_ptr(off), len(off) - 1, int(given), int(count), _ptr(out))
    return out


def dobfs(off, nbr, source, alpha=15, beta=18, threads=1, want_steps=True):
    """Direction-optimizing BFS.  Returns (parent, trace, steps, seconds).

    trace is a list of (kind_name, count) in PrintStep order; steps (serial
    form only) a list of dicts with the counts of the byte model.
    """
    off = np.ascontiguousarray(off, dtype=np.int64)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    n = len(off) - 1
    parent = np.empty(n, dtype=np.int32)
    cap = 4096
    trace = np.zeros(2 * cap, dtype=np.int64)
    steps = (OrcStep * cap)() if want_steps else None
    secs = ctypes.c_double(0.0)
    k = lib().orc_dobfs(_ptr(off), _ptr(nbr if len(nbr) else np.zeros(1, np.int32)), n,
                        int(source), int(alpha), int(beta), int(threads), _ptr(parent),
                        _ptr(trace), cap,
                        ctypes.cast(steps, ctypes.c_void_p) if steps is not None else None,
                        ctypes.byref(secs))
    if k < 0:
        raise RuntimeError("trace capacity exceeded")
    tr = [(KIND_NAME[int(trace[2 * i])], int(trace[2 * i + 1])) for i in range(k)]
    st = None
    if steps is not None:
        st = [dict(kind=KIND_NAME[int(steps[i].kind)], frontier=steps[i].frontier,
                   edges=steps[i].edges, claimed=steps[i].claimed,
                   unvisited=steps[i].unvisited) for i in range(k)]
        st_raw = (OrcStep * k)(*[steps[i] for i in range(k)])
        alg = lib().orc_alg_bytes(n, ctypes.cast(st_raw, ctypes.c_void_p), k)
        st = dict(records=st, alg_bytes=int(alg))
    return parent, tr, st, secs.value


def depth(off, nbr, source):
    off = np.ascontiguousarray(off, dtype=np.int64)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    n = len(off) - 1
    d = np.empty(n, dtype=np.int32)
    lib().orc_depth(_ptr(off), _ptr(nbr if len(nbr) else np.zeros(1, np.int32)), n,
                    int(source), _ptr(d))
    return d


def verify(off, nbr, source, parent):
    """BFSVerifier restatement: returns (ok, reason_code)."""
    off = np.ascontiguousarray(off, dtype=np.int64)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    parent = np.ascontiguousarray(parent, dtype=np.int32)
    why = ctypes.c_int(0)
    ok = lib().orc_verify(_ptr(off), _ptr(nbr if len(nbr) else np.zeros(1, np.int32)),
                          len(off) - 1, int(source), _ptr(parent), ctypes.byref(why))
    return bool(ok), why.value


def degree_sum_reached(off, parent):
    """Sum of out-degrees over vertices with parent >= 0 (the TEPS numerator x2)."""
    deg = np.diff(np.asarray(off, dtype=np.int64))
    return int(deg[np.asarray(parent) >= 0].sum())


# ---------------------------------------------------------------------------
# The reference itself, compiled from its sources into oracle/_ref/ (only on a
# host that has the reference checkout).

def ref_available():
    return os.path.exists(os.path.join(_build.REF_OUT, "gapbs_ref"))


def ref_run(mode, prefix, flags, threads=None):
    exe = os.path.join(_build.REF_OUT, "gapbs_ref")
    env = dict(os.environ)
    if threads is not None:
        env["OMP_NUM_THREADS"] = str(threads)
    r = subprocess.run([exe, mode, prefix] + list(flags), capture_output=True,
                       text=True, env=env, check=True)
    return r.stdout


def ref_graph(flags, workdir):
    prefix = os.path.join(workdir, "refgraph")
    ref_run("graph", prefix, flags)
    off = np.fromfile(prefix + ".off", dtype=np.int64)
    nbr = np.fromfile(prefix + ".nbr", dtype=np.int32)
    return off, nbr


def parse_trace(stdout):
    """Per-source lists of (kind, count) from the reference's PrintStep lines."""
    runs = []
    for line in stdout.splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "Source:":
            runs.append((int(f[1]), []))
        elif runs and f[0] in ("td", "bu"):
            runs[-1][1].append((f[0], int(f[1])))
        elif runs and f[0] in ("e", "c"):
            runs[-1][1].append((f[0], 0))
    return runs


def bc_bfs(off, nbr, source):
    """BC's BFS phase (gapbs-verify/bc.cc:51-92), serial: (path counts
    uint64[n], depth int32[n], successor bitmap uint32[(m+31)//32], order of
    the reached vertices int32, level starts int64[levels + 1])."""
    off = np.ascontiguousarray(off, dtype=np.int64)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    n = len(off) - 1
    sigma = np.empty(n, np.uint64)
    dep = np.empty(n, np.int32)
    succ = np.empty(max(1, (len(nbr) + 31) // 32), np.uint32)
    order = np.empty(max(n, 1), np.int32)
    starts = np.empty(n + 2, np.int64)
    levels = lib().orc_bc_bfs(_ptr(off), _ptr(nbr), n, int(source), _ptr(sigma), _ptr(dep),
                              _ptr(succ), _ptr(order), _ptr(starts))
    reached = int(starts[levels])
    return sigma, dep, succ[:(len(nbr) + 31) // 32], order[:reached], starts[:levels + 1]


def bc(off, nbr, sources, precise=False):
    """Brandes over `sources` (src/bc.cc:106-171), serial: float32[n] scores
    divided by their maximum.  precise=True sums in double throughout (the
    values the reference's float sums approximate)."""
    off = np.ascontiguousarray(off, dtype=np.int64)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    src = np.ascontiguousarray(sources, dtype=np.int32)
    scores = np.empty(len(off) - 1, np.float32)
    lib().orc_bc(_ptr(off), _ptr(nbr), len(off) - 1, _ptr(src), len(src), 1 if precise else 0,
                 _ptr(scores))
    return scores

"""In-tree build of the native library and the command-line drop-in.

Produces, under ``dist_mem_gapbs_gb300/_lib/``:

* ``libgbbfs.so`` — the CUDA kernels (sm_103a only) and the C ABI of
  ``include/gbbfs.h``, plus the host-side graph builder (C++/OpenMP);
* ``bfs_gpu`` — the command-line drop-in for the reference's BFS binary.

Translation units compile in parallel; nothing is rebuilt when its sources
are older than its object.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")

LIB = os.path.join(OUT, "libgbbfs.so")
CLI = os.path.join(OUT, "bfs_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function",
             "-I", INCLUDE, "-I", CSRC]

CUDA_SOURCES = ["bfs_engine.cu", "msbfs.cu", "serve.cu", "noalloc.cu", "gpu_build.cu", "bc.cu"]
CXX_SOURCES = ["host_graph.cc", "host_io.cc"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose=False, extra_nvcc=()):
    """Compile everything that is stale; return the path of libgbbfs.so."""
    os.makedirs(OBJ, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + NVCC_FLAGS + list(extra_nvcc) + ["-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs +
             ["-Xcompiler", "-fopenmp", "-lgomp"])
        os.replace(tmp, LIB)
    cli_src = os.path.join(CSRC, "bfs_gpu.cc")
    if _stale(CLI, [cli_src, LIB] + hdrs):
        _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, cli_src, "-o", CLI,
              "-L", OUT, "-lgbbfs", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

"""Build recipe for the oracle (test infrastructure, not product code).

Two things are built:

* ``oracle/_build/libgapbs_oracle.so`` from ``oracle/gapbs_oracle.cc``: the CPU
  restatement of the reference's BFS path that tests/, smoke() and bench.py's
  CPU-baseline leg use as the checker.  It builds on any host with g++ and
  OpenMP (the x86 container and the Arm GPU host alike).
* ``oracle/_ref/`` from the reference's own sources, only where they are
  present (``GAPBS_REF_DIR``, default the read-only reference checkout):
  ``gapbs_ref`` (``oracle/ref_driver.cc`` wrapped around the reference's
  ``gapbs-verify/bfs.cc``) and ``BFS-V`` (``gapbs-verify/bfs.cc`` compiled
  unchanged: the reference's own output checker).  Only g++ is run on the
  reference files where they lie; nothing is copied out of the reference.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
DEFAULT_REF = "/root/reference"

ORACLE_SO = os.path.join(BUILD_DIR, "libgapbs_oracle.so")


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    """Compile the restatement into a shared library; return its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "gapbs_oracle.cc")
    if force or _stale(ORACLE_SO, [src]):
        tmp = ORACLE_SO + ".tmp%d" % os.getpid()
        _run(["g++", "-std=c++17", "-O3", "-fopenmp", "-shared", "-fPIC",
              "-o", tmp, src])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def ref_dir():
    return os.environ.get("GAPBS_REF_DIR", DEFAULT_REF)


def build_ref(force=False):
    """Compile the reference's gapbs-verify BFS into oracle/_ref/.

    Returns the output directory, or None when the reference sources are not
    present on this host (the GPU host never has them).
    """
    gv = os.path.join(ref_dir(), "gapbs-verify")
    if not os.path.exists(os.path.join(gv, "bfs.cc")):
        return None
    if shutil.which("g++") is None:
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    driver = os.path.join(HERE, "ref_driver.cc")
    targets = [
        (os.path.join(REF_OUT, "gapbs_ref"), [driver], driver),
        (os.path.join(REF_OUT, "BFS-V"), [os.path.join(gv, "bfs.cc")],
         os.path.join(gv, "bfs.cc")),
    ]
    for out, deps, main_src in targets:
        if force or _stale(out, deps):
            _run(["g++", "-std=c++11", "-O3", "-fopenmp", "-w", "-I", gv,
                  main_src, "-o", out])
    return REF_OUT


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))

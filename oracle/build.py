"""Build recipe for the oracle (test infrastructure, not product code).

Two things are built:

* ``oracle/_build/libgapbs_oracle.so`` from ``oracle/gapbs_oracle.cc``: the CPU
  restatement of the reference's BFS path that tests/, smoke() and bench.py's
  CPU-baseline leg use as the checker.  It builds on any host with g++ and
  OpenMP (the x86 container and the Arm GPU host alike).
* ``oracle/_ref/`` from the reference's own sources, wherever a copy of its
  ``gapbs-verify/`` directory is found: ``gapbs_ref`` (``oracle/ref_driver.cc``
  wrapped around the reference's ``gapbs-verify/bfs.cc``), ``gapbs_ref_bc``
  (``oracle/ref_bc_driver.cc`` around ``gapbs-verify/bc.cc``) and ``BFS-V``
  (``gapbs-verify/bfs.cc`` compiled unchanged: the reference's own output
  checker).  Only g++ is run on those files; nothing of them is changed.

Where the reference sources come from: ``GAPBS_REF_DIR`` (a reference
checkout), else ``baseline/_ref`` at the repository root, the git-ignored
reference install.  The reference is a C++ project with no Python packaging,
so that install is an unmodified copy of its ``gapbs-verify/`` directory, made
once on a host that has the checkout:

    python oracle/build.py --stage <reference checkout>

It travels with the working tree, so the GPU host (Arm) compiles the
reference there, where binaries built on x86 cannot run.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(ROOT, "baseline", "_ref")

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
    """Directory holding the reference's gapbs-verify/ sources, or None."""
    for d in (os.environ.get("GAPBS_REF_DIR"), STAGE):
        if d and os.path.exists(os.path.join(d, "gapbs-verify", "bfs.cc")):
            return d
    return None


def stage(checkout):
    """Copy the reference's gapbs-verify/ directory, unchanged, into baseline/_ref."""
    src = os.path.join(checkout, "gapbs-verify")
    if not os.path.exists(os.path.join(src, "bfs.cc")):
        raise SystemExit("no gapbs-verify/bfs.cc under %s" % checkout)
    dst = os.path.join(STAGE, "gapbs-verify")
    os.makedirs(dst, exist_ok=True)
    for f in sorted(os.listdir(src)):
        if f.endswith((".cc", ".h")):
            shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
    return dst


def build_ref(force=False):
    """Compile the reference's gapbs-verify BFS (and BC) into oracle/_ref/.

    Returns the output directory, or None when no copy of the reference
    sources is present on this host.
    """
    base = ref_dir()
    if base is None or shutil.which("g++") is None:
        return None
    gv = os.path.join(base, "gapbs-verify")
    os.makedirs(REF_OUT, exist_ok=True)
    headers = [os.path.join(gv, f) for f in os.listdir(gv) if f.endswith(".h")]
    bfs_drv = os.path.join(HERE, "ref_driver.cc")
    bc_drv = os.path.join(HERE, "ref_bc_driver.cc")
    sha = os.path.join(HERE, "sha256.h")
    targets = [
        (os.path.join(REF_OUT, "gapbs_ref"), [bfs_drv, sha, os.path.join(gv, "bfs.cc")], bfs_drv),
        (os.path.join(REF_OUT, "gapbs_ref_bc"), [bc_drv, sha, os.path.join(gv, "bc.cc")], bc_drv),
        (os.path.join(REF_OUT, "BFS-V"), [os.path.join(gv, "bfs.cc")],
         os.path.join(gv, "bfs.cc")),
    ]
    for out, deps, main_src in targets:
        if force or _stale(out, deps + headers):
            tmp = out + ".tmp%d" % os.getpid()
            _run(["g++", "-std=c++11", "-O3", "-fopenmp", "-w", "-I", gv, main_src, "-o", tmp])
            os.replace(tmp, out)
    return REF_OUT


if __name__ == "__main__":
    if "--stage" in sys.argv:
        print(stage(sys.argv[sys.argv.index("--stage") + 1]))
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))

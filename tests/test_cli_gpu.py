"""The bfs_gpu drop-in, end to end: reference flags in, reference stdout lines
and bfs_output.txt out.  The file is checked the way the reference's BFS-V
checks it (gapbs-verify/benchmark.h:132-173): n lines per trial, one decimal
parent per line, every trial's slice passing BFSVerifier."""
import subprocess

import numpy as np
import pytest

from conftest import config_args

pytestmark = pytest.mark.gpu


def run_cli(native, args, cwd):
    r = subprocess.run([native.CLI_PATH] + args, cwd=cwd, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def parse_cli_trace(stdout, prefix=""):
    runs = []
    for line in stdout.splitlines():
        assert line.startswith(prefix), line
        f = line[len(prefix):].split()
        if not f:
            continue
        if f[0] == "Source:":
            runs.append((int(f[1]), []))
        elif runs and f[0] in ("td", "bu"):
            runs[-1][1].append([f[0], int(f[1])])
        elif runs and f[0] in ("e", "c"):
            runs[-1][1].append([f[0], 0])
    return runs


@pytest.mark.parametrize("name", ["u10", "g10", "u15", "g15"])
@pytest.mark.parametrize("stepped", [False, True])
def test_cli_trace_and_output_file(native, oracle, golden, name, stepped, tmp_path):
    gd = golden[name]
    trials = 3
    args = gd["flags"] + ["-n", str(trials), "-v"] + (["--stepped"] if stepped else [])
    out = run_cli(native, args, str(tmp_path))
    lines = out.splitlines()
    assert lines[0] == "Graph has %d nodes and %d undirected edges for degree: %d" % (
        gd["num_nodes"], gd["num_edges_directed"] // 2,
        gd["num_edges_directed"] // 2 // gd["num_nodes"])
    runs = parse_cli_trace(out)
    assert [s for s, _ in runs] == gd["sources16"][:trials]
    for (s, tr), t in zip(runs, gd["trials"]):
        assert tr == t["trace"]
    assert sum(1 for ln in lines if ln.startswith("Trial Time:")) == trials
    assert lines[-2].startswith("Average Time:")
    # bfs_output.txt as BFS-V reads it
    text = (tmp_path / "bfs_output.txt").read_text()
    vals = np.array([int(x) for x in text.split("\n")[:-1]], dtype=np.int64)
    n = gd["num_nodes"]
    assert len(vals) == trials * n
    assert text.endswith("\n")
    off, nbr = native.make_graph(*config_args(gd["flags"]))
    for i in range(trials):
        parent = vals[i * n:(i + 1) * n].astype(np.int32)
        assert parent.min() >= -1
        ok, why = oracle.verify(off, nbr, gd["sources16"][i], parent)
        assert ok, why


def test_cli_dmm_format_and_given_source(native, tmp_path):
    out = run_cli(native, ["-g", "12", "-n", "2", "-r", "5", "--dmm-format", "-a"],
                  str(tmp_path))
    assert all(ln.startswith("PE: 0 | ") for ln in out.splitlines())
    runs = parse_cli_trace(out, "PE: 0 | ")
    assert [s for s, _ in runs] == [5, 5]
    assert "BFS Tree has" in out
    assert not (tmp_path / "bfs_output.txt").exists()


def test_cli_sg_roundtrip(native, tmp_path):
    sg = str(tmp_path / "g13.sg")
    out1 = run_cli(native, ["-g", "13", "-n", "2", "--sg-out", sg], str(tmp_path))
    out2 = run_cli(native, ["-f", sg, "-n", "2"], str(tmp_path))
    assert parse_cli_trace(out1) == parse_cli_trace(out2)

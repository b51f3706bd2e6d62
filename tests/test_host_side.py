"""Host side of the product library (no GPU): graph construction, sources,
graph files, the bfs_output.txt writer, and the exported C ABI."""
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, config_args


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["u10", "g10", "u15", "g15", "g16k8", "u16k4", "g18"])
def test_product_graph_matches_reference(native, golden, name):
    g = golden[name]
    off, nbr = native.make_graph(*config_args(g["flags"]))
    assert len(off) - 1 == g["num_nodes"]
    assert sha(off) == g["offsets_sha256"]
    assert sha(nbr) == g["neigh_sha256"]
    assert [int(s) for s in native.pick_sources(off, 16)] == g["sources16"]


def test_source_picker_incremental(native, golden):
    off, _ = native.make_graph(10, 16, True)
    sp = native.SourcePicker(off)
    picks = [sp.PickNext() for _ in range(16)]
    assert picks == golden["u10"]["sources16"]
    assert list(native.SourcePicker(off, given_source=7).take(3)) == [7, 7, 7]


def _reference_csr(edges, n=None):
    """CSR the reference's Builder makes: symmetrize, sort, unique, drop self."""
    n = n if n is not None else int(np.max(edges)) + 1
    adj = [set() for _ in range(n)]
    for u, v in edges:
        adj[u].add(v)
        adj[v].add(u)
    off = [0]
    nbr = []
    for u in range(n):
        s = sorted(x for x in adj[u] if x != u)
        nbr += s
        off.append(len(nbr))
    return np.array(off, np.int64), np.array(nbr, np.int32)


def test_build_csr_squishes(native):
    edges = np.array([[0, 1], [1, 0], [1, 1], [2, 5], [5, 2], [2, 5], [3, 3], [0, 4],
                      [4, 0], [6, 0]], np.int32)
    off, nbr = native.build_csr(edges)
    ro, rn = _reference_csr(edges)
    assert np.array_equal(off, ro) and np.array_equal(nbr, rn)
    # isolated vertex 3 (only a self loop) keeps degree 0
    assert off[4] - off[3] == 0


def test_build_csr_random(native):
    rng = np.random.default_rng(5)
    edges = rng.integers(0, 300, size=(5000, 2)).astype(np.int32)
    off, nbr = native.build_csr(edges)
    ro, rn = _reference_csr(edges)
    assert np.array_equal(off, ro) and np.array_equal(nbr, rn)


def test_build_csr_rejects_bad_ids(native):
    with pytest.raises(native.GbbfsError):
        native.build_csr(np.array([[0, -3]], np.int32))
    with pytest.raises(native.GbbfsError):
        native.build_csr(np.array([[0, 9]], np.int32), num_nodes=5)


def test_sg_roundtrip(native, tmp_path):
    off, nbr = native.make_graph(12, 8, False)
    p = str(tmp_path / "g12.sg")
    native.write_sg(p, off, nbr)
    raw = open(p, "rb").read()
    # bool directed, int64 num_edges_directed, int64 num_nodes (src/writer.h:49-54)
    assert raw[0] == 0
    assert int.from_bytes(raw[1:9], "little") == len(nbr)
    assert int.from_bytes(raw[9:17], "little") == len(off) - 1
    assert len(raw) == 17 + 8 * len(off) + 4 * len(nbr)
    o2, n2 = native.make_graph(filename=p)
    assert np.array_equal(off, o2) and np.array_equal(nbr, n2)


def test_sg_rejects_corrupt(native, tmp_path):
    p = str(tmp_path / "bad.sg")
    with open(p, "wb") as f:
        f.write(b"\x00" + (100).to_bytes(8, "little") + (10).to_bytes(8, "little") + b"\x01" * 8)
    with pytest.raises(native.GbbfsError):
        native.make_graph(filename=p)
    with open(p, "wb") as f:
        f.write(b"\x01" + (0).to_bytes(8, "little") + (1).to_bytes(8, "little") + b"\x00" * 16)
    with pytest.raises(native.GbbfsError):   # directed .sg
        native.make_graph(filename=p)


def test_edge_list_files(native, tmp_path):
    rng = np.random.default_rng(1)
    edges = rng.integers(0, 60, size=(400, 2))
    el = tmp_path / "g.el"
    el.write_text("".join("%d %d\n" % (u, v) for u, v in edges))
    off, nbr = native.make_graph(filename=str(el), symmetrize=True)
    ro, rn = _reference_csr(edges)
    assert np.array_equal(off, ro) and np.array_equal(nbr, rn)
    wel = tmp_path / "g.wel"
    wel.write_text("".join("%d %d 7\n" % (u, v) for u, v in edges))
    o2, n2 = native.make_graph(filename=str(wel), symmetrize=True)
    assert np.array_equal(o2, ro) and np.array_equal(n2, rn)
    gr = tmp_path / "g.gr"
    gr.write_text("c comment\np sp 60 400\n" +
                  "".join("a %d %d 3\n" % (u + 1, v + 1) for u, v in edges))
    o3, n3 = native.make_graph(filename=str(gr), symmetrize=True)
    assert np.array_equal(o3, ro) and np.array_equal(n3, rn)
    with pytest.raises(native.GbbfsError):   # directed edge lists are not served
        native.make_graph(filename=str(el), symmetrize=False)


def test_matrix_market_files(native, tmp_path):
    rng = np.random.default_rng(2)
    edges = rng.integers(0, 50, size=(300, 2))
    ro, rn = _reference_csr(edges)
    body = "".join("%d %d\n" % (u + 1, v + 1) for u, v in edges)
    gen = tmp_path / "g.mtx"
    gen.write_text("%%MatrixMarket matrix coordinate pattern general\n% a comment\n"
                   "50 50 300\n" + body)
    off, nbr = native.make_graph(filename=str(gen), symmetrize=True)
    assert np.array_equal(off[:len(ro)], ro) and np.array_equal(nbr, rn)
    with pytest.raises(native.GbbfsError):   # general = directed: needs -s
        native.make_graph(filename=str(gen), symmetrize=False)
    # a symmetric file lists each edge once; weights are ignored
    sym = tmp_path / "s.mtx"
    sym.write_text("%%MatrixMarket matrix coordinate real symmetric\n50 50 300\n" +
                   "".join("%d %d 0.5\n" % (u + 1, v + 1) for u, v in edges))
    o2, n2 = native.make_graph(filename=str(sym), symmetrize=False)
    assert np.array_equal(o2, off) and np.array_equal(n2, nbr)
    for bad in ("%%MatrixMarket matrix coordinate complex general\n50 50 1\n1 2 1 1\n",
                "%%MatrixMarket matrix array real general\n50 50 1\n1 2 1\n",
                "%%MatrixMarket matrix coordinate pattern general\n50 40 1\n1 2\n",
                "not a header\n"):
        f = tmp_path / "bad.mtx"
        f.write_text(bad)
        with pytest.raises(native.GbbfsError):
            native.make_graph(filename=str(f), symmetrize=True)


def test_bfs_output_writer(native, tmp_path):
    p = str(tmp_path / "bfs_output.txt")
    a = np.array([3, -1, -7, 0, 2147483647, -2147483648], np.int32)
    native.write_bfs_output(p, a)
    native.write_bfs_output(p, a[:2])
    lines = open(p).read().split("\n")
    assert lines[-1] == ""
    assert lines[:-1] == ["3", "-1", "-1", "0", "2147483647", "-1", "3", "-1"]


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "gbbfs.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbbfs_\w+)\s*\(", src)))


def test_abi_exports_every_declared_symbol(native):
    declared = _declared_functions()
    assert set(declared) == set(native.EXPORTS)
    L = native.lib()
    for name in declared:
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (gbbfs_\w+)", out))
    assert set(declared) <= exported


def test_strerror(native):
    L = native.lib()
    assert L.gbbfs_strerror(0) == b"ok"
    assert L.gbbfs_strerror(native.ERR_NOMEM) == b"not enough device memory"
    assert L.gbbfs_strerror(99) == b"unknown status"


def test_graph_create_rejects_bad_csr(native):
    # Argument checks run before any CUDA call.
    with pytest.raises(native.GbbfsError) as e:
        native.Graph(np.array([1, 2], np.int64), np.array([0, 0], np.int32))
    assert e.value.status == native.ERR_ARG


def test_cli_usage_and_missing_input(native):
    r = subprocess.run([native.CLI_PATH], capture_output=True, text=True)
    assert r.returncode == 255
    assert "No graph input specified" in r.stdout
    r = subprocess.run([native.CLI_PATH, "-h"], capture_output=True, text=True)
    assert r.returncode == 0
    assert " -u <scale>  : generate 2^scale uniform-random graph" in r.stdout
    assert "[16]" in r.stdout


def test_edge_list_files_malformed(native, tmp_path):
    """Edge-list parsing: CRLF endings, blank, indented and comment lines are
    accepted; a record with one number, a negative id, an empty file, an
    unknown suffix and a missing file are refused."""
    good = tmp_path / "crlf.el"
    good.write_bytes(b"# header\r\n\r\n  0 1\r\n\t1 2\r\n% note\r\n2 0\r\n")
    off, nbr = native.make_graph(filename=str(good), symmetrize=True)
    ro, rn = _reference_csr(np.array([[0, 1], [1, 2], [2, 0]]))
    assert np.array_equal(off, ro) and np.array_equal(nbr, rn)
    for name, body in (("one.el", "0 1\n7\n"), ("neg.el", "0 1\n-2 3\n"),
                       ("empty.el", ""), ("neg.gr", "a 0 1 5\n")):
        f = tmp_path / name
        f.write_text(body)
        with pytest.raises(native.GbbfsError) as e:
            native.make_graph(filename=str(f), symmetrize=True)
        assert e.value.status == native.ERR_IO, name
    for name in ("g.txt", "g.wsg"):   # unknown suffix; weighted serialized graph
        other = tmp_path / name
        other.write_text("0 1\n")
        with pytest.raises(native.GbbfsError) as e:
            native.make_graph(filename=str(other), symmetrize=True)
        assert e.value.status == native.ERR_ARG, name
    with pytest.raises(native.GbbfsError) as e:
        native.make_graph(filename=str(tmp_path / "missing.el"), symmetrize=True)
    assert e.value.status == native.ERR_IO


def test_abi_argument_checks_without_a_gpu(native):
    """Calls that fail on their arguments fail before any CUDA call."""
    L = native.lib()
    # the batched state's size: a pure function of the graph's shape
    b1 = native.msbfs_state_bytes(1 << 20, 1 << 24, 1)
    b4 = native.msbfs_state_bytes(1 << 20, 1 << 24, 4)
    assert 0 < b1 < b4 < native.msbfs_state_bytes(1 << 21, 1 << 24, 4)
    assert native.msbfs_state_bytes(1 << 20, 1 << 25, 1) - b1 == 4 * (1 << 24)
    assert L.gbbfs_msbfs_state_bytes(-1, 0, 1) == -1
    assert L.gbbfs_msbfs_state_bytes(10, 10, 2) == -1
    assert L.gbbfs_msbfs_order(None, None, 0, None) == native.ERR_ARG
    assert L.gbbfs_msbfs_autotune(None, None, 1, 1, None) == native.ERR_ARG
    assert L.gbbfs_bfs_many(None, None, 1, 15, 18, None, None) == native.ERR_ARG
    # server configurations outside the documented values
    for cfg in (dict(mode=2), dict(order=3), dict(batches_only=2)):
        with pytest.raises(native.GbbfsError) as e:
            native.Server(**cfg)
        assert e.value.status == native.ERR_ARG

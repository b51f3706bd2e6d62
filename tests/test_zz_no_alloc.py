"""gbbfs_bfs_noalloc, the search for callers that cannot allocate device
memory, against the regular entry point gbbfs_bfs.

Both entry points run through the C ABI.  The inputs and outputs of the
no-allocation call are device buffers this test owns (torch tensors, used only
as device memory).  Depths must agree bit for bit.  Parent trees may differ
where top-down claims race, so each one must pass the BFSVerifier
restatement.  Two calls in a row show that the shared scratch array carries
nothing from one call into the next.  This file runs last in the suite (its
name sorts last), and it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from conftest import config_args

pytestmark = pytest.mark.gpu


def _device_csr(torch, off, nbr):
    d_off = torch.from_numpy(np.ascontiguousarray(off, np.int64)).cuda()
    d_nbr = torch.from_numpy(np.ascontiguousarray(nbr, np.int32)).cuda()
    return d_off, d_nbr


def _noalloc(native, torch, d_off, d_nbr, n, m, src):
    parent = torch.empty(n, dtype=torch.int32, device="cuda")
    depth = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = native.lib().gbbfs_bfs_noalloc(
        ctypes.c_void_p(d_off.data_ptr()), ctypes.c_void_p(d_nbr.data_ptr()), n, m, int(src),
        15, 18, ctypes.c_void_p(parent.data_ptr()), ctypes.c_void_p(depth.data_ptr()), None)
    assert rc == native.OK, native.lib().gbbfs_last_error()
    return parent.cpu().numpy(), depth.cpu().numpy()


@pytest.mark.parametrize("name", ["u15", "g15", "g16k8"])
def test_noalloc_matches_gbbfs_bfs(native, oracle, golden, name):
    torch = pytest.importorskip("torch")
    off, nbr = native.make_graph(*config_args(golden[name]["flags"]))
    n, m = len(off) - 1, len(nbr)
    d_off, d_nbr = _device_csr(torch, off, nbr)
    srcs = [int(s) for s in native.pick_sources(off, 3)]
    with native.Graph(off, nbr) as g:
        # two different sources back to back, then the first one again
        for src in (srcs[0], srcs[1], srcs[0]):
            p_new, d_new = _noalloc(native, torch, d_off, d_nbr, n, m, src)
            p_ref, d_ref = native.DOBFS(g, src, depth=True)
            assert np.array_equal(d_new, d_ref)
            assert np.array_equal(d_new, oracle.depth(off, nbr, src))
            assert oracle.verify(off, nbr, src, p_new)[0]
            assert oracle.verify(off, nbr, src, p_ref)[0]
            assert p_new[src] == src


def test_noalloc_depth_optional_and_ragged(native, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    off, nbr = native.build_csr(rng.integers(0, 1001, size=(4000, 2)).astype(np.int32),
                                num_nodes=1003)             # n not a multiple of 32
    n, m = len(off) - 1, len(nbr)
    d_off, d_nbr = _device_csr(torch, off, nbr)
    parent = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    src = int(native.pick_sources(off, 1)[0])
    rc = native.lib().gbbfs_bfs_noalloc(
        ctypes.c_void_p(d_off.data_ptr()), ctypes.c_void_p(d_nbr.data_ptr()), n, m, src, 0, 0,
        ctypes.c_void_p(parent.data_ptr()), None, None)
    assert rc == native.OK
    p = parent.cpu().numpy()
    assert oracle.verify(off, nbr, src, p)[0]
    with native.Graph(off, nbr) as g:
        _, d_ref = native.DOBFS(g, src, depth=True)
    assert np.array_equal(p >= 0, d_ref >= 0)


def test_noalloc_rejects_oversize_and_bad_source(native):
    torch = pytest.importorskip("torch")
    off, nbr = native.make_graph(10, 16, True)
    d_off, d_nbr = _device_csr(torch, off, nbr)
    parent = torch.empty(len(off) - 1, dtype=torch.int32, device="cuda")
    L = native.lib()
    args = (ctypes.c_void_p(d_off.data_ptr()), ctypes.c_void_p(d_nbr.data_ptr()))
    rc = L.gbbfs_bfs_noalloc(*args, (1 << 18) + 1, len(nbr), 0, 15, 18,
                             ctypes.c_void_p(parent.data_ptr()), None, None)
    assert rc == native.ERR_ARG
    assert b"262144" in L.gbbfs_last_error()
    rc = L.gbbfs_bfs_noalloc(*args, len(off) - 1, len(nbr), len(off) + 4, 15, 18,
                             ctypes.c_void_p(parent.data_ptr()), None, None)
    assert rc == native.ERR_ARG


def _driver():
    """The CUDA driver library, for stream capture without any other package."""
    for name in ("libcuda.so.1", "libcuda.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            pass
    pytest.skip("libcuda not found")


def test_noalloc_allocates_nothing(native, oracle):
    """Device free memory is the same before and after a call (the kernels it
    launches were loaded by the same call just before)."""
    torch = pytest.importorskip("torch")
    off, nbr = native.make_graph(14, 16, False)
    n, m = len(off) - 1, len(nbr)
    d_off, d_nbr = _device_csr(torch, off, nbr)
    src = int(native.pick_sources(off, 1)[0])
    _noalloc(native, torch, d_off, d_nbr, n, m, src)
    _noalloc(native, torch, d_off, d_nbr, n, m, src)
    parent = torch.empty(n, dtype=torch.int32, device="cuda")
    depth = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rc = native.lib().gbbfs_bfs_noalloc(
        ctypes.c_void_p(d_off.data_ptr()), ctypes.c_void_p(d_nbr.data_ptr()), n, m, src, 15, 18,
        ctypes.c_void_p(parent.data_ptr()), ctypes.c_void_p(depth.data_ptr()), None)
    assert rc == native.OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert np.array_equal(depth.cpu().numpy(), oracle.depth(off, nbr, src))


def test_noalloc_refuses_a_capturing_stream(native):
    """The call synchronises its stream after every step, so on a stream under
    capture it must return GBBFS_ERR_STATE and leave the capture untouched."""
    torch = pytest.importorskip("torch")
    off, nbr = native.make_graph(10, 16, True)
    n, m = len(off) - 1, len(nbr)
    d_off, d_nbr = _device_csr(torch, off, nbr)
    parent = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    cu = _driver()
    stream, graph = ctypes.c_void_p(), ctypes.c_void_p()
    assert cu.cuStreamCreate(ctypes.byref(stream), 1) == 0          # non-blocking
    try:
        assert cu.cuStreamBeginCapture_v2(stream, 1) == 0           # thread-local mode
        rc = native.lib().gbbfs_bfs_noalloc(
            ctypes.c_void_p(d_off.data_ptr()), ctypes.c_void_p(d_nbr.data_ptr()), n, m, 0,
            15, 18, ctypes.c_void_p(parent.data_ptr()), None, stream)
        err = native.lib().gbbfs_last_error()
        assert cu.cuStreamEndCapture(stream, ctypes.byref(graph)) == 0   # still valid
        assert rc == native.ERR_STATE and b"captured" in err
        nodes = ctypes.c_size_t(99)
        assert cu.cuGraphGetNodes(graph, None, ctypes.byref(nodes)) == 0
        assert nodes.value == 0                                     # nothing was enqueued
        cu.cuGraphDestroy(graph)
    finally:
        cu.cuStreamDestroy_v2(stream)

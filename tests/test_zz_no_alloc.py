"""gu_bfs_noalloc: the multi-source BFS entry point that allocates no device memory.

It serves callers that may not call cudaMalloc while they search (their process's
allocator owns the GPU's memory, their budget is fixed at start-up, or they cannot
pay for cudaMalloc's implicit synchronisation).  It keeps its scratch in a fixed
array compiled into the library and works on the caller's own device CSR.

The test calls it through the C ABI, twice in a row on the same device (the
second call finds the first call's leftovers in the shared scratch), and checks
each result against the existing entry point gu_bfs, which allocates its own
workspace, and against the oracle (the C restatement of the reference's CPU
BFS, examples/multi_search/multi_search_test.cu:17-38).  Distances are
integers: the comparisons are exact.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import gu
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _noalloc(R_dev, C_dev, n, m, src_dev, dist_dev, ld):
    L = gu.lib()
    return L.gu_bfs_noalloc(ctypes.c_void_p(R_dev.data_ptr()), ctypes.c_void_p(C_dev.data_ptr() if m else 0),
                            n, m, ctypes.c_void_p(src_dev.data_ptr()), int(src_dev.numel()),
                            ctypes.c_void_p(dist_dev.data_ptr()), ld, None)


def _reference_rows(hg, srcs):
    g = gu.Graph(hg)
    s = torch.as_tensor(srcs, device="cuda")
    out = torch.empty((len(srcs), hg.n), dtype=torch.int32, device="cuda")
    g.bfs(s, out, variant="auto")
    torch.cuda.synchronize()
    g.close()
    return out.cpu().numpy()


@pytest.mark.parametrize("kind", ["rmat", "dag"])
def test_noalloc_matches_gu_bfs_twice(kind):
    if kind == "rmat":
        hg = gu.HostGraph.rmat(14, 16, seed=7)        # 16384 vertices, undirected
    else:
        hg = gu.HostGraph.dag(20000, 160000, seed=5)  # directed
    dev = torch.device("cuda:0")
    R = torch.as_tensor(hg.R, device=dev)
    C = torch.as_tensor(hg.C, device=dev)
    for call, (k, seed) in enumerate([(150, 2), (70, 9)]):   # two calls in a row
        srcs = gu.sources(hg.n, k, seed=seed)
        s = torch.as_tensor(srcs, device=dev)
        ld = hg.n + 5
        dist = torch.full((k, ld), -3, dtype=torch.int32, device=dev)
        st = _noalloc(R, C, hg.n, hg.m, s, dist, ld)
        assert st == gu.OK, gu.lib().gu_last_error().decode()
        torch.cuda.synchronize()
        got = dist.cpu().numpy()
        np.testing.assert_array_equal(got[:, :hg.n], _reference_rows(hg, srcs), err_msg=f"call {call}")
        ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
        np.testing.assert_array_equal(got[:, :hg.n], ref, err_msg=f"call {call} vs oracle")
        assert np.all(got[:, hg.n:] == -3)


def test_noalloc_rejects_without_launching():
    dev = torch.device("cuda:0")
    L = gu.lib()
    # too many vertices for the static scratch
    big = gu.HostGraph.rmat(16, 4, seed=1)
    R = torch.as_tensor(big.R, device=dev)
    C = torch.as_tensor(big.C, device=dev)
    s = torch.zeros(4, dtype=torch.int32, device=dev)
    d = torch.zeros((4, big.n), dtype=torch.int32, device=dev)
    assert _noalloc(R, C, big.n, big.m, s, d, big.n) == 4  # GU_ERR_CAPACITY
    assert b"32768" in L.gu_last_error()
    # a source out of range
    hg = gu.HostGraph.rmat(10, 8, seed=1)
    R = torch.as_tensor(hg.R, device=dev)
    C = torch.as_tensor(hg.C, device=dev)
    s = torch.tensor([0, hg.n], dtype=torch.int32, device=dev)
    d = torch.zeros((2, hg.n), dtype=torch.int32, device=dev)
    assert _noalloc(R, C, hg.n, hg.m, s, d, hg.n) == 1    # GU_ERR_INVALID_ARGUMENT
    assert b"source" in L.gu_last_error()

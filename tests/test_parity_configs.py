"""Parity at the benchmark configurations' full sizes, against the oracle.

* R-MAT scale 20, edge factor 16, 512 sources (the headline BFS workload): every
  one of the 512 distance rows equals the oracle's (the C restatement of
  examples/multi_search/multi_search_test.cu:17-38), bit for bit.
* R-MAT scale 18, edge factor 16 (the sampled-BC workload): the first 1024 of its
  8192 sources, FP64 Brandes BC at 64, 256 and 1024 sources per pass, within
  1e-12 relative of the FP64 oracle (examples/betweenness_centrality/bc.cu:11-57
  with double delta); sigma (uint64) of the first 256 sources bit-exact.
* 2048 x 2048 grid with 5 % of the edges deleted (seed 7), 256 sources: all 256
  rows of AUTO (the per-source engine) and of the batched bit-matrix engine equal
  the oracle's, and the diameter over the sources is the oracle's.

The oracle runs on all host threads, 64 rows at a time, so that host memory
stays at a few hundred MB per chunk.
"""
import os

import numpy as np
import pytest

import gu
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
RTOL = 1e-12
CORES = os.cpu_count() or 1


def _rows_equal_oracle(hg, srcs, dist, chunk=64):
    """Every row of the device tensor dist equals the oracle's, compared chunk by chunk."""
    for b in range(0, len(srcs), chunk):
        ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs[b:b + chunk], nthreads=CORES)
        got = dist[b:b + chunk].cpu().numpy()
        if not np.array_equal(got, ref):
            r, v = np.argwhere(got != ref)[0]
            raise AssertionError(f"row {b + r} (source {srcs[b + r]}) vertex {v}: got {got[r, v]}, "
                                 f"oracle {ref[r, v]}")


def test_rmat20_all_512_rows():
    hg = gu.HostGraph.rmat(20, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 512, seed=2)
    s = torch.as_tensor(srcs, device="cuda")
    dist = torch.empty((512, hg.n), dtype=torch.int32, device="cuda")
    g.bfs(s, dist, variant="auto")
    torch.cuda.synchronize()
    _rows_equal_oracle(hg, srcs, dist)
    g.close()
    del dist
    torch.cuda.empty_cache()


@pytest.fixture(scope="module")
def rmat18():
    hg = gu.HostGraph.rmat(18, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    srcs = gu.sources(hg.n, 8192, seed=2)[:1024]
    ref = oracle.bc(hg.R, hg.C, hg.n, srcs, nthreads=CORES)
    return hg, srcs, ref


def _max_rel(got, ref):
    scale = np.maximum(np.abs(ref), 1e-300)
    rel = np.abs(got - ref) / scale
    rel[np.abs(got - ref) <= 1e-300] = 0.0
    return float(rel.max()), int(np.argmax(rel))


@pytest.mark.parametrize("batch", [64, 256, 1024])
def test_rmat18_bc_1024_sources(rmat18, batch):
    hg, srcs, ref = rmat18
    g = gu.Graph(hg)
    s = torch.as_tensor(srcs, device="cuda")
    bc = torch.empty(hg.n, dtype=torch.float64, device="cuda")
    g.bc(s, bc, batch=batch)
    torch.cuda.synchronize()
    got = bc.cpu().numpy()
    err, at = _max_rel(got, ref)
    assert err <= RTOL, f"batch {batch}: max relative error {err:.3e} at vertex {at}"
    g.bc(s, bc, batch=batch)
    torch.cuda.synchronize()
    assert np.array_equal(bc.cpu().numpy().view(np.uint64), got.view(np.uint64)), "repeat differs"
    g.close()


def test_rmat18_sigma_256_sources(rmat18):
    hg, srcs, _ = rmat18
    g = gu.Graph(hg)
    k = 256
    s = torch.as_tensor(srcs[:k], device="cuda")
    sig = torch.empty((k, hg.n), dtype=torch.int64, device="cuda")
    d = torch.empty((k, hg.n), dtype=torch.int32, device="cuda")
    g.sigma(s, sig, dist_dev=d)
    torch.cuda.synchronize()
    for b in range(0, k, 64):
        rd, rs = oracle.sigma_multi(hg.R, hg.C, hg.n, srcs[b:b + 64], nthreads=CORES)
        np.testing.assert_array_equal(d[b:b + 64].cpu().numpy(), rd, err_msg=f"distances, rows {b}..")
        np.testing.assert_array_equal(sig[b:b + 64].cpu().numpy().view(np.uint64), rs,
                                      err_msg=f"sigma, rows {b}..")
    g.close()


@pytest.mark.parametrize("engine", ["auto", "batched"])
def test_grid2048_all_256_rows(engine, monkeypatch):
    if engine == "batched":
        monkeypatch.setenv("GU_AUTO_LOCAL", "0")
    hg = gu.HostGraph.grid(2048, 2048, 0.05, seed=7)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 256, seed=2)
    s = torch.as_tensor(srcs, device="cuda")
    dist = torch.empty((256, hg.n), dtype=torch.int32, device="cuda")
    g.bfs(s, dist, variant="auto")
    torch.cuda.synchronize()
    _rows_equal_oracle(hg, srcs, dist)
    if engine == "auto":
        assert g.diameter(s) == oracle.diameter(hg.R, hg.C, hg.n, srcs, nthreads=CORES)
    g.close()
    del dist
    torch.cuda.empty_cache()

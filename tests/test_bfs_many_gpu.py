"""gu_bfs_many: many searches on many graphs in one work-queue launch.

CTA groups of one persistent grid drain a device queue of (graph, block of up to
256 sources) items.  Every request's rows and counts must equal the oracle's
(the C restatement of examples/multi_search/multi_search_test.cu:17-38 and
reachability.cu:11-33) bit for bit, whatever else shares the launch.
"""
import numpy as np
import pytest

import gu
import oracle
from conftest import load_golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
INF = gu.UNREACHABLE


@pytest.fixture(scope="module")
def graphs():
    d = load_golden("jazz")
    hgs = {"rmat14": gu.HostGraph.rmat(14, 16, seed=9),
           "rmat10_ef4": gu.HostGraph.rmat(10, 4, seed=3),     # degree-0 vertices
           "rmat16_ef8": gu.HostGraph.rmat(16, 8, seed=5),
           "dag5000": gu.HostGraph.dag(5000, 40000, seed=4),   # directed
           "grid96x80": gu.HostGraph.grid(96, 80, 0.05, seed=7),  # high diameter
           "jazz": gu.HostGraph(d["R"], d["C"], int(d["n"]), bool(d["directed"]))}
    return {k: (hg, gu.Graph(hg)) for k, hg in hgs.items()}


def _request(hg, g, k, seed, rows=True, counts=False, pad=0):
    srcs = gu.sources(hg.n, k, seed=seed)
    s = torch.as_tensor(srcs, device="cuda")
    d = torch.full((k, hg.n + pad), -7, dtype=torch.int32, device="cuda") if rows else None
    r = torch.full((k,), -1, dtype=torch.int64, device="cuda") if counts else None
    return srcs, (g, s, d, r)


def test_many_graphs_one_launch_equal_the_oracle(graphs):
    plan = [("rmat14", 300, 1, True, False, 0), ("rmat10_ef4", 37, 2, True, True, 5), ("dag5000", 100, 3, True, True, 0),
            ("grid96x80", 70, 4, True, False, 3), ("jazz", 198, 5, True, True, 0), ("rmat16_ef8", 700, 6, False, True, 0),
            ("rmat14", 1, 7, True, True, 0), ("dag5000", 256, 8, False, True, 0)]
    reqs, meta = [], []
    for name, k, seed, rows, counts, pad in plan:
        hg, g = graphs[name]
        srcs, req = _request(hg, g, k, seed, rows, counts, pad)
        reqs.append(req)
        meta.append((name, hg, srcs, pad))
    for rep in range(2):  # the second launch finds the first one's leftovers in the workspace
        gu.bfs_many(reqs)
        torch.cuda.synchronize()
        for (name, hg, srcs, pad), (g, s, d, r) in zip(meta, reqs):
            ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
            if d is not None:
                got = d.cpu().numpy()
                np.testing.assert_array_equal(got[:, :hg.n], ref, err_msg=f"{name} rows, launch {rep}")
                assert np.all(got[:, hg.n:] == -7), f"{name}: padding beyond n untouched"
            if r is not None:
                np.testing.assert_array_equal(r.cpu().numpy(), (ref != INF).sum(1), err_msg=f"{name} counts, launch {rep}")


def test_same_results_as_one_graph_calls(graphs):
    hg, g = graphs["rmat14"]
    srcs, req = _request(hg, g, 513, 11)
    gu.bfs_many([req])
    alone = torch.empty_like(req[2])
    g.bfs(req[1], alone, variant="auto")
    torch.cuda.synchronize()
    assert torch.equal(req[2], alone)


def test_errors_and_empty(graphs):
    hg, g = graphs["rmat10_ef4"]
    gu.bfs_many([])  # nothing to do
    s = torch.tensor([0, hg.n, 3], dtype=torch.int32, device="cuda")
    d = torch.zeros((3, hg.n), dtype=torch.int32, device="cuda")
    with pytest.raises(gu.GuError) as e:
        gu.bfs_many([(g, s, d, None)])
    assert e.value.status == 1
    with pytest.raises(gu.GuError) as e:
        gu.bfs_many([(g, s[:1], None, None)])  # no output
    assert e.value.status == 1
    # the handles stay usable
    hg2, g2 = graphs["jazz"]
    srcs, req = _request(hg2, g2, 50, 3)
    gu.bfs_many([req, (g, torch.zeros(0, dtype=torch.int32, device="cuda"), d, None)])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(req[2].cpu().numpy(), oracle.bfs_multi(hg2.R, hg2.C, hg2.n, srcs)[0])

"""The continuous-batching server: every result in the mix equals the same request alone.

Requests of three kinds (BFS rows, BC over a source set, reachable counts on a
DAG) against three device-resident graphs are submitted from several host
threads with random gaps, so batches form while others run.  BFS rows and
reach counts must be bit-identical to a lone call; BC within 1e-12 relative.
"""
import threading
import time

import numpy as np
import pytest

import gu
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def lone_bfs(g, srcs):
    s = torch.as_tensor(np.asarray(srcs, np.int32), device="cuda")
    d = torch.empty((len(srcs), g.n), dtype=torch.int32, device="cuda")
    g.bfs(s, d)
    return d.cpu().numpy()


def lone_bc(g, srcs):
    s = torch.as_tensor(np.asarray(srcs, np.int32), device="cuda")
    bc = torch.empty(g.n, dtype=torch.float64, device="cuda")
    g.bc(s, bc)
    return bc.cpu().numpy()


@pytest.fixture(scope="module")
def graphs():
    return {"rmat12": gu.Graph(gu.HostGraph.rmat(12, 16, seed=21)),
            "rmat13": gu.Graph(gu.HostGraph.rmat(13, 8, seed=22)),
            "dag": gu.Graph(gu.HostGraph.dag(20000, 160000, seed=23))}


def test_results_alone_and_in_the_mix(graphs):
    srv = gu.Server(hbm_budget_bytes=16 << 30, slots=4, max_batch=256)
    rng = np.random.default_rng(7)
    plan = []
    for i in range(72):
        kind = rng.choice(["bfs", "bc", "reach"], p=[0.5, 0.25, 0.25])
        if kind == "reach":
            gname = "dag"
        else:
            gname = rng.choice(["rmat12", "rmat13"])
        g = graphs[gname]
        k = int(rng.integers(1, 65 if kind != "bc" else 41))
        srcs = rng.choice(g.n, size=k, replace=False).astype(np.int32)
        plan.append((kind, gname, srcs, float(rng.exponential(0.002))))
    results = [None] * len(plan)
    errors = []

    def client(idx):
        try:
            for i in idx:
                kind, gname, srcs, gap = plan[i]
                g = graphs[gname]
                time.sleep(gap)
                if kind == "bfs":
                    out, q = np.empty((len(srcs), g.n), np.int32), gu.QUERY_BFS
                elif kind == "bc":
                    out, q = np.empty(g.n, np.float64), gu.QUERY_BC
                else:
                    out, q = np.empty(len(srcs), np.int64), gu.QUERY_REACH
                rid = srv.submit(g, q, srcs, out)
                results[i] = (rid, out)
        except Exception as e:  # surfaced below
            errors.append(e)

    threads = [threading.Thread(target=client, args=(list(range(t, len(plan), 4)),)) for t in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    lat = [srv.wait(rid) for rid, _ in results]
    assert all(x is not None and x >= 0 for x in lat)
    st = srv.stats()
    assert st["completed"] == len(plan)
    assert st["batches"] <= len(plan), st
    for i, (kind, gname, srcs, _) in enumerate(plan):
        g = graphs[gname]
        out = results[i][1]
        if kind == "bfs":
            np.testing.assert_array_equal(out, lone_bfs(g, srcs), err_msg=f"request {i}")
        elif kind == "reach":
            rows = lone_bfs(g, srcs)
            np.testing.assert_array_equal(out, (rows != gu.UNREACHABLE).sum(1), err_msg=f"request {i}")
            assert out[0] == oracle.reach_count(g.host.R, g.host.C, g.n, srcs[:1])
        else:
            ref = lone_bc(g, srcs)
            rel = np.abs(out - ref) / np.maximum(np.abs(ref), 1e-300)
            assert np.all((rel <= 1e-12) | (np.abs(out - ref) == 0)), f"request {i}: {rel.max()}"
    srv.close()


def test_queued_requests_share_a_batch(graphs):
    """With one slot, requests submitted while a batch runs are merged into the next one."""
    g = graphs["rmat13"]
    srv = gu.Server(hbm_budget_bytes=16 << 30, slots=1, max_batch=256)
    rng = np.random.default_rng(11)
    reqs = []
    for i in range(48):
        srcs = rng.choice(g.n, size=4, replace=False).astype(np.int32)
        out = np.empty((4, g.n), np.int32)
        reqs.append((srv.submit(g, gu.QUERY_BFS, srcs, out), srcs, out))
    for rid, _, _ in reqs:
        srv.wait(rid)
    st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["batches"] < len(reqs), st  # the burst did not run one request per batch
    for _, srcs, out in reqs:
        np.testing.assert_array_equal(out, lone_bfs(g, srcs))
    srv.close()


def test_admission_by_hbm_budget(graphs):
    g = graphs["rmat13"]
    srv = gu.Server(hbm_budget_bytes=1 << 20, slots=2, max_batch=64)  # 1 MiB: nothing fits
    out = np.empty((4, g.n), np.int32)
    rid = srv.submit(g, gu.QUERY_BFS, np.arange(4, dtype=np.int32), out)
    with pytest.raises(gu.GuError) as e:
        srv.wait(rid)
    assert e.value.status == 4  # GU_ERR_CAPACITY
    srv.close()


def test_bad_request_rejected(graphs):
    srv = gu.Server(slots=1)
    g = graphs["rmat12"]
    with pytest.raises(gu.GuError):
        srv.submit(g, gu.QUERY_BFS, np.array([g.n], np.int32), np.empty((1, g.n), np.int32))
    srv.close()


def test_page_touching_stays_inside_the_buffers(graphs):
    """The helper threads touch each request's host buffer while its batch runs; on
    buffers that start and end inside pages shared with other data, the bytes around
    them must keep their values (results land exactly in the buffers)."""
    g = graphs["rmat13"]
    srv = gu.Server(hbm_budget_bytes=16 << 30, slots=2, max_batch=256)
    rng = np.random.default_rng(3)
    reqs = []
    for i in range(6):
        k = int(rng.integers(1, 9))
        srcs = rng.choice(g.n, size=k, replace=False).astype(np.int32)
        words = k * g.n
        arena = np.full(words + 4096 + 3, -123, np.int32)  # guard words on both sides
        off = 1 + int(rng.integers(0, 1000))                 # start inside a page
        out = arena[off:off + words].reshape(k, g.n)
        reqs.append((srv.submit(g, gu.QUERY_BFS, srcs, out), srcs, out, arena, off, words))
    for rid, srcs, out, arena, off, words in reqs:
        srv.wait(rid)
        np.testing.assert_array_equal(out, lone_bfs(g, srcs))
        assert (arena[:off] == -123).all() and (arena[off + words:] == -123).all()
    srv.close()


def test_requests_on_different_graphs_share_a_launch(graphs):
    """With the only slot busy, BFS and reachability requests on three graphs queue
    up; they then run as one work-queue launch (one batch for all of them), and
    each result equals the oracle's."""
    srv = gu.Server(hbm_budget_bytes=16 << 30, slots=1, max_batch=4096)
    big = graphs["rmat13"]
    hold = np.empty(big.n, np.float64)
    rid0 = srv.submit(big, gu.QUERY_BC, np.arange(0, 1024, dtype=np.int32), hold)  # keeps the slot busy
    rng = np.random.default_rng(3)
    reqs = []
    for i in range(18):
        gname = ["rmat12", "rmat13", "dag"][i % 3]
        g = graphs[gname]
        k = int(rng.integers(1, 300))
        srcs = rng.choice(g.n, size=k, replace=False).astype(np.int32)
        if i % 2:
            out, q = np.empty((k, g.n), np.int32), gu.QUERY_BFS
        else:
            out, q = np.empty(k, np.int64), gu.QUERY_REACH
        reqs.append((srv.submit(g, q, srcs, out), gname, q, srcs, out))
    srv.wait(rid0)
    for rid, gname, q, srcs, out in reqs:
        srv.wait(rid)
        hg = graphs[gname].host
        ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
        if q == gu.QUERY_BFS:
            np.testing.assert_array_equal(out, ref, err_msg=gname)
        else:
            np.testing.assert_array_equal(out, (ref != gu.UNREACHABLE).sum(1), err_msg=gname)
    st = srv.stats()
    srv.close()
    assert st["completed"] == 19
    assert st["batches"] <= 3, st  # the BC request, then the queued searches together

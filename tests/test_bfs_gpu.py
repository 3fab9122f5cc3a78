"""Parity of the CUDA multi-source BFS (every variant) with the oracle.

Distances must be bit-exact.  Small cases compare against the golden vectors
of the reference's own checkers and against oracle/gu_oracle.c; the full-size
R-MAT scale-20 case is checked through BFS certificates that hold at any size.
"""
import os

import numpy as np
import pytest

import gu
import oracle
from conftest import golden_names, load_golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# "auto" lets AUTO pick its engine (the per-source one on small or low-degree
# graphs); "auto_batched" keeps AUTO on the batched bit-matrix engine
# (GU_AUTO_LOCAL=0), so both engines are checked on the same graphs.
VARIANTS = ["auto", "auto_batched", "linear", "edge", "warp", "cta_warp", "scan", "shuffle", "bottom_up", "plain"]


def run_bfs(g, srcs, variant, ld=None):
    dev = torch.device("cuda:0")
    s = torch.as_tensor(np.asarray(srcs, np.int32), device=dev)
    ld = g.n if ld is None else ld
    out = torch.full((max(len(srcs), 1), ld), -7, dtype=torch.int32, device=dev)
    if variant == "auto_batched":
        os.environ["GU_AUTO_LOCAL"] = "0"
        try:
            g.bfs(s, out, variant="auto", ld=ld)
        finally:
            del os.environ["GU_AUTO_LOCAL"]
    else:
        g.bfs(s, out, variant=variant, ld=ld)
    torch.cuda.synchronize()
    return out[: len(srcs), : g.n].cpu().numpy(), out.cpu().numpy()


@pytest.fixture(scope="module")
def golden_graphs():
    out = {}
    for name in golden_names():
        d = load_golden(name)
        hg = gu.HostGraph(d["R"], d["C"], int(d["n"]), bool(d["directed"]))
        out[name] = (gu.Graph(hg), d)
    return out


@pytest.mark.parametrize("variant", VARIANTS)
def test_golden_all_variants(golden_graphs, variant):
    for name, (g, d) in golden_graphs.items():
        got, _ = run_bfs(g, d["sources"], variant)
        np.testing.assert_array_equal(got, d["dist"], err_msg=f"{name}/{variant}")


@pytest.mark.parametrize("variant", VARIANTS)
def test_rmat14_vs_oracle(variant):
    hg = gu.HostGraph.rmat(14, 16, seed=9)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 150, seed=2)  # two full batches + a partial one
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    got, _ = run_bfs(g, srcs, variant)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("variant", ["auto", "auto_batched", "linear", "scan", "bottom_up", "plain"])
def test_grid_high_diameter_vs_oracle(variant):
    hg = gu.HostGraph.grid(96, 80, 0.05, seed=7)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 70, seed=2)
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    got, _ = run_bfs(g, srcs, variant)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("variant", ["auto", "auto_batched", "shuffle", "bottom_up", "edge"])
def test_directed_dag_vs_oracle(variant):
    hg = gu.HostGraph.dag(5000, 40000, seed=4)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 100, seed=2)
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    got, _ = run_bfs(g, srcs, variant)
    np.testing.assert_array_equal(got, ref)


def test_edge_cases():
    hg = gu.HostGraph.rmat(10, 4, seed=3)  # has degree-0 vertices
    g = gu.Graph(hg)
    deg = hg.degrees()
    zero = np.nonzero(deg == 0)[0]
    assert len(zero) > 0
    srcs = np.array([zero[0], 5, 5, zero[0], hg.n - 1, 0], np.int32)  # duplicates + isolated
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs)
    for v in VARIANTS:
        got, full = run_bfs(g, srcs, v, ld=hg.n + 13)
        np.testing.assert_array_equal(got, ref, err_msg=v)
        assert np.all(full[:, hg.n:] == -7), "padding beyond n untouched"
    # k = 0 is a no-op
    s = torch.zeros(0, dtype=torch.int32, device="cuda")
    out = torch.zeros((1, hg.n), dtype=torch.int32, device="cuda")
    g.bfs(s, out)
    # an out-of-range source is rejected: on the host before the launch for the
    # one-CTA-per-source and per-source engines, by the batched kernel itself
    # (which skips it) for the batched variants
    for v in ("auto", "plain", "warp", "shuffle", "bottom_up"):
        for bad in (hg.n, -1):
            s = torch.tensor([0, bad, 3], dtype=torch.int32, device="cuda")
            out = torch.zeros((3, hg.n), dtype=torch.int32, device="cuda")
            with pytest.raises(gu.GuError) as e:
                g.bfs(s, out, variant=v)
            assert e.value.status == 1, v
        # the graph handle stays usable
        got, _ = run_bfs(g, srcs, v)
        np.testing.assert_array_equal(got, ref, err_msg=v)


@pytest.mark.parametrize("engine", ["auto", "batched"])
@pytest.mark.parametrize("kind", ["rmat", "dag", "jazz"])
def test_reach_counts_vs_oracle(kind, engine, golden_graphs, monkeypatch):
    """gu_reach counts (source included) equal the oracle's reachable pairs per source."""
    if engine == "batched":
        monkeypatch.setenv("GU_AUTO_LOCAL", "0")
    if kind == "rmat":
        hg = gu.HostGraph.rmat(14, 8, seed=6)
        srcs = gu.sources(hg.n, 300, seed=7)  # two batches of the 256-source engine
    elif kind == "dag":
        hg = gu.HostGraph.dag(6000, 48000, seed=8)
        srcs = gu.sources(hg.n, 150, seed=9)
    else:
        d = golden_graphs["jazz"][1]
        hg = gu.HostGraph(d["R"], d["C"], int(d["n"]), bool(d["directed"]))
        srcs = np.arange(hg.n, dtype=np.int32)
    g = gu.Graph(hg)
    s = torch.as_tensor(srcs, device="cuda")
    cnt = torch.full((len(srcs),), -1, dtype=torch.int64, device="cuda")
    g.reach(s, cnt)
    got = cnt.cpu().numpy()
    ref = np.array([oracle.reach_count(hg.R, hg.C, hg.n, srcs[i:i + 1]) for i in range(len(srcs))])
    np.testing.assert_array_equal(got, ref)
    if kind == "jazz":
        assert got.sum() == 39204  # reachability.cu known answer: every ordered pair


def test_per_source_engine_overflow_falls_back():
    """A low-degree graph whose frontiers outgrow the per-source engine's shared
    queues (an expander: ER with mean degree 3) is rerun on the batched engine."""
    hg = gu.HostGraph.er(200000, 300000, seed=11)
    assert hg.degrees().max() <= 16  # AUTO picks the per-source engine first
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 40, seed=3)
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    got, _ = run_bfs(g, srcs, "auto")
    np.testing.assert_array_equal(got, ref)
    s = torch.as_tensor(srcs, device="cuda")
    assert g.diameter(s) == int(ref[ref != gu.UNREACHABLE].max())
    cnt = torch.empty(len(srcs), dtype=torch.int64, device="cuda")
    g.reach(s, cnt)
    np.testing.assert_array_equal(cnt.cpu().numpy(), (ref != gu.UNREACHABLE).sum(1))


def _layered_graph(width=5000, depth=6):
    """Undirected, out-degree <= 5: a binary tree from vertex 0 down to a layer of
    `width` vertices, then `depth` such layers joined vertex to vertex (and each
    vertex to its right-hand neighbour in the layer)."""
    u, v, layer, nxt = [], [], [0], 1
    while len(layer) < width:
        children = []
        for p in layer:
            for _ in range(2):
                if len(children) < width:
                    u.append(p)
                    v.append(nxt)
                    children.append(nxt)
                    nxt += 1
        layer = children
    for _ in range(depth):
        below = list(range(nxt, nxt + width))
        nxt += width
        u += layer + below[:-1]
        v += below + below[1:]
        layer = below
    return gu.HostGraph.from_edges(nxt, np.array(u), np.array(v))


def test_per_source_engine_wide_levels():
    """Levels of 5000 vertices, near the per-source engine's shared queue (6144):
    rows, counts and levels equal the oracle's, and so they do on the same graph
    cut to levels of 3000."""
    hg = _layered_graph()
    assert hg.degrees().max() <= 16 and not hg.directed
    g = gu.Graph(hg)
    srcs = np.concatenate([[0], gu.sources(hg.n, 63, seed=4)]).astype(np.int32)
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    assert np.bincount(ref[0][ref[0] != gu.UNREACHABLE]).max() == 5000  # from the root
    got, _ = run_bfs(g, srcs, "auto")
    np.testing.assert_array_equal(got, ref)
    s = torch.as_tensor(srcs, device="cuda")
    assert g.diameter(s) == int(ref[ref != gu.UNREACHABLE].max())
    cnt = torch.empty(len(srcs), dtype=torch.int64, device="cuda")
    g.reach(s, cnt)
    np.testing.assert_array_equal(cnt.cpu().numpy(), (ref != gu.UNREACHABLE).sum(1))
    # the same graph cut to levels of 3000
    hg2 = _layered_graph(width=3000)
    g2 = gu.Graph(hg2)
    ref2, _ = oracle.bfs_multi(hg2.R, hg2.C, hg2.n, srcs % hg2.n, nthreads=8)
    got2, _ = run_bfs(g2, srcs % hg2.n, "auto")
    np.testing.assert_array_equal(got2, ref2)


def test_host_form_matches_device_form():
    hg = gu.HostGraph.rmat(12, 16, seed=1)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 100, seed=5)
    dev, _ = run_bfs(g, srcs, "auto")
    host = g.bfs_host(srcs, "auto")
    np.testing.assert_array_equal(dev, host)


def test_rmat20_full_size_certificates():
    """R-MAT scale 20, 512 sources: per-edge BFS certificates on the GPU (they hold
    at any size and need no oracle)."""
    hg = gu.HostGraph.rmat(20, 16, seed=1)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 512, seed=2)
    dev = torch.device("cuda:0")
    s = torch.as_tensor(srcs, device=dev)
    dist = torch.empty((512, hg.n), dtype=torch.int32, device=dev)
    g.bfs(s, dist, variant="auto")
    R = torch.as_tensor(hg.R.astype(np.int64), device=dev)
    C = torch.as_tensor(hg.C.astype(np.int64), device=dev)
    src_of = torch.repeat_interleave(torch.arange(hg.n, device=dev), R[1:] - R[:-1])
    INF = gu.UNREACHABLE
    B = 8
    for b in range(0, 512, B):
        d = dist[b:b + B]
        du, dv = d[:, src_of], d[:, C]
        fin_u, fin_v = du != INF, dv != INF
        # an edge never joins reached and unreached vertices (undirected graph)
        assert torch.equal(fin_u, fin_v)
        # adjacent reached vertices differ by at most one level
        diff = torch.where(fin_u, (du - dv).abs(), torch.zeros_like(du))
        assert int(diff.max()) <= 1
        # every reached non-source vertex has a neighbour one level closer
        has = (fin_u & (du + 1 == dv)).to(torch.int32)
        parent = torch.zeros_like(d).scatter_reduce_(1, C.unsqueeze(0).expand(B, -1), has, reduce="amax")
        need = (d != INF) & (d > 0)
        assert bool(((parent > 0) | ~need).all())
        # no negative level, and level 0 exactly once per row: at the row's source
        assert bool((d >= 0).all())
        rows = torch.arange(b, b + B, device=dev)
        assert bool((d[torch.arange(B, device=dev), s[rows].long()] == 0).all())
        assert bool(((d == 0).sum(1) == 1).all())
        del du, dv, fin_u, fin_v, diff, has, parent
    # every row against the oracle: tests/test_parity_configs.py::test_rmat20_all_512_rows


def test_rows_beyond_2_31_elements():
    """2304 sources on R-MAT scale 20 (nine 256-source batches in one launch):
    the distance rows hold 2.4 G elements (9.7 GB), so row offsets pass 2^31
    elements.  Rows on both sides of that point, and the last row, equal the
    oracle's; every source is at level 0 of its own row."""
    hg = gu.HostGraph.rmat(20, 16, seed=1)
    g = gu.Graph(hg)
    k = 2304
    assert k * hg.n > 2 ** 31
    srcs = gu.sources(hg.n, k, seed=3)
    dev = torch.device("cuda:0")
    s = torch.as_tensor(srcs, device=dev)
    dist = torch.empty((k, hg.n), dtype=torch.int32, device=dev)
    g.bfs(s, dist, variant="auto")
    assert bool((dist[torch.arange(k, device=dev), s.long()] == 0).all())
    first_past = (2 ** 31) // hg.n  # the first row that starts beyond element 2^31
    sample = [0, 255, 256, first_past - 1, first_past, first_past + 1, k - 1]
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs[sample], nthreads=os.cpu_count() or 1)
    np.testing.assert_array_equal(dist[sample].cpu().numpy(), ref)
    del dist
    torch.cuda.empty_cache()


@pytest.mark.parametrize("shape", ["rmat", "grid"])
def test_autotune_keeps_distances(shape):
    """gu_graph_autotune times the candidates on a sample and makes the fastest AUTO's
    choice; distances after tuning (and under every explicitly set choice) equal the
    oracle's, and clearing the tuning restores the built-in choice."""
    hg = gu.HostGraph.rmat(13, 16, seed=9) if shape == "rmat" else gu.HostGraph.grid(96, 64, 0.05, seed=4)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 96, seed=6)
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    best, trials = g.autotune(torch.as_tensor(srcs, device="cuda"))
    engines = {t["engine"] for t in trials}
    assert "batched" in engines and best in trials
    assert ("per-source" in engines) == (shape == "grid")  # out-degree <= 16 only on the grid
    assert best["seconds"] == min(t["seconds"] for t in trials) > 0
    assert all(0 < t["seconds"] < 10 for t in trials)
    np.testing.assert_array_equal(run_bfs(g, srcs, "auto")[0], ref)
    for t in trials[:4]:
        g.set_tuning(t)
        np.testing.assert_array_equal(run_bfs(g, srcs, "auto")[0], ref, err_msg=str(t))
    with pytest.raises(gu.GuError):
        g.set_tuning({"engine": "batched", "alpha": 2.0, "beta": 24.0, "words": 3})
    # the grid's CTAs per SM is a tuning dimension too: one CTA per SM gives the same rows
    assert any(t["engine"] == "batched" and t["ctas_per_sm"] == 1 for t in trials)
    g.set_tuning({"engine": "batched", "alpha": 2.0, "beta": 24.0, "words": 0, "ctas_per_sm": 1})
    np.testing.assert_array_equal(run_bfs(g, srcs, "auto")[0], ref)
    with pytest.raises(gu.GuError):
        g.set_tuning({"engine": "batched", "alpha": 2.0, "beta": 24.0, "words": 0, "ctas_per_sm": 3})
    # and the fraction of sources left to top-down in bottom-up levels
    assert {round(t["rare_frac"], 3) for t in trials if t["engine"] == "batched"} >= {0.06, 0.15, 0.333}
    for rare in (0.0, 0.06, 1.0):
        g.set_tuning({"engine": "batched", "alpha": 2.0, "beta": 24.0, "words": 0, "rare_frac": rare})
        np.testing.assert_array_equal(run_bfs(g, srcs, "auto")[0], ref, err_msg=f"rare_frac {rare}")
    with pytest.raises(gu.GuError):
        g.set_tuning({"engine": "batched", "alpha": 2.0, "beta": 24.0, "words": 0, "rare_frac": 1.5})
    g.set_tuning(None)
    np.testing.assert_array_equal(run_bfs(g, srcs, "auto")[0], ref)


@pytest.mark.parametrize("k", [40, 100, 256, 600])
def test_scan_built_queues_every_width(k, monkeypatch):
    """Top-down levels over more edges than vertices build their queue by a scan of
    F_j (R-MAT's hub levels): distances stay exact at every batch width (1, 2 and 4
    words) and across batches.  With the bottom-up switch pushed out of reach
    (alpha 0.25), every level is top-down and the scan is certainly taken."""
    hg = gu.HostGraph.rmat(15, 16, seed=13)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, k, seed=8)
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    np.testing.assert_array_equal(run_bfs(g, srcs, "auto_batched")[0], ref)
    monkeypatch.setenv("GU_MS_ALPHA", "0.25")
    np.testing.assert_array_equal(run_bfs(g, srcs, "auto_batched")[0], ref)
    tl = g.level_profile()
    assert all(e["kind"] in ("init", "top-down", "rows") for e in tl)
    assert any(e["kind"] == "top-down" and e["frontier_edges"] > hg.n for e in tl)


def test_launch_times_ring():
    """gu_graph_launch_times: the kernel time of each of the last launches, oldest
    first; the newest is the one gu_graph_last_launch reports."""
    hg = gu.HostGraph.rmat(13, 16, seed=4)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 64, seed=1)
    for _ in range(70):
        run_bfs(g, srcs, "auto")
    t = g.launch_times()
    assert len(t) == 64 and all(x > 0 for x in t)
    assert t[-1] == pytest.approx(g.last_launch()[0])
    assert len(g.launch_times(5)) == 5


def test_level_idle_per_phase():
    """gu_graph_level_idle: one entry per timeline phase, the CTAs' barrier waits,
    between zero and the phase's duration times the launch's CTAs."""
    hg = gu.HostGraph.rmat(15, 16, seed=2)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 300, seed=4)
    ref, _ = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    np.testing.assert_array_equal(run_bfs(g, srcs, "auto_batched")[0], ref)
    tl = g.level_profile()
    idle, nblocks = g.level_idle()
    assert len(idle) == len(tl) and nblocks >= torch.cuda.get_device_properties(0).multi_processor_count
    assert (idle >= 0).all() and idle.sum() > 0
    t = [0.0] + [e["t_ms"] for e in tl]
    for i in range(1, len(tl)):
        # a phase's waits end with the barrier after it; the slowest CTA's stamp
        # precedes that barrier, so allow the barrier's own time on top
        assert idle[i] <= (t[i + 1] - t[i] + 0.05) * nblocks, i
    g2 = gu.Graph(gu.HostGraph.rmat(12, 8, seed=1))
    g2.bc(torch.as_tensor(gu.sources(g2.n, 64, seed=1), device="cuda"),
          torch.empty(g2.n, dtype=torch.float64, device="cuda"))
    with pytest.raises(gu.GuError):
        g2.level_idle()  # BC passes have no idle record

"""The bench line's arithmetic, on the CPU: the batch-aware minimum bytes, the
roofline object (physical fraction from the recorded ncu traffic over the live
kernel time), the recorded traffic itself, and the config both arms print."""
import argparse
import os
import re
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_alg_min_bytes_per_batch():
    n, m = 1000, 5000
    per_full = 4 * n * 256 + 4 * (n + 1) + 4 * m + 8 * 4 * n  # 256 sources, 4 words
    assert bench.alg_min_bytes(n, m, 512) == 2 * per_full
    tail = 4 * n * 44 + 4 * (n + 1) + 4 * m + 8 * 1 * n  # 44 sources: one word
    assert bench.alg_min_bytes(n, m, 300) == per_full + tail
    assert bench.alg_min_bytes(n, m, 0) == 0


def test_roofline_fraction_is_physical():
    r = bench.roofline_line(5e9, bench.kernel_source_hash(), 1e-3, 8e10, 2.5e9, 6000.0, "measured")
    assert r["achieved"] == pytest.approx(5000.0)  # GB/s: 5 GB in 1 ms
    assert r["frac"] == pytest.approx(5000.0 / 6000.0)
    assert r["traffic_matches_build"] is True
    assert r["alg_min_frac"] == pytest.approx(2500.0 / 6000.0)
    assert r["traffic_over_alg_min"] == pytest.approx(2.0)
    assert r["effective_frac"] == pytest.approx(80000.0 / 6000.0)  # the per-source model may exceed 1
    assert r["kernel_ms"] == pytest.approx(1.0)
    stale = bench.roofline_line(5e9, "0" * 16, 1e-3, 8e10, 2.5e9, 6000.0, "measured")
    assert stale["traffic_matches_build"] is False
    none = bench.roofline_line(None, None, 1e-3, 8e10, 2.5e9, 6000.0, "fallback")
    assert none["frac"] is None and none["traffic_over_alg_min"] is None
    assert "fallback" in none["peak_source"]


def test_recorded_traffic_has_a_source_hash():
    traffic, src = bench.ncu_traffic_per_launch()
    assert isinstance(traffic, int) and traffic > 2 * (1 << 30)  # at least the 2 GiB of rows
    assert re.fullmatch(r"[0-9a-f]{16}", src)
    assert re.fullmatch(r"[0-9a-f]{16}", bench.kernel_source_hash())


def test_both_arms_print_the_same_config():
    src = open(os.path.join(ROOT, "bench.py")).read()
    ours = src[src.index("def run_ours"):]
    ref = src[src.index("def run_reference"):src.index("def run_ours")]
    assert '"config": config_of(args, hg)' in ours and '"config": config_of(args, hg)' in ref

    class Hg:
        n, m = 1 << 20, 31402260
    args = argparse.Namespace(scale=20, sources=512, variant="auto")
    c = bench.config_of(args, Hg())
    assert c["workload"] == bench.workload_name(20, 512)
    assert (c["n"], c["m_csr"], c["sources"], c["graph_seed"], c["source_seed"]) == (1 << 20, 31402260, 512, 1, 2)


def test_cpu_model_names_the_host():
    assert isinstance(bench.cpu_model(), str) and bench.cpu_model()


def test_serving_plan_mix_and_ranges():
    """The serving workload's requests: Poisson arrivals, 60 % BFS rows of 1-256
    sources, 20 % BC of 64..bc_max sources, 20 % DAG reachability of 1-256
    sources, distinct in-range sources, the same plan for the same seed."""
    np = pytest.importorskip("numpy")
    import bench_configs
    import gu

    class G:
        def __init__(self, n):
            self.n = n
    rmats = [("r0", G(5000), None), ("r1", G(9000), None)]
    dags = [("d0", G(7000), None)]
    plan = bench_configs._serving_plan(np.random.default_rng(4), rmats, dags, 4000.0, 1.0, 512)
    again = bench_configs._serving_plan(np.random.default_rng(4), rmats, dags, 4000.0, 1.0, 512)
    assert len(plan) == len(again) and all(a[0] == b[0] and a[1] == b[1] and np.array_equal(a[4], b[4])
                                           for a, b in zip(plan, again))
    assert 3600 < len(plan) < 4400
    times = [p[0] for p in plan]
    assert all(b >= a for a, b in zip(times, times[1:]))
    kinds = [p[1] for p in plan]
    share = {q: kinds.count(q) / len(plan) for q in (gu.QUERY_BFS, gu.QUERY_BC, gu.QUERY_REACH)}
    assert abs(share[gu.QUERY_BFS] - 0.6) < 0.04 and abs(share[gu.QUERY_BC] - 0.2) < 0.03
    assert abs(share[gu.QUERY_REACH] - 0.2) < 0.03
    for t, q, hg, g, srcs in plan:
        lo, hi = (64, 512) if q == gu.QUERY_BC else (1, 256)
        assert lo <= len(srcs) <= hi
        assert srcs.dtype == np.int32 and len(np.unique(srcs)) == len(srcs)
        assert srcs.min() >= 0 and srcs.max() < hg.n
        assert (hg in [r[1] for r in dags]) == (q == gu.QUERY_REACH)
    # result sizes: BFS rows, one BC vector, one count per source
    assert bench_configs._out_bytes(gu.QUERY_BFS, G(100), np.arange(3)) == 3 * 100 * 4
    assert bench_configs._out_bytes(gu.QUERY_BC, G(100), np.arange(3)) == 100 * 8
    assert bench_configs._out_bytes(gu.QUERY_REACH, G(100), np.arange(3)) == 3 * 8

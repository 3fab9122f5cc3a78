"""All-vertex DAG reachability (gu_dag_reach) against the oracle and the
reference's reachable-pair totals (graph-utils/dag_reachability.cpp:36-65)."""
import numpy as np
import pytest

import gu
import oracle
from conftest import load_golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def run(hg, engine, monkeypatch):
    if engine == "batched":
        monkeypatch.setenv("GU_AUTO_LOCAL", "0")
    g = gu.Graph(hg)
    cnt = torch.full((hg.n,), -5, dtype=torch.int64, device="cuda")
    tot = g.dag_reach(cnt)
    return cnt.cpu().numpy(), tot


@pytest.mark.parametrize("engine", ["auto", "batched"])
@pytest.mark.parametrize("name", ["dag300", "test7"])
def test_golden_pair_totals(name, engine, monkeypatch):
    d = load_golden(name)
    hg = gu.HostGraph(d["R"], d["C"], int(d["n"]), True)
    counts, tot = run(hg, engine, monkeypatch)
    assert tot == int(d["dag_pairs"]) == counts.sum()
    ref, _ = oracle.dag_reach_counts(hg.R, hg.C, hg.n)
    np.testing.assert_array_equal(counts, ref)


@pytest.mark.parametrize("engine", ["auto", "batched"])
@pytest.mark.parametrize("n,m,seed", [(3000, 24000, 1), (20000, 160000, 2), (65536, 524288, 3)])
def test_random_dags_vs_oracle(n, m, seed, engine, monkeypatch):
    hg = gu.HostGraph.dag(n, m, seed=seed)
    counts, tot = run(hg, engine, monkeypatch)
    ref, rtot = oracle.dag_reach_counts(hg.R, hg.C, hg.n)
    np.testing.assert_array_equal(counts, ref)
    assert tot == rtot


def test_undirected_rejected():
    g = gu.Graph(gu.HostGraph.rmat(8, 4, seed=1))
    cnt = torch.empty(g.n, dtype=torch.int64, device="cuda")
    with pytest.raises(gu.GuError) as e:
        g.dag_reach(cnt)
    assert e.value.status == 1

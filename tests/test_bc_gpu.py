"""Parity of the CUDA shortest-path counting, Brandes BC and diameter with the oracle.

sigma (uint64) and distances must be bit-exact; delta and BC are FP64 and must be
within 1e-12 relative of the FP64 oracle (oracle/gu_oracle.c, pinned to the
reference's bc.cu by tests/test_oracle.py).  On undirected graphs the oracle is
the push form of bc.cu:43-55; on directed graphs the successor-pull form of the
reference's GPU design (shuffle_based.cu:217-354), which is the Brandes value.
"""
import numpy as np
import pytest

import gu
import oracle
from conftest import golden_names, load_golden

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
RTOL = 1e-12


def dev(x):
    return torch.as_tensor(np.asarray(x), device="cuda:0")


def close(got, ref, rtol=RTOL, msg=""):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    scale = np.maximum(np.abs(ref), 1e-300)
    rel = np.abs(got - ref) / scale
    bad = (rel > rtol) & (np.abs(got - ref) > 1e-300)
    assert not bad.any(), f"{msg}: max rel err {rel.max():.3e} at {np.argmax(rel)}"


def run_sigma(g, srcs):
    s = dev(np.asarray(srcs, np.int32))
    sig = torch.empty((len(srcs), g.n), dtype=torch.int64, device="cuda")
    d = torch.empty((len(srcs), g.n), dtype=torch.int32, device="cuda")
    g.sigma(s, sig, dist_dev=d)
    torch.cuda.synchronize()
    return d.cpu().numpy(), sig.cpu().numpy().view(np.uint64)


def run_bc(g, srcs, batch=0, deltas=False):
    s = dev(np.asarray(srcs, np.int32))
    bc = torch.empty(g.n, dtype=torch.float64, device="cuda")
    de = torch.empty((len(srcs), g.n), dtype=torch.float64, device="cuda") if deltas else None
    g.bc(s, bc, delta_dev=de, batch=batch)
    torch.cuda.synchronize()
    return bc.cpu().numpy(), (de.cpu().numpy() if deltas else None)


@pytest.fixture(scope="module")
def golden_graphs():
    out = {}
    for name in golden_names():
        d = load_golden(name)
        out[name] = (gu.Graph(gu.HostGraph(d["R"], d["C"], int(d["n"]), bool(d["directed"]))), d)
    return out


def test_sigma_golden(golden_graphs):
    for name, (g, d) in golden_graphs.items():
        dist, sig = run_sigma(g, d["sources"])
        np.testing.assert_array_equal(dist, d["dist"], err_msg=name)
        np.testing.assert_array_equal(sig, d["sigma"], err_msg=name)


def test_bc_and_delta_golden(golden_graphs):
    for name, (g, d) in golden_graphs.items():
        n = int(d["n"])
        pull = bool(d["directed"])
        bc, de = run_bc(g, d["sources"], deltas=True)
        close(bc, oracle.bc(d["R"], d["C"], n, d["sources"], pull=pull), msg=name)
        for i, s in enumerate(d["sources"][:64]):
            _, _, ref = oracle.brandes(d["R"], d["C"], n, int(s), "pull" if pull else "f64")
            close(de[i], ref, msg=f"{name} delta row {i}")
        if not pull:  # the reference's own FP32 deltas, to FP32 accuracy
            np.testing.assert_allclose(de, d["delta_f32"].astype(np.float64), rtol=2e-5, atol=1e-4)


def test_jazz_known_answer(golden_graphs):
    g, d = golden_graphs["jazz"]
    bc, _ = run_bc(g, np.arange(int(d["n"])))
    assert int(np.argmax(bc)) == 135
    assert abs(bc.max() - 5832.580306529999) / 5832.58 < 1e-7  # value of the reference's FP32 deltas


@pytest.mark.parametrize("batch", [64, 128, 256, 512, 1024])
def test_rmat_bc_batches(batch):
    hg = gu.HostGraph.rmat(13, 16, seed=3)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 300, seed=4)
    ref = oracle.bc(hg.R, hg.C, hg.n, srcs, nthreads=8)
    bc1, _ = run_bc(g, srcs, batch=batch)
    close(bc1, ref, msg=f"batch {batch}")
    bc2, _ = run_bc(g, srcs, batch=batch)
    np.testing.assert_array_equal(bc1.view(np.uint64), bc2.view(np.uint64))  # deterministic


def test_rmat_sigma_vs_oracle_and_edge_cases():
    hg = gu.HostGraph.rmat(12, 4, seed=8)   # degree-0 vertices present
    g = gu.Graph(hg)
    zero = np.nonzero(np.diff(hg.R) == 0)[0]
    srcs = np.concatenate([gu.sources(hg.n, 90, seed=1), [zero[0], 3, 3]]).astype(np.int32)
    dist, sig = run_sigma(g, srcs)
    rd, rs = oracle.sigma_multi(hg.R, hg.C, hg.n, srcs, nthreads=8)
    np.testing.assert_array_equal(dist, rd)
    np.testing.assert_array_equal(sig, rs)
    bc, de = run_bc(g, srcs, deltas=True)
    close(bc, oracle.bc(hg.R, hg.C, hg.n, srcs, nthreads=8))
    assert np.all(de[90] == 0.0)  # isolated source: no dependencies


def test_directed_dag_bc():
    hg = gu.HostGraph.dag(3000, 24000, seed=2)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 130, seed=6)
    dist, sig = run_sigma(g, srcs)
    rd, rs = oracle.sigma_multi(hg.R, hg.C, hg.n, srcs)
    np.testing.assert_array_equal(dist, rd)
    np.testing.assert_array_equal(sig, rs)
    bc, _ = run_bc(g, srcs)
    close(bc, oracle.bc(hg.R, hg.C, hg.n, srcs, pull=True, nthreads=8))


@pytest.mark.parametrize("engine", ["auto", "batched"])
def test_diameter(golden_graphs, engine, monkeypatch):
    if engine == "batched":  # AUTO would take the per-source engine on these graphs
        monkeypatch.setenv("GU_AUTO_LOCAL", "0")
    for name, (g, d) in golden_graphs.items():
        assert g.diameter(dev(d["sources"].astype(np.int32))) == int(d["diameter"]), name
    hg = gu.HostGraph.grid(60, 50, 0.05, seed=7)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 100, seed=2)
    assert g.diameter(dev(srcs)) == oracle.diameter(hg.R, hg.C, hg.n, srcs, nthreads=8)


def test_phase_timeline():
    """The profiling hook's BC timeline: per batch, forward levels 1..L+1 then
    backward levels L..1, each ending after the one before."""
    hg = gu.HostGraph.rmat(12, 8, seed=5)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 192, seed=3)
    run_bc(g, srcs, batch=128)
    tl = g.level_profile()
    assert tl and all(e["kind"] in ("init", "bc-forward", "bc-backward", "bc-combine", "bc-finish", "bc-clear")
                      for e in tl)
    t = [e["t_ms"] for e in tl]
    assert t == sorted(t)
    for b in (0, 1):
        fw = [e["level"] for e in tl if e["batch"] == b and e["kind"] == "bc-forward"]
        bw = [e["level"] for e in tl if e["batch"] == b and e["kind"] == "bc-backward"]
        assert fw == list(range(1, len(fw) + 1)) and bw == list(range(len(fw) - 1, 0, -1))
    assert sum(e["kind"] == "bc-finish" for e in tl) == 2
    # a BFS afterwards replaces it with the batched search's own timeline
    s = dev(np.asarray(srcs, np.int32))
    d = torch.empty((len(srcs), hg.n), dtype=torch.int32, device="cuda")
    g.bfs(s, d, variant="warp")  # a batched-engine variant (AUTO picks the per-source engine here)
    torch.cuda.synchronize()
    assert all(e["kind"] in ("init", "top-down", "bottom-up", "rows", "bu-final", "bu-light", "bu-scan")
               for e in g.level_profile())

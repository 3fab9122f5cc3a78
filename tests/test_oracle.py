"""The CPU oracle against the golden vectors made by the reference's own code.

Every golden file in tests/golden/ was produced by oracle/_ref/ref_oracle, i.e.
the reference graph-utils checkers compiled from their sources (see
tests/golden/make_golden.py).  These tests pin oracle/gu_oracle.c to them
bit-for-bit before it is trusted as the parity checker of the CUDA path.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden

GRAPHS = golden_names()


@pytest.mark.parametrize("name", GRAPHS)
def test_bfs_matches_reference(name):
    g = load_golden(name)
    d, _ = oracle.bfs_multi(g["R"], g["C"], int(g["n"]), g["sources"])
    np.testing.assert_array_equal(d, g["dist"])


@pytest.mark.parametrize("name", GRAPHS)
def test_bfs_multithreaded_same(name):
    g = load_golden(name)
    d, _ = oracle.bfs_multi(g["R"], g["C"], int(g["n"]), g["sources"], nthreads=4)
    np.testing.assert_array_equal(d, g["dist"])


@pytest.mark.parametrize("name", GRAPHS)
def test_sigma_matches_reference(name):
    g = load_golden(name)
    d, s = oracle.sigma_multi(g["R"], g["C"], int(g["n"]), g["sources"])
    np.testing.assert_array_equal(d, g["dist"])
    np.testing.assert_array_equal(s, g["sigma"])


@pytest.mark.parametrize("name", GRAPHS)
def test_brandes_f32_bit_exact(name):
    g = load_golden(name)
    n = int(g["n"])
    for i, s in enumerate(g["sources"]):
        _, _, de = oracle.brandes(g["R"], g["C"], n, int(s), "f32")
        np.testing.assert_array_equal(de.view(np.uint32), g["delta_f32"][i].view(np.uint32))


@pytest.mark.parametrize("name", GRAPHS)
def test_brandes_f64_close_to_reference_f32(name):
    g = load_golden(name)
    n = int(g["n"])
    for i, s in enumerate(g["sources"][:40]):
        _, _, de = oracle.brandes(g["R"], g["C"], n, int(s), "f64")
        ref = g["delta_f32"][i].astype(np.float64)
        np.testing.assert_allclose(de, ref, rtol=2e-5, atol=1e-5)


@pytest.mark.parametrize("name", [n for n in GRAPHS if n not in ("test7", "dag300")])
def test_pull_equals_push_on_undirected(name):
    g = load_golden(name)
    n = int(g["n"])
    for s in g["sources"][:40]:
        _, _, a = oracle.brandes(g["R"], g["C"], n, int(s), "f64")
        _, _, b = oracle.brandes(g["R"], g["C"], n, int(s), "pull")
        np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("name", GRAPHS)
def test_diameter_matches_reference(name):
    g = load_golden(name)
    assert oracle.diameter(g["R"], g["C"], int(g["n"]), g["sources"]) == int(g["diameter"])


def test_dag_reach_counts_sum_to_pairs():
    import gu
    for seed in (1, 2):
        hg = gu.HostGraph.dag(400, 3000, seed=seed)
        counts, tot = oracle.dag_reach_counts(hg.R, hg.C, hg.n)
        assert tot == counts.sum() == oracle.dag_reach_pairs(hg.R, hg.C, hg.n)
        # a vertex's set is its successors and their sets (the reference's recursion)
        for v in range(0, hg.n, 37):
            succ = hg.C[hg.R[v]:hg.R[v + 1]]
            reach = set(succ.tolist())
            frontier = list(succ)
            while frontier:
                w = frontier.pop()
                for x in hg.C[hg.R[w]:hg.R[w + 1]]:
                    if x not in reach:
                        reach.add(int(x))
                        frontier.append(int(x))
            assert counts[v] == len(reach)


def test_dag_reachability_matches_reference():
    for name in ("test7", "dag300"):
        g = load_golden(name)
        assert oracle.dag_reach_pairs(g["R"], g["C"], int(g["n"])) == int(g["dag_pairs"])


@pytest.mark.parametrize("name", golden_names("lbs_"))
def test_lbs_matches_reference(name):
    g = load_golden(name, "lbs_")
    scanned, result, total = oracle.lbs(g["counts"])
    assert total == int(g["counts"].sum())
    np.testing.assert_array_equal(scanned, g["scanned"])
    np.testing.assert_array_equal(result, g["result"])


def test_lbs_overflow_rejected():
    with pytest.raises(ValueError):
        oracle.lbs(np.full(4, 2**30, np.int32))


def test_race_and_resolve_semantics():
    assert oracle.race_and_resolve(0, 7) == 7
    assert oracle.race_and_resolve(1, 5) == 0
    assert oracle.race_and_resolve(0x80000001, 3) == 31
    assert oracle.race_and_resolve(0b0110, 0) == 2


def test_jazz_known_answers():
    """Values of the reference checkers on graphs/jazz.graph (n=198)."""
    g = load_golden("jazz")
    n = int(g["n"])
    reach = oracle.reach_count(g["R"], g["C"], n, np.arange(n))
    assert reach == 39204
    assert oracle.diameter(g["R"], g["C"], n, np.arange(n)) == 6
    bc = oracle.bc(g["R"], g["C"], n, np.arange(n))
    assert int(np.argmax(bc)) == 135
    # the reference's FP32 deltas (golden) summed in double give exactly this value
    d32 = g["delta_f32"].astype(np.float64)
    bc32 = d32.sum(0) - np.diag(d32)
    assert abs(bc32.max() - 5832.580306529999) < 1e-9
    # the FP64 oracle differs from it by FP32 rounding only
    assert abs(bc.max() - 5832.580306529999) / 5832.58 < 1e-7
    np.testing.assert_allclose(bc, bc32, rtol=1e-5, atol=1e-6)


def test_textbook_bc_maxima():
    """test1..5 maxima of the all-source BC (ordered pairs, source excluded)."""
    expect = {"test1": 38, "test2": 20, "test3": 7, "test4": 30, "test5": 18}
    for name, mx in expect.items():
        g = load_golden(name)
        n = int(g["n"])
        bc = oracle.bc(g["R"], g["C"], n, np.arange(n))
        assert abs(bc.max() - mx) < 1e-9, (name, bc.max())


def test_bc_threads_deterministic_and_close():
    g = load_golden("er198")
    n = int(g["n"])
    a = oracle.bc(g["R"], g["C"], n, np.arange(n), nthreads=1)
    b = oracle.bc(g["R"], g["C"], n, np.arange(n), nthreads=4)
    c = oracle.bc(g["R"], g["C"], n, np.arange(n), nthreads=4)
    np.testing.assert_array_equal(b, c)
    np.testing.assert_allclose(a, b, rtol=1e-14)


def test_port_speed_script_against_reference_checker():
    """oracle/compare_speed.py, where the reference checkers were built here: the
    port and the reference's own BFS checker scan the same CSR entries on the
    benchmark graph's generator (small scale), and both rates are reported."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if not os.path.exists(os.path.join(root, "oracle", "_ref", "ref_oracle")):
        pytest.skip("reference checkers not built (no reference tree)")
    out = subprocess.run([sys.executable, os.path.join(root, "oracle", "compare_speed.py"), "--scale", "12",
                          "--sources", "4"], check=True, capture_output=True, text=True).stdout
    r = json.loads(out.strip().splitlines()[-1])
    assert r["sources"] == 4 and r["reference_gteps"] > 0 and r["port_gteps"] > 0


def _random_csr(rng, n, m, directed):
    """Random simple graph as CSR (no self-loops, no duplicates; undirected graphs
    symmetrised), neighbour order shuffled as a file parser may leave it."""
    if n < 2 or m == 0:
        return np.zeros(n + 1, np.int32), np.zeros(0, np.int32)
    u = rng.integers(0, n, m)
    v = rng.integers(0, n, m)
    keep = u != v
    u, v = u[keep], v[keep]
    if not directed:
        u, v = np.concatenate([u, v]), np.concatenate([v, u])
    key = np.unique(u.astype(np.int64) * n + v)
    u, v = (key // n).astype(np.int32), (key % n).astype(np.int32)
    perm = rng.permutation(len(u))
    order = np.argsort(u[perm], kind="stable")
    u, v = u[perm][order], v[perm][order]
    R = np.zeros(n + 1, np.int32)
    np.add.at(R, u + 1, 1)
    return np.cumsum(R).astype(np.int32), v


def test_oracle_vs_reference_checkers_on_random_graphs(tmp_path):
    """Where the reference checkers were built here: distances, sigma, FP32 deltas
    and the diameter of the oracle equal the reference's own checkers
    (multi_search_test.cu:17-38, shortest_paths.cu:11-39, bc.cu:11-57,
    diameter_sampling_test.cu:9-38) bit for bit on seeded random graphs, directed
    and undirected, from one vertex to a few hundred."""
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    ref = os.path.join(root, "oracle", "_ref", "ref_oracle")
    if not os.path.exists(ref):
        pytest.skip("reference checkers not built (no reference tree)")
    rng = np.random.default_rng(20)
    for case in range(16):
        n = int(rng.choice([1, 2, 7, 40, 150, 300]))
        directed = bool(case % 2)
        m = int(rng.integers(0, 4 * n + 1))
        R, C = _random_csr(rng, n, m, directed)
        k = min(n, 6)
        src = rng.choice(n, k, replace=False).astype(np.int32)
        pre = str(tmp_path / f"g{case}")
        R.tofile(pre + ".R")
        C.tofile(pre + ".C")
        with open(pre + ".meta", "w") as f:
            f.write(f"{n} {len(C)} {int(directed)}\n")
        src.tofile(pre + ".src")
        subprocess.run([ref, "run", pre, pre + ".src", pre + ".out"], check=True)
        dist = np.fromfile(pre + ".out.dist", np.int32).reshape(k, n)
        sigma = np.fromfile(pre + ".out.sigma", np.uint64).reshape(k, n)
        delta = np.fromfile(pre + ".out.delta_f32", np.float32).reshape(k, n)
        diam = int(np.fromfile(pre + ".out.diameter", np.int32)[0])
        d, _ = oracle.bfs_multi(R, C, n, src)
        np.testing.assert_array_equal(d, dist, err_msg=f"case {case}")
        _, sg = oracle.sigma_multi(R, C, n, src)
        np.testing.assert_array_equal(sg, sigma, err_msg=f"case {case}")
        for i, s in enumerate(src):
            _, _, de = oracle.brandes(R, C, n, int(s), kind="f32")
            np.testing.assert_array_equal(de.view(np.uint32), delta[i].view(np.uint32), err_msg=f"case {case}")
        assert oracle.diameter(R, C, n, src) == diam, f"case {case}"


def test_oracle_dag_and_lbs_vs_reference_on_random_inputs(tmp_path):
    """Where the reference checkers were built here: reachable pairs of seeded random
    DAGs equal get_reachability_dag's (dag_reachability.cpp:36-65), and the LBS
    scan and owners of random ragged counts (zeros included) equal the reference
    example's (examples/load_balanced_search/lbs.cu:18-31), bit for bit."""
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    ref = os.path.join(root, "oracle", "_ref", "ref_oracle")
    if not os.path.exists(ref):
        pytest.skip("reference checkers not built (no reference tree)")
    rng = np.random.default_rng(21)
    for case in range(10):
        n = int(rng.choice([1, 3, 30, 200, 400]))
        m = int(rng.integers(0, 3 * n + 1))
        topo = rng.permutation(n)  # vertex topo[i] comes i-th in the order
        a, b = rng.integers(0, n, m), rng.integers(0, n, m)
        keep = a != b
        lo, hi = np.minimum(a, b)[keep], np.maximum(a, b)[keep]
        u, v = topo[lo], topo[hi]
        if len(u):
            key = np.unique(u.astype(np.int64) * n + v)
            u, v = (key // n).astype(np.int32), (key % n).astype(np.int32)
        R = np.zeros(n + 1, np.int32)
        np.add.at(R, np.asarray(u, np.int64) + 1, 1)
        R = np.cumsum(R).astype(np.int32)
        C = np.asarray(v, np.int32)
        pre = str(tmp_path / f"d{case}")
        R.tofile(pre + ".R")
        C.tofile(pre + ".C")
        with open(pre + ".meta", "w") as f:
            f.write(f"{n} {len(C)} 1\n")
        subprocess.run([ref, "dag", pre, pre + ".out"], check=True)
        pairs = int(np.fromfile(pre + ".out.pairs", np.int64)[0])
        assert oracle.dag_reach_pairs(R, C, n) == pairs, f"dag case {case}"
        assert oracle.dag_reach_counts(R, C, n)[1] == pairs, f"dag case {case}"
    for case in range(8):
        N = int(rng.choice([1, 5, 64, 700]))
        counts = rng.integers(0, 11, N).astype(np.int32)
        counts[rng.random(N) < 0.4] = 0
        pre = str(tmp_path / f"l{case}")
        counts.tofile(pre + ".counts")
        subprocess.run([ref, "lbs", pre + ".counts", pre + ".out"], check=True)
        scanned = np.fromfile(pre + ".out.scanned", np.int32)
        result = np.fromfile(pre + ".out.result", np.int32)
        s, r, t = oracle.lbs(counts)
        assert t == int(counts.sum()) == len(result), f"lbs case {case}"
        np.testing.assert_array_equal(s[:N], scanned, err_msg=f"lbs case {case}")
        np.testing.assert_array_equal(r[:t], result, err_msg=f"lbs case {case}")


@pytest.mark.parametrize("scale,permute,seed", [(10, True, 3), (12, False, 5), (14, True, 1)])
def test_oracle_generator_equals_the_library(scale, permute, seed):
    """The oracle's restated R-MAT generator and source sampler (used by the CPU
    baseline to build its input without the library) give the library's CSR and
    sources exactly."""
    import gu
    hg = gu.HostGraph.rmat(scale, 16, 0.57, 0.19, 0.19, seed=seed, permute=permute)
    R, C = oracle.rmat(scale, 16, 0.57, 0.19, 0.19, seed=seed, permute=permute)
    np.testing.assert_array_equal(hg.R, R)
    np.testing.assert_array_equal(hg.C, C)
    np.testing.assert_array_equal(gu.sources(hg.n, 300, seed=seed + 1), oracle.sources(hg.n, 300, seed + 1))

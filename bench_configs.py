"""The non-headline benchmark configurations, one JSON line each (`bench.py --workload cN`).

    c1  ER G(198, 2742) seed 1 and the jazz graph: BFS and exact BC from every vertex.
    c3  R-MAT scale 18 (ef 16), 8192 sources: sigma (u64) and FP64 Brandes BC with
        64, 128, 256, 512 and 1024 sources per pass.
    c4  2048 x 2048 4-neighbour grid, each edge deleted with probability 0.05 (seed 7),
        256 sources: BFS (batched and the one-CTA-per-source form), diameter, and
        load-balanced search over the int32 degree array.
    c5  serving: 12 R-MAT graphs (scales 12-22) and 4 random DAGs (2^16-2^20) resident,
        Poisson arrivals of BFS / BC / reachability requests at several rates, p50 / p99
        latency, and a saturation burst against one call per request.
    io  graph files: R-MAT scale 20 as METIS / SNAP / MatrixMarket text and the
        binary CSR cache, read by this library and by the reference parser.
    dag all-vertex reachability of random DAGs (m = 8n), n = 2^16 and 2^18.

GPU times are CUDA-event kernel times of the library's own launch (`last_launch`)
unless named `call_ms` (wall time of the synchronous C-ABI call).  CPU times are
the oracle (test infrastructure: the C restatement of the reference checkers) on
one host thread and on all host threads; long CPU runs are timed on a seeded
subset of the sources and extrapolated per source, and say so.
"""
import json
import os
import statistics
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "graph-utils_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

INF = 2147483647


def _torch():
    import torch
    torch.cuda.set_device(0)
    return torch


def _median_kernel_ms(g, fn, reps=5):
    times = []
    for _ in range(reps):
        fn()
        times.append(g.last_launch()[0] * 1e3)
    return statistics.median(times)


def _median_call_ms(fn, reps=3):
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        times.append((time.perf_counter() - t0) * 1e3)
    return statistics.median(times)


def _edges_reached(torch, g, srcs, deg):
    """Sum over sources of scanned CSR entries (E_s) and reached vertices, via the engine's rows."""
    E = V = 0.0
    for b in range(0, len(srcs), 1024):
        s = torch.as_tensor(srcs[b:b + 1024], device="cuda")
        d = torch.empty((len(s), g.n), dtype=torch.int32, device="cuda")
        g.bfs(s, d)
        r = (d != INF).to(torch.float64)
        E += float((r @ deg).sum())
        V += float(r.sum())
        del d, r
    return E, V


def _cpu(fn, *a, **kw):
    t0 = time.perf_counter()
    out = fn(*a, **kw)
    return out, time.perf_counter() - t0


def _emit(line):
    print(json.dumps(line), flush=True)


def wl_c1(args):
    import gu
    import oracle
    torch = _torch()
    cores = os.cpu_count() or 1
    d = dict(np.load(os.path.join(ROOT, "tests", "golden", "graph_jazz.npz")))
    graphs = {"er198_m2742_seed1": gu.HostGraph.er(198, 2742, seed=1),
              "jazz": gu.HostGraph(d["R"], d["C"], int(d["n"]), bool(d["directed"]))}
    out = {}
    for name, hg in graphs.items():
        g = gu.Graph(hg)
        srcs = np.arange(hg.n, dtype=np.int32)
        s = torch.as_tensor(srcs, device="cuda")
        dist = torch.empty((hg.n, hg.n), dtype=torch.int32, device="cuda")
        bc = torch.empty(hg.n, dtype=torch.float64, device="cuda")
        deg = torch.as_tensor(np.diff(hg.R).astype(np.float64), device="cuda")
        E, V = _edges_reached(torch, g, srcs, deg)
        edges = E / 2.0
        t_b = _median_kernel_ms(g, lambda: g.bfs(s, dist, variant="auto"))
        t_p = _median_kernel_ms(g, lambda: g.bfs(s, dist, variant="plain"))
        t_bc = _median_kernel_ms(g, lambda: g.bc(s, bc))
        c_bc = _median_call_ms(lambda: g.bc(s, bc))
        _, t1 = _cpu(oracle.bfs_multi, hg.R, hg.C, hg.n, srcs, nthreads=1)
        _, tN = _cpu(oracle.bfs_multi, hg.R, hg.C, hg.n, srcs, nthreads=cores)
        _, b1 = _cpu(oracle.bc, hg.R, hg.C, hg.n, srcs, nthreads=1)
        _, bN = _cpu(oracle.bc, hg.R, hg.C, hg.n, srcs, nthreads=cores)
        out[name] = {"n": hg.n, "m_csr": hg.m, "sources": len(srcs), "edges_per_bfs": edges,
                     "bfs_auto_kernel_ms": t_b, "bfs_plain_kernel_ms": t_p,
                     "bfs_auto_gteps": edges / t_b / 1e6, "bfs_plain_gteps": edges / t_p / 1e6,
                     "bc_kernel_ms": t_bc, "bc_call_ms": c_bc, "bc_gteps": edges / t_bc / 1e6,
                     "cpu_bfs_ms_1thread": t1 * 1e3, f"cpu_bfs_ms_{cores}threads": tN * 1e3,
                     "cpu_bc_f64_ms_1thread": b1 * 1e3, f"cpu_bc_f64_ms_{cores}threads": bN * 1e3}
        g.close()
    _emit({"workload": "c1_er198_jazz_all_sources", "metric": "BFS and exact BC, all sources",
           "unit": "ms / GTEPS", "results": out, "cpu_cores": cores,
           "note": "tiny graphs: launch- and barrier-latency bound, GTEPS is not the point"})


def _hbm_peak():
    """Measured HBM copy bandwidth (GB/s) of this machine's GPUs, or the fallback figure."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


BC_PROFILE = os.path.join(ROOT, "profiles", "bc_grid_kernel_rmat18.md")


def _profile_value(path, key):
    """A `key: value` line of a committed profile summary (None if absent)."""
    if not os.path.exists(path):
        return None
    for line in open(path):
        k, _, v = line.partition(":")
        if k == key:
            return v.strip()
    return None


def source_hash(files):
    """sha256 (first 16 hex digits) of kernel sources, as the profile summaries record it."""
    import hashlib
    h = hashlib.sha256()
    for f in files:
        with open(os.path.join(ROOT, "graph-utils_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


BC_SOURCES = ("bc.cu", "device_utils.cuh", "gu_internal.h")


def bc_subline(torch):
    """Sampled BC for the default bench line: R-MAT scale 18 (ef 16, seed 1), 8192 sources
    (seed 2) in passes of 1024 in one persistent launch; kernel time (median of 3 after a
    warm-up), GTEPS of forward-sweep edges, the launch's physical DRAM fraction (ncu bytes of
    the same launch from the committed profile, with the build it was taken on), and the
    largest relative error against the FP64 oracle over the first 256 sources."""
    import gu
    import oracle
    cores = os.cpu_count() or 1
    hg = gu.HostGraph.rmat(18, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 8192, seed=2)
    deg = torch.as_tensor(np.diff(hg.R).astype(np.float64), device="cuda")
    E, V = _edges_reached(torch, g, srcs, deg)
    edges = E / 2.0
    s = torch.as_tensor(srcs, device="cuda")
    bc = torch.empty(hg.n, dtype=torch.float64, device="cuda")
    g.bc(s, bc, batch=1024)
    times = []
    for _ in range(3):
        g.bc(s, bc, batch=1024)
        times.append(g.last_launch()[0])
    kt = statistics.median(times)
    g.bc(s[:256], bc, batch=256)
    got = bc.cpu().numpy()
    want = oracle.bc(hg.R, hg.C, hg.n, srcs[:256], nthreads=cores)
    diff = np.abs(got - want)
    rel = np.where(diff > 1e-300, diff / np.maximum(np.abs(want), 1e-300), 0.0)
    peak = _hbm_peak()
    tr = _profile_value(BC_PROFILE, "traffic_bytes_per_launch_8192src_batch1024")
    tr = int(tr) if tr else None
    src_prof = _profile_value(BC_PROFILE, "kernel_source_sha16")
    src_now = source_hash(BC_SOURCES)
    alg = len(srcs) * 28.0 * hg.n + 32.0 * V + 40.0 * E
    g.close()
    return {"workload": "rmat18_ef16_8192src_bc_batch1024", "unit": "GTEPS", "value": edges / kt / 1e9,
            "kernel_ms": kt * 1e3, "edges": edges, "dtype": "u64 sigma, f64 delta/bc",
            "max_rel_err_256src": float(rel.max()), "tolerance": 1e-12,
            "roofline": {"bound": "hbm", "traffic": tr, "achieved": tr / kt / 1e9 if tr else None,
                         "peak": peak, "unit": "GB/s", "frac": tr / kt / 1e9 / peak if tr else None,
                         "traffic_kernel_source_sha16": src_prof, "kernel_source_sha16": src_now,
                         "traffic_matches_build": src_prof == src_now,
                         "effective_frac": alg / kt / 1e9 / peak,
                         "effective_model": "per-source 28n + 32 V_s + 40 E_s (a pass shares its reads among "
                                            "up to 1024 sources, so this can exceed 1)"}}


def wl_c3_launch(args):
    """Profiling case: the sampled-BC launch of the default bench line (8192 sources of the
    C3 graph, 1024 per pass), three times; prints the kernel times."""
    import gu
    torch = _torch()
    hg = gu.HostGraph.rmat(18, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    g = gu.Graph(hg)
    s = torch.as_tensor(gu.sources(hg.n, 8192, seed=2), device="cuda")
    bc = torch.empty(hg.n, dtype=torch.float64, device="cuda")
    times = []
    for _ in range(3):
        g.bc(s, bc, batch=1024)
        times.append(g.last_launch()[0] * 1e3)
    _emit({"workload": "c3_launch_rmat18_8192src_bc_batch1024", "metric": "kernel time of the BC launch",
           "unit": "ms", "kernel_ms": times})


def wl_c3_pass(args):
    """Profiling case: one Brandes pass over 256 of the C3 sources (batch 256), three
    times, on the C3 graph; prints the kernel times and the pass's phase timeline."""
    import gu
    torch = _torch()
    hg = gu.HostGraph.rmat(18, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    g = gu.Graph(hg)
    s = torch.as_tensor(gu.sources(hg.n, 8192, seed=2)[:256], device="cuda")
    bc = torch.empty(hg.n, dtype=torch.float64, device="cuda")
    times = []
    for _ in range(3):
        g.bc(s, bc, batch=256)
        times.append(g.last_launch()[0] * 1e3)
    tl = g.level_profile()
    _emit({"workload": "c3_pass_rmat18_256src_bc", "metric": "kernel time of one 256-source BC pass",
           "unit": "ms", "kernel_ms": times,
           "phases_us": [[e["kind"], e["level"], round(1e3 * (e["t_ms"] - tl[i - 1]["t_ms"]), 1)]
                         for i, e in enumerate(tl) if i > 0]})


def wl_lbs(args):
    """Load-balanced search over the int32 degree array of the C4 grid (N = 4,194,304
    counts): 25 calls (the last 20 timed, synchronous C-ABI call), the last checked
    against the oracle (examples/load_balanced_search/lbs.cu:18-31)."""
    import gu
    import oracle
    torch = _torch()
    hg = gu.HostGraph.grid(2048, 2048, 0.05, seed=7)
    deg = np.diff(hg.R).astype(np.int32)
    counts = torch.as_tensor(deg, device="cuda")
    scanned = torch.empty_like(counts)
    result = torch.empty(int(deg.sum()), dtype=torch.int32, device="cuda")
    ts, dev_ms = [], []
    for i in range(25):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gu.lbs(counts, scanned, result)
        if i >= 5:
            ts.append(time.perf_counter() - t0)
            dev_ms.append(gu.lbs_last_ms())
    s_ref, r_ref, tot = oracle.lbs(deg)
    exact = bool(np.array_equal(scanned.cpu().numpy(), s_ref) and np.array_equal(result.cpu().numpy(), r_ref))
    alg = 4.0 * len(deg) * 2 + 4.0 * tot
    dev = statistics.median(dev_ms)
    peak = _hbm_peak()
    _emit({"workload": "lbs_grid2048_degrees", "metric": "load-balanced search call time", "unit": "ms",
           "N": len(deg), "total": tot, "call_ms_min": 1e3 * min(ts), "call_ms_median": 1e3 * statistics.median(ts),
           "device_ms_median": dev, "device_ms_min": min(dev_ms), "alg_bytes": alg,
           "alg_frac_of_hbm": alg / (dev * 1e-3) / 1e9 / peak, "bit_exact": exact})


def wl_c4_pass(args):
    """Profiling case: the per-source engine in counting mode (diameter over the 256 C4
    sources, no rows), three times, on the C4 grid."""
    import gu
    torch = _torch()
    hg = gu.HostGraph.grid(2048, 2048, 0.05, seed=7)
    g = gu.Graph(hg)
    s = torch.as_tensor(gu.sources(hg.n, 256, seed=2), device="cuda")
    times, diam = [], None
    for _ in range(3):
        diam = g.diameter(s)
        times.append(g.last_launch()[0] * 1e3)
    _emit({"workload": "c4_pass_grid2048_256src_diameter", "metric": "kernel time of the per-source engine, counting mode",
           "unit": "ms", "kernel_ms": times, "diameter": diam})


def wl_c3(args):
    import gu
    import oracle
    torch = _torch()
    cores = os.cpu_count() or 1
    hg = gu.HostGraph.rmat(18, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 8192, seed=2)
    deg = torch.as_tensor(np.diff(hg.R).astype(np.float64), device="cuda")
    E, V = _edges_reached(torch, g, srcs, deg)
    edges = E / 2.0  # per direction (forward sweep); the backward sweep walks the same edges again
    s = torch.as_tensor(srcs, device="cuda")
    bc = torch.empty(hg.n, dtype=torch.float64, device="cuda")
    res = {}
    for batch in (64, 128, 256, 512, 1024):
        t = _median_kernel_ms(g, lambda: g.bc(s, bc, batch=batch), reps=3)
        res[f"bc_batch{batch}_kernel_ms"] = t
        res[f"bc_batch{batch}_gteps"] = edges / t / 1e6
    # the plain form: one launch per source (32 sources, extrapolated to the 8192)
    t1 = []
    for i in range(32):
        g.bc(s[i:i + 1], bc)
        t1.append(g.last_launch()[0] * 1e3)
    res["bc_one_source_per_launch_ms_extrapolated"] = float(np.mean(t1[1:])) * len(srcs)
    # per-phase timeline of one 256-source pass (the library's profiling hook)
    g.bc(s[:256], bc, batch=256)
    torch.cuda.synchronize()
    tl = g.level_profile()
    res["phases_256src_us"] = [[e["kind"], e["level"], round(1e3 * (e["t_ms"] - tl[i - 1]["t_ms"]), 1)]
                               for i, e in enumerate(tl) if i > 0]
    ks = 1024
    s1 = s[:ks]
    sig = torch.empty((ks, hg.n), dtype=torch.int64, device="cuda")
    dst = torch.empty((ks, hg.n), dtype=torch.int32, device="cuda")
    res["sigma_1024src_kernel_ms"] = _median_kernel_ms(g, lambda: g.sigma(s1, sig, dist_dev=dst), reps=3)
    del sig, dst
    # BC algorithmic bytes per source: 28n + 32 V_s + 40 E_s (dist, sigma, delta rows and bc; forward
    # and backward reads of the adjacency, levels, sigma and delta per reached vertex and edge)
    alg = len(srcs) * 28.0 * hg.n + 32.0 * V + 40.0 * E
    best = min(res[f"bc_batch{b}_kernel_ms"] for b in (64, 128, 256, 512, 1024))
    # accuracy on a fixed subset (the first 256 sources, one pass of 256) against the FP64 oracle
    g.bc(s[:256], bc, batch=256)
    got = bc.cpu().numpy()
    want = oracle.bc(hg.R, hg.C, hg.n, srcs[:256], nthreads=cores)
    diff = np.abs(got - want)
    res["max_rel_err_first256"] = float(np.where(diff > 1e-300, diff / np.maximum(np.abs(want), 1e-300), 0).max())
    sub1, subN = srcs[:4], srcs[:4 * cores]
    _, c1 = _cpu(oracle.bc, hg.R, hg.C, hg.n, sub1, nthreads=1)
    _, cN = _cpu(oracle.bc, hg.R, hg.C, hg.n, subN, nthreads=cores)
    _emit({"workload": "c3_rmat18_ef16_8192src_bc", "metric": "FP64 Brandes BC GTEPS (forward-sweep edges)",
           "unit": "GTEPS", "value": edges / best / 1e6, "n": hg.n, "m_csr": hg.m, "sources": len(srcs),
           "edges": edges, "results": res,
           "roofline": {"bound": "hbm", "alg_bytes": alg, "achieved_gbs": alg / best / 1e6,
                        "peak_gbs": _hbm_peak(), "effective_frac": alg / best / 1e6 / _hbm_peak(),
                        "model": "per-source 28n + 32 V_s + 40 E_s (effective: a pass shares reads)",
                        "physical": "ncu of one 256-source pass: 9.87 GB DRAM in 6.32 ms, 1.56 TB/s, 0.23 of "
                                    "the measured HBM peak (profiles/bc_grid_kernel_rmat18.md)"},
           "cpu_bc_f64": {"per_source_ms_1thread": c1 * 1e3 / len(sub1),
                          f"per_source_ms_{cores}threads": cN * 1e3 / len(subN),
                          "extrapolated_8192_s_all_threads": cN / len(subN) * 8192,
                          "sample": f"first {len(sub1)} sources on 1 thread, first {len(subN)} on {cores}"}})


def wl_c4(args):
    import gu
    import oracle
    torch = _torch()
    cores = os.cpu_count() or 1
    hg = gu.HostGraph.grid(2048, 2048, 0.05, seed=7)
    g = gu.Graph(hg)
    srcs = gu.sources(hg.n, 256, seed=2)
    s = torch.as_tensor(srcs, device="cuda")
    deg_np = np.diff(hg.R).astype(np.int32)
    deg = torch.as_tensor(deg_np.astype(np.float64), device="cuda")
    E, V = _edges_reached(torch, g, srcs, deg)
    edges = E / 2.0
    dist = torch.empty((len(srcs), hg.n), dtype=torch.int32, device="cuda")
    t_b = _median_kernel_ms(g, lambda: g.bfs(s, dist, variant="auto"), reps=3)
    levels = g.last_launch()[1:]
    t_p = _median_kernel_ms(g, lambda: g.bfs(s, dist, variant="plain"), reps=1)
    c_d = _median_call_ms(lambda: g.diameter(s), reps=3)
    diam = g.diameter(s)
    # load-balanced search over the degree array
    counts = torch.as_tensor(deg_np, device="cuda")
    scanned = torch.empty_like(counts)
    result = torch.empty(int(deg_np.sum()), dtype=torch.int32, device="cuda")
    c_l = _median_call_ms(lambda: gu.lbs(counts, scanned, result), reps=5)
    lbs_bytes = 4.0 * len(deg_np) * 2 + 4.0 * int(deg_np.sum())
    sub = srcs[:cores]
    _, cb = _cpu(oracle.bfs_multi, hg.R, hg.C, hg.n, sub, nthreads=cores)
    _, cl = _cpu(oracle.lbs, deg_np)
    _emit({"workload": "c4_grid2048_p005_256src", "metric": "multi-source BFS GTEPS (high diameter)",
           "unit": "GTEPS", "value": edges / t_b / 1e6, "n": hg.n, "m_csr": hg.m, "sources": len(srcs),
           "edges": edges, "diameter_of_sample": diam, "levels_td_bu_max": levels,
           "bfs_auto_kernel_ms": t_b, "bfs_plain_kernel_ms": t_p, "plain_gteps": edges / t_p / 1e6,
           "diameter_call_ms": c_d,
           "lbs": {"N": len(deg_np), "total": int(deg_np.sum()), "call_ms": c_l,
                   "alg_gbs": lbs_bytes / c_l / 1e6, "cpu_ms_1thread": cl * 1e3,
                   "model": "4N counts + 4N scanned + 4 total result bytes"},
           "cpu_bfs": {"gteps": (E / len(srcs) * len(sub) / 2.0) / cb / 1e9, "cores": cores,
                       "sample": f"first {len(sub)} sources, per-source edges from the full set"}})


def _serving_set(torch, n_rmat, scales, n_dag, dag_log2, rng):
    """R-MAT graphs and random DAGs resident on the device (a serving replica's set),
    with the per-vertex component edge counts GTEPS needs."""
    import gu
    import scipy.sparse
    import scipy.sparse.csgraph
    rmats, dags = [], []
    for i in range(n_rmat):
        sc, ef = int(rng.integers(scales[0], scales[1] + 1)), int(rng.choice([8, 16, 32]))
        hg = gu.HostGraph.rmat(sc, ef, 0.57, 0.19, 0.19, seed=100 + i, permute=True)
        rmats.append((f"rmat{sc}_ef{ef}_s{100 + i}", hg, gu.Graph(hg)))
    for i in range(n_dag):
        n = int(2 ** rng.uniform(dag_log2[0], dag_log2[1]))
        hg = gu.HostGraph.dag(n, 8 * n, seed=200 + i)
        dags.append((f"dag{n}_s{200 + i}", hg, gu.Graph(hg)))
    torch.cuda.synchronize()
    # edges a search from s traverses on an undirected graph: its component's CSR entries
    # (each undirected edge once per direction); GTEPS counts them once, as the other lines do
    comp_edges = {}
    for name, hg, g in rmats:
        A = scipy.sparse.csr_matrix((np.ones(hg.m, np.int8), hg.C, hg.R), shape=(hg.n, hg.n))
        _, lab = scipy.sparse.csgraph.connected_components(A, directed=False)
        per = np.bincount(lab, weights=np.diff(hg.R).astype(np.float64))
        comp_edges[id(hg)] = per[lab] / 2.0
    return rmats, dags, comp_edges


def _serving_plan(rng, rmats, dags, rate, dur, bc_max):
    """Poisson arrivals: 60% BFS rows (1-256 sources), 20% BC (64-bc_max), 20% DAG reachable counts (1-256)."""
    import gu
    plan, t = [], 0.0
    while t < dur:
        t += float(rng.exponential(1.0 / rate))
        u = rng.random()
        if u < 0.6:
            name, hg, g = rmats[int(rng.integers(len(rmats)))]
            k = int(rng.integers(1, 257))
            plan.append((t, gu.QUERY_BFS, hg, g, rng.choice(hg.n, k, replace=False).astype(np.int32)))
        elif u < 0.8:
            name, hg, g = rmats[int(rng.integers(len(rmats)))]
            k = int(rng.integers(64, bc_max + 1))
            plan.append((t, gu.QUERY_BC, hg, g, rng.choice(hg.n, k, replace=False).astype(np.int32)))
        else:
            name, hg, g = dags[int(rng.integers(len(dags)))]
            k = int(rng.integers(1, 257))
            plan.append((t, gu.QUERY_REACH, hg, g, rng.choice(hg.n, k, replace=False).astype(np.int32)))
    return plan


def _req_edges(comp_edges, q, hg, srcs):
    import gu
    return float(comp_edges[id(hg)][srcs].sum()) if q != gu.QUERY_REACH else 0.0


def _out_bytes(q, hg, srcs):
    import gu
    return len(srcs) * hg.n * 4 if q == gu.QUERY_BFS else (hg.n * 8 if q == gu.QUERY_BC else len(srcs) * 8)


def _host_cap(limit):
    """limit, or a quarter of the host's available memory if that is smaller."""
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return min(limit, int(line.split()[1]) * 1024 // 4)
    except OSError:
        pass
    return limit


def _serve_stream(plan, comp_edges, slots=4, max_batch=1024, max_out_bytes=48 << 30):
    """Runs one open-loop request stream through a gu.Server; latency from the planned
    arrival.  The client holds at most max_out_bytes of result buffers: beyond that
    it waits before submitting (that wait counts in the latency)."""
    import gu
    import queue
    import threading
    srv = gu.Server(hbm_budget_bytes=64 << 30, slots=slots, max_batch=max_batch)
    max_out_bytes = _host_cap(max_out_bytes)
    pending = queue.Queue()
    lat = []  # open-loop latency: from the planned arrival, so a late submit counts
    held = [0]
    cv = threading.Condition()

    def waiter():  # waits in submission order, so finished outputs are released as it goes
        while True:
            item = pending.get()
            if item is None:
                return
            rid, lag, b = item
            lat.append(srv.wait(rid) + lag)
            with cv:
                held[0] -= b
                cv.notify_all()

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    for (ta, q, hg, g, srcs) in plan:
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        b = _out_bytes(q, hg, srcs)
        with cv:
            cv.wait_for(lambda: held[0] + b <= max_out_bytes or held[0] == 0)
            held[0] += b
        if q == gu.QUERY_BFS:
            out = np.empty((len(srcs), hg.n), np.int32)
        elif q == gu.QUERY_BC:
            out = np.empty(hg.n, np.float64)
        else:
            out = np.empty(len(srcs), np.int64)
        rid = srv.submit(g, q, srcs, out)
        del out
        pending.put((rid, max(0.0, time.perf_counter() - t0 - ta), b))
    pending.put(None)
    th.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat.sort()
    edges = sum(_req_edges(comp_edges, q, hg, srcs) for (_, q, hg, _, srcs) in plan)
    return {"requests": len(plan), "wall_s": wall,
            "served_per_s": len(plan) / wall, "served_gteps_bfs_bc": edges / wall / 1e9,
            "p50_ms": 1e3 * lat[len(lat) // 2], "p99_ms": 1e3 * lat[min(len(lat) - 1, int(0.99 * len(lat)))],
            "server_p50_ms": st["p50_s"] * 1e3, "server_p99_ms": st["p99_s"] * 1e3,
            "batches": st["batches"], "mean_requests_per_batch": st["mean_requests_per_batch"]}


def _one_call_per_request(torch, plan, comp_edges):
    """The same requests one synchronous C-ABI call each (host sources in, host results
    out), no batching and no overlap: the plain per-request form."""
    import gu
    t0 = time.perf_counter()
    for (_, q, hg, g, srcs) in plan:
        if q == gu.QUERY_BFS:
            g.bfs_host(srcs, variant="auto")
        else:
            sd = torch.as_tensor(srcs, device="cuda")
            if q == gu.QUERY_BC:
                o = torch.empty(hg.n, dtype=torch.float64, device="cuda")
                g.bc(sd, o)
            else:
                o = torch.zeros(len(srcs), dtype=torch.int64, device="cuda")
                g.reach(sd, o)
            o.cpu()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    edges = sum(_req_edges(comp_edges, q, hg, srcs) for (_, q, hg, _, srcs) in plan)
    return {"requests": len(plan), "wall_s": wall, "requests_per_s": len(plan) / wall,
            "gteps_bfs_bc": edges / wall / 1e9}


def serve_subline(torch, rate=800.0, seconds=1.0, burst=2000):
    """Short serving run for the default bench line, on 6 R-MAT graphs (scales 12-16) and 2
    random DAGs (n about 2^16) resident on the device, with the C5 request mix (BC of 64-256
    sources): p50 / p99 latency of a Poisson stream at `rate`, and at saturation (`burst`
    requests submitted at once) the served throughput against the same requests issued one
    synchronous call each; both forms run the saturation requests once untimed first."""
    rng = np.random.default_rng(11)
    rmats, dags, comp = _serving_set(torch, 6, (12, 16), 2, (16, 16.5), rng)
    plan = _serving_plan(rng, rmats, dags, rate, seconds, 256)
    sat_plan = [(0.0,) + p[1:] for p in _serving_plan(rng, rmats, dags, float(burst), 1.0, 256)[:burst]]
    # warm-up, untimed: the first pass of a process through the server and the one-call
    # form ran at about 70 % of later passes (5220 / 1363 against 7550 / 1740 requests/s)
    _serve_stream(sat_plan, comp)
    _one_call_per_request(torch, sat_plan, comp)
    lat = _serve_stream(plan, comp)
    sat = _serve_stream(sat_plan, comp)
    plain = _one_call_per_request(torch, sat_plan, comp)
    for _, _, g in rmats + dags:
        g.close()
    return {"workload": "6 R-MAT graphs (scales 12-16, ef 8/16/32) + 2 DAGs (n ~ 2^16, m = 8n); requests: 60% BFS "
                        "rows (1-256 sources), 20% BC (64-256), 20% DAG reachable counts (1-256); host buffers in "
                        "and out",
            "latency": {"offered_rate_per_s": rate, "requests": lat["requests"], "p50_ms": lat["p50_ms"],
                        "p99_ms": lat["p99_ms"], "mean_requests_per_batch": lat["mean_requests_per_batch"]},
            "saturation": {"requests": sat["requests"], "served_per_s": sat["served_per_s"],
                           "served_gteps_bfs_bc": sat["served_gteps_bfs_bc"],
                           "mean_requests_per_batch": sat["mean_requests_per_batch"],
                           "one_call_per_request_per_s": plain["requests_per_s"],
                           "speedup_vs_one_call_per_request": sat["served_per_s"] / plain["requests_per_s"]},
            "note": "latency is open-loop, from each request's planned arrival; at saturation every request is "
                    "submitted at once and the one-call form runs the same requests back to back"}


def wl_c5(args):
    """Serving at the stated configuration: 12 R-MAT graphs (scales 12-22, edge factors
    8/16/32) and 4 random DAGs (n = 2^16..2^20, m = 8n) resident; Poisson streams of 60%
    BFS rows (1-256 sources), 20% BC (64-1024 sources), 20% DAG reachable counts (1-256)
    at three rates, then a saturation burst against the same requests one call each."""
    import gu
    import oracle
    torch = _torch()
    rng = np.random.default_rng(5)
    t_build = time.perf_counter()
    rmats, dags, comp_edges = _serving_set(torch, 12, (12, 22), 4, (16, 20), rng)
    t_build = time.perf_counter() - t_build
    results = []
    for rate in (50.0, 200.0, 800.0):
        plan = _serving_plan(rng, rmats, dags, rate, 2.0, 1024)
        r = _serve_stream(plan, comp_edges)
        r["offered_rate_per_s"] = rate
        results.append(r)
    burst = [(0.0,) + p[1:] for p in _serving_plan(rng, rmats, dags, 1000.0, 1.0, 1024)[:600]]
    sat = _serve_stream(burst, comp_edges)
    one_by_one = _one_call_per_request(torch, burst, comp_edges)
    saturation = {"requests": sat["requests"], "served_per_s": sat["served_per_s"],
                  "served_gteps_bfs_bc": sat["served_gteps_bfs_bc"], "p50_ms": sat["p50_ms"],
                  "p99_ms": sat["p99_ms"], "mean_requests_per_batch": sat["mean_requests_per_batch"],
                  "one_call_per_request_per_s": one_by_one["requests_per_s"],
                  "one_call_per_request_gteps": one_by_one["gteps_bfs_bc"],
                  "speedup_vs_one_call_per_request": sat["served_per_s"] / one_by_one["requests_per_s"]}
    # CPU: per-request oracle time on a sample of requests of each kind
    cpu_ms = []
    for (t_, q, hg, g, srcs) in burst[:24]:
        if q == gu.QUERY_BC:
            _, c = _cpu(oracle.bc, hg.R, hg.C, hg.n, srcs[:8], nthreads=os.cpu_count() or 1)
            c *= len(srcs) / 8.0
        elif q == gu.QUERY_REACH:
            _, c = _cpu(oracle.reach_count, hg.R, hg.C, hg.n, srcs, nthreads=os.cpu_count() or 1)
        else:
            _, c = _cpu(oracle.bfs_multi, hg.R, hg.C, hg.n, srcs, nthreads=os.cpu_count() or 1)
        cpu_ms.append(c * 1e3)
    _emit({"workload": "c5_serving_rmat12-22_dag2^16-2^20", "metric": "request latency p50 / p99", "unit": "ms",
           "graphs": [n for n, _, _ in rmats + dags], "graph_build_s": t_build, "results": results,
           "saturation": saturation,
           "mix": "60% BFS rows (1-256 sources), 20% BC (64-1024 sources), 20% DAG reachable counts (1-256)",
           "client": "open loop from the planned arrivals, at most min(48 GiB, a quarter of the host's available "
                     "memory) of result buffers held",
           "cpu_per_request_ms_median": statistics.median(cpu_ms),
           "cpu_sample": "first 24 requests of the burst, oracle on all host threads (BC extrapolated "
                         "from 8 sources per request)"})


def wl_io(args):
    """Graph files at the boundary: R-MAT scale 20 (ef 16) written as METIS, SNAP
    and MatrixMarket text and as the binary CSR cache, read back by this library
    and -- where oracle/_ref holds the reference parser built from its sources --
    by the reference parser (parse.cpp:88-441).  Host only."""
    import subprocess
    import tempfile
    import gu
    hg = gu.HostGraph.rmat(20, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    ref = os.path.join(ROOT, "oracle", "_ref", "ref_oracle")
    res = {}
    with tempfile.TemporaryDirectory() as tmp:
        files = {}
        p = os.path.join(tmp, "g.graph")  # METIS: header, then 1-based neighbour lists
        with open(p, "w") as f:
            f.write(f"{hg.n} {hg.m // 2}\n")
            for v in range(0, hg.n, 65536):
                lo, hi = v, min(hg.n, v + 65536)
                f.write("".join(" ".join(map(str, (hg.C[hg.R[u]:hg.R[u + 1]] + 1).tolist())) + "\n"
                                for u in range(lo, hi)))
        files["dimacs"] = p
        # SNAP wants every id in 0..n-1 present: relabel away the isolated vertices
        keep = np.diff(hg.R) > 0
        newid = np.cumsum(keep) - 1
        Rk = np.concatenate([[0], np.cumsum(np.diff(hg.R)[keep])]).astype(np.int32)
        dense = gu.HostGraph(Rk, newid[hg.C].astype(np.int32), int(keep.sum()), True)
        p = os.path.join(tmp, "g.txt")
        dense.write_edgelist(p)
        files["edgelist"] = p
        p = os.path.join(tmp, "g.mtx")
        src = np.repeat(np.arange(hg.n, dtype=np.int64), np.diff(hg.R))
        keep = src < hg.C
        with open(p, "w") as f:
            f.write(f"%%MatrixMarket matrix coordinate pattern symmetric\n{hg.n} {hg.n} {int(keep.sum())}\n")
            np.savetxt(f, np.stack([src[keep] + 1, hg.C[keep].astype(np.int64) + 1], 1), fmt="%d")
        files["market"] = p
        p = os.path.join(tmp, "g.csr")
        hg.write_csr(p)
        files["csrbin"] = p
        for fmt, path in files.items():
            mb = os.path.getsize(path) / 1e6
            _, t = _cpu(gu.HostGraph.parse, path, fmt)
            row = {"file_mb": mb, "ours_s": t, "ours_mb_per_s": mb / t}
            if fmt != "csrbin" and os.path.exists(ref):
                t0 = time.perf_counter()
                subprocess.run([ref, "parse", path, fmt, os.path.join(tmp, "ref_" + fmt)], check=True,
                               stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
                row["reference_s"] = time.perf_counter() - t0
                row["speedup"] = row["reference_s"] / t
            res[fmt] = row
    _emit({"workload": "io_rmat20_ef16_graph_files", "metric": "graph file read time", "unit": "s",
           "n": hg.n, "m_csr": hg.m, "results": res,
           "note": "reference_s includes writing its CSR out (a few hundred MB), a small share"})


def wl_dag(args):
    """All-vertex reachability of random DAGs (m = 8n): gu_dag_reach against the
    oracle's bitset closure (n = 2^16) and a per-vertex BFS sample (n = 2^18)."""
    import gu
    import oracle
    torch = _torch()
    cores = os.cpu_count() or 1
    res = {}
    for n, seed in ((1 << 16, 1), (1 << 18, 2)):
        hg = gu.HostGraph.dag(n, 8 * n, seed=seed)
        g = gu.Graph(hg)
        cnt = torch.empty(n, dtype=torch.int64, device="cuda")
        tot = g.dag_reach(cnt)
        c = _median_call_ms(lambda: g.dag_reach(cnt), reps=3)
        row = {"m": hg.m, "pairs": tot, "gpu_call_ms": c}
        if n <= 1 << 16:
            (_, rtot), t = _cpu(oracle.dag_reach_counts, hg.R, hg.C, hg.n)
            row.update({"cpu_bitset_closure_ms_1thread": t * 1e3, "pairs_match": rtot == tot})
        sub = np.arange(0, n, max(1, n // (4 * cores)), dtype=np.int32)[: 4 * cores]
        _, t = _cpu(oracle.reach_count, hg.R, hg.C, hg.n, sub, nthreads=cores)
        row[f"cpu_bfs_per_vertex_extrapolated_ms_{cores}threads"] = t / len(sub) * n * 1e3
        res[f"n{n}"] = row
        g.close()
    _emit({"workload": "dag_reach_m8n", "metric": "all-vertex DAG reachability", "unit": "ms", "results": res,
           "note": "the reference's recursion with std::set per vertex is the baseline these restate"})


def run(workload, args):
    {"c1": wl_c1, "c3": wl_c3, "c3-pass": wl_c3_pass, "c3-launch": wl_c3_launch, "c4": wl_c4, "c4-pass": wl_c4_pass, "lbs": wl_lbs, "c5": wl_c5, "io": wl_io, "dag": wl_dag}[workload](args)

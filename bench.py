"""Benchmark: multi-source BFS GTEPS on one GB300 (R-MAT scale 20, 512 sources).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the headline multi-source BFS configuration): undirected R-MAT,
scale 20 (2^20 vertices), edge factor 16, (a,b,c,d) = (0.57,0.19,0.19,0.05),
symmetrised, duplicates and self-loops removed, vertex labels permuted, seed 1;
512 distinct sources drawn uniformly with seed 2; int32 distance rows.

One step = one multi-source BFS over the 512 sources (one persistent kernel
launch).  GTEPS counts, per source, the undirected edges of the component it
reaches (Graph500 convention: sum over sources of scanned CSR entries / 2).

ours:      `value`  -- device-resident inputs, CUDA events around K steps.
           `e2e`    -- the C-ABI host-buffer call (gu_bfs_host): pinned host
                       sources in, pinned host distance rows out, copies inside.
Also on the default line (one GPU): `bc`, sampled Brandes BC on R-MAT scale 18
(8192 sources, 1024 per pass: GTEPS, kernel time, physical DRAM fraction, error
against the FP64 oracle), and `serve`, a short serving run (p50 / p99 at a
moderate rate; saturation throughput against one call per request).

reference: the oracle port of the reference CPU path
           (examples/multi_search/multi_search_test.cu:17-38) on all host
           threads, each step a bounded sample of the sources.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "graph-utils_gb300"))

import numpy as np  # noqa: E402

SCALE, EDGE_FACTOR, GRAPH_SEED, K_SOURCES, SOURCE_SEED = 20, 16, 1, 512, 2
WORKLOAD = "rmat20_ef16_512src_bfs"  # the default workload's name


def workload_name(scale, k):
    """rmat<scale>_ef16_<k>src_bfs: the default names the headline workload."""
    return f"rmat{scale}_ef{EDGE_FACTOR}_{k}src_bfs"
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--variant", default="auto")
    p.add_argument("--scale", type=int, default=SCALE)
    p.add_argument("--sources", type=int, default=K_SOURCES)
    p.add_argument("--autotune", action="store_true",
                   help="before the timed region, time AUTO's candidates on the workload's sources "
                        "(gu_graph_autotune) and keep the fastest; reported under 'tuning'")
    p.add_argument("--no-sublines", action="store_true",
                   help="leave out the sampled-BC and serving objects of the default line")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the cpu_baseline sample")
    p.add_argument("--kernel-only", action="store_true", help="skip e2e (for profiling runs)")
    p.add_argument("--power", action="store_true",
                   help="sample board power (NVML, read-only) during the timed region: adds a power object")
    p.add_argument("--workload", choices=["c2", "c1", "c3", "c3-pass", "c3-launch", "c4", "c4-pass", "lbs", "c5", "io", "dag"], default="c2",
                   help="c2: the headline BFS line (default); c1/c3/c4/c5/io/dag: the other configurations, "
                        "one JSON line each (bench_configs.py)")
    return p.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws, device=None):
    """The largest of the ranks' values (every rank gets it); x itself on one rank.
    The job's time is its slowest rank's, as the timing contract asks."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_gteps(ws, edges_per_rank_step, steps, seconds):
    """Whole-job GTEPS: every rank (a replica) processes the same edges per step."""
    return ws * edges_per_rank_step * steps / seconds / 1e9


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


PROFILE = os.path.join(ROOT, "profiles", "ms_grid_kernel_auto_rmat20.md")
KERNEL_SOURCES = ("msbfs.cu", "device_utils.cuh", "gu_internal.h")


def kernel_source_hash():
    """sha256 (first 16 hex digits) of the batched BFS kernel's sources, as the
    ncu summary records it for the build it profiled."""
    import hashlib
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(ROOT, "graph-utils_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def ncu_traffic_per_launch():
    """(dram bytes per launch, source hash) of the dominant kernel from the committed ncu summary."""
    if not os.path.exists(PROFILE):
        return None, None
    traffic = src = None
    for line in open(PROFILE):
        key, _, val = line.partition(":")
        if key == "traffic_bytes_per_launch":
            try:
                traffic = int(val.strip())
            except ValueError:
                traffic = None
        elif key == "kernel_source_sha16":
            src = val.strip()
    return traffic, src


def alg_min_bytes(n, m, k):
    """Batch-aware algorithmic minimum of one launch: per batch of up to 256 sources
    (W = ceil(k_b / 64) 64-bit words per vertex) the distance rows are written once
    (4 n bytes per source), the CSR is read once (4 (n + 1) + 4 m) and the per-vertex
    seen words are written once (8 W n)."""
    total = 0.0
    for b in range(0, k, 256):
        kb = min(256, k - b)
        words = (kb + 63) // 64
        total += 4.0 * n * kb + 4.0 * (n + 1) + 4.0 * m + 8.0 * words * n
    return total


def roofline_line(traffic, traffic_src, kt_avg, alg_eff, alg_min, peak, peak_kind):
    """The roofline object: frac is the physical DRAM fraction (ncu bytes per launch over
    the live kernel time); the batch-aware minimum and the per-source model beside it."""
    phys = traffic / kt_avg / 1e9 if traffic else None
    src_now = kernel_source_hash()
    return {"bound": "hbm", "achieved": phys, "peak": peak, "unit": "GB/s",
            "frac": phys / peak if phys else None, "traffic": traffic,
            "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
            else "fallback 6800 GB/s",
            "kernel": "gu::ms_grid_kernel<V,4>", "kernel_ms": 1e3 * kt_avg,
            "achieved_basis": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch (traffic, "
                              "profiles/ms_grid_kernel_auto_rmat20.md) / this run's mean CUDA-event kernel time",
            "traffic_kernel_source_sha16": traffic_src, "kernel_source_sha16": src_now,
            "traffic_matches_build": traffic_src == src_now,
            "alg_min_bytes": alg_min, "alg_min_achieved": alg_min / kt_avg / 1e9,
            "alg_min_frac": alg_min / kt_avg / 1e9 / peak,
            "traffic_over_alg_min": traffic / alg_min if traffic else None,
            "alg_min_model": "per 256-source batch: rows 4 n k_b + CSR 4 (n+1) + 4 m + seen 8 W n",
            "effective_bytes": alg_eff, "effective_frac": alg_eff / kt_avg / 1e9 / peak,
            "effective_model": "per-source 4n + 8 V_s + 8 E_s summed over the sources (a batch shares its "
                               "CSR and bitmap reads among 256 sources, so this can exceed 1)"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        except OSError:
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def config_of(args, hg):
    """The workload's config object, the same on both arms."""
    return {"workload": workload_name(args.scale, args.sources), "scale": args.scale,
            "edge_factor": EDGE_FACTOR, "rmat_abcd": [0.57, 0.19, 0.19, 0.05], "n": hg.n, "m_csr": hg.m,
            "sources": args.sources, "graph_seed": GRAPH_SEED, "source_seed": SOURCE_SEED,
            "variant": args.variant,
            "l2": "inputs larger than L2 (CSR 134 MB + 2 GiB distance rows per step)"}


def build_workload(scale, k):
    import gu
    hg = gu.HostGraph.rmat(scale, EDGE_FACTOR, 0.57, 0.19, 0.19, seed=GRAPH_SEED, permute=True)
    srcs = gu.sources(hg.n, k, seed=SOURCE_SEED)
    return hg, srcs


def edges_and_bytes(torch, dist, deg, n):
    """Per-source scanned CSR entries E_s and reached vertices V_s, on the GPU."""
    INF = 2147483647
    E = torch.zeros(dist.shape[0], dtype=torch.float64, device=dist.device)
    V = torch.zeros(dist.shape[0], dtype=torch.float64, device=dist.device)
    for b in range(0, dist.shape[0], 64):
        reached = dist[b:b + 64] != INF
        E[b:b + 64] = (reached.to(torch.float64) @ deg)
        V[b:b + 64] = reached.sum(1).to(torch.float64)
    E_tot = float(E.sum())
    V_tot = float(V.sum())
    # algorithmic bytes per source: 4n (distance row) + 8 V_s (R pairs) + 8 E_s (C + dist check)
    alg_bytes = dist.shape[0] * 4.0 * n + 8.0 * V_tot + 8.0 * E_tot
    return E_tot, V_tot, alg_bytes


def cpu_model():
    """The host CPU as /proc/cpuinfo names it (x86: model name; Arm: implementer and part codes)."""
    import platform
    try:
        with open("/proc/cpuinfo") as f:
            info = f.read().splitlines()
    except OSError:
        return platform.machine()
    fields = {}
    for line in info:
        if ":" in line:
            k, v = line.split(":", 1)
            fields.setdefault(k.strip(), v.strip())
    if "model name" in fields:
        return fields["model name"]
    parts = [f"{k} {fields[k]}" for k in ("CPU implementer", "CPU part") if k in fields]
    return platform.machine() + (" (" + ", ".join(parts) + ")" if parts else "")


def cpu_one_thread(hg, srcs, nsrc=4):
    """The oracle port on one host thread over the first `nsrc` sources: GTEPS."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    part = np.asarray(srcs[:nsrc])
    t0 = time.perf_counter()
    _, scanned = oracle.bfs_multi(hg.R, hg.C, hg.n, part, nthreads=1)
    return scanned / 2.0 / (time.perf_counter() - t0) / 1e9, len(part)


def cpu_sample(hg, srcs, seconds):
    """Oracle port on all host threads over growing source samples until `seconds`."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    cores = os.cpu_count() or 1
    done, edges, t_total = 0, 0, 0.0
    chunk = cores
    while done < len(srcs) and t_total < seconds:
        part = srcs[done:done + chunk]
        t0 = time.perf_counter()
        _, scanned = oracle.bfs_multi(hg.R, hg.C, hg.n, part, nthreads=cores)
        t_total += time.perf_counter() - t0
        edges += scanned
        done += len(part)
    return edges / 2.0, t_total, done, cores


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    # the input is built by the oracle's own restatement of the generator (the same CSR and
    # sources as the library's), so that this arm runs without the library
    R, C = oracle.rmat(args.scale, EDGE_FACTOR, 0.57, 0.19, 0.19, seed=GRAPH_SEED, permute=True)

    class _Graph:
        pass
    hg = _Graph()
    hg.R, hg.C, hg.n, hg.m = R, C, len(R) - 1, len(C)
    srcs = oracle.sources(hg.n, args.sources, SOURCE_SEED)
    cores = os.cpu_count() or 1
    per_step = cores  # one source per host thread per step
    times, edges = [], []
    off = 0
    for i in range(args.warmup + args.steps):
        part = np.take(srcs, np.arange(off, off + per_step) % len(srcs))
        off += per_step
        t0 = time.perf_counter()
        _, scanned = oracle.bfs_multi(hg.R, hg.C, hg.n, part, nthreads=cores)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
            edges.append(scanned / 2.0)
    T = sum(times)
    value = sum(edges) / T / 1e9
    sample = f"{per_step} sources per step ({cores} host threads), of the {args.sources} workload sources"
    v1, n1 = cpu_one_thread(hg, srcs)
    line = {"impl": "reference", "metric": "multi-source BFS GTEPS", "value": value, "unit": "GTEPS",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * T / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic",
            "config": config_of(args, hg),
            "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": cores, "kind": "port", "sample": sample,
                             "value_1thread": v1, "sample_1thread": f"first {n1} workload sources on one thread",
                             "cpu_model": cpu_model()},
            "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import gu
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    hg, srcs = build_workload(args.scale, args.sources)
    g = gu.Graph(hg)
    stream = torch.cuda.Stream(device=dev)
    s_dev = torch.as_tensor(srcs, device=dev)
    dist_buf = torch.empty((len(srcs), hg.n), dtype=torch.int32, device=dev)
    deg = torch.as_tensor(np.diff(hg.R).astype(np.float64), device=dev)

    tuning = None
    if args.autotune:
        best, trials = g.autotune(s_dev)
        tuning = {"best": best, "trials": len(trials)}

    def step():
        g.bfs(s_dev, dist_buf, variant=args.variant, stream=stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    E_tot, V_tot, alg_bytes = edges_and_bytes(torch, dist_buf, deg, hg.n)
    gteps_edges = E_tot / 2.0  # undirected graph: each edge once per reaching source

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    kernel_times = []
    levels = None
    power = None
    psampler = gu.PowerSampler(local, 10) if args.power else None
    with ClockSampler(local) as clk:
        if psampler:
            psampler.__enter__()
        barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        barrier()
        # the kernel of every step, from the library's own CUDA events on the launch
        # stream (kept for the last 64 launches), read after the timed region
        kernel_times = g.launch_times()[-args.steps:]
        _, td, bu, ml = g.last_launch()
        levels = (td, bu, ml)
        if psampler:
            psampler.__exit__(None, None, None)
    clocks = clk.summary()
    t_total = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, ws, dev)
    value = job_gteps(ws, gteps_edges, args.steps, t_total)
    if psampler:
        power = {"avg_w": psampler.watts, "samples": psampler.samples,
                 "gteps_per_w": value / ws / psampler.watts if psampler.watts else None,
                 "source": "NVML power draw of this rank's GPU, sampled every 10 ms over the timed region"}

    e2e = None
    if not args.kernel_only:
        pin_src = torch.as_tensor(srcs).pin_memory()
        pin_out = torch.empty((len(srcs), hg.n), dtype=torch.int32).pin_memory()
        src_np, out_np = pin_src.numpy(), pin_out.numpy()
        for _ in range(max(1, args.warmup // 2)):
            g.bfs_host(src_np, args.variant, out=out_np, stream=stream)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            g.bfs_host(src_np, args.variant, out=out_np, stream=stream)
        barrier()
        t_e2e = max_over_ranks(time.perf_counter() - t0, ws, dev)
        ok = np.array_equal(out_np[:4], dist_buf[:4].cpu().numpy())
        e2e = {"value": job_gteps(ws, gteps_edges, args.steps, t_e2e), "unit": "GTEPS",
               "h2d_bytes_per_step": int(srcs.nbytes), "d2h_bytes_per_step": int(len(srcs) * hg.n * 4),
               "ms_per_step": 1e3 * t_e2e / args.steps, "host_rows_match_device": bool(ok)}

    peak, peak_kind = peaks()
    kt_avg = statistics.mean(kernel_times)
    traffic, traffic_src = ncu_traffic_per_launch()
    roofline = roofline_line(traffic, traffic_src, kt_avg, alg_bytes, alg_min_bytes(hg.n, hg.m, len(srcs)),
                             peak, peak_kind)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        e_cpu, t_cpu, nsrc, cores = cpu_sample(hg, srcs, args.cpu_seconds)
        v1, n1 = cpu_one_thread(hg, srcs)
        cpu = {"value": e_cpu / t_cpu / 1e9, "unit": "GTEPS", "cores": cores, "kind": "port",
               "sample": f"first {nsrc} of the {len(srcs)} workload sources, oracle port of "
                         f"multi_search_test.cu:17-38 on {cores} host threads, {t_cpu:.1f} s",
               "value_1thread": v1, "sample_1thread": f"first {n1} workload sources on one thread",
               "cpu_model": cpu_model()}

    sub = {}
    if rank == 0 and ws == 1 and not (args.kernel_only or args.no_sublines):
        import bench_configs
        g.close()
        del dist_buf
        torch.cuda.empty_cache()
        sub["bc"] = bench_configs.bc_subline(torch)
        sub["serve"] = bench_configs.serve_subline(torch)

    if rank == 0:
        line = {"metric": "multi-source BFS GTEPS", "value": value, "unit": "GTEPS", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
                "data": "synthetic",
                "config": config_of(args, hg),
                "workload_stats": {"edges_per_step": gteps_edges, "levels_td_bu_max": levels},
                "tuning": tuning,
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
                "gpu_launches": args.steps}
        if power:
            line["power"] = power
        line.update(sub)
        print(json.dumps(line), flush=True)
    g.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse_args()
    if args.workload != "c2":
        import bench_configs
        bench_configs.run(args.workload, args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

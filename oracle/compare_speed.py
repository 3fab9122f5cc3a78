"""Single-thread speed of the oracle's BFS port against the reference's own
BFS checker (examples/multi_search/multi_search_test.cu:17-38, compiled from
the reference sources into oracle/_ref/ref_oracle by oracle/build_ref.sh), on
the same graph and sources.  Test infrastructure: it shows that the CPU
baseline measured with the port is the reference's speed, not a slower stand-in.

    python oracle/compare_speed.py [--scale 20] [--sources 16]

Prints one JSON line with both rates (GTEPS, Graph500 count: scanned CSR
entries / 2) and their ratio.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "graph-utils_gb300"))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--scale", type=int, default=20)
    p.add_argument("--sources", type=int, default=16)
    args = p.parse_args()
    ref = os.path.join(HERE, "_ref", "ref_oracle")
    if not os.path.exists(ref):
        sys.exit("oracle/_ref/ref_oracle is not built (oracle/build_ref.sh needs the reference tree)")
    import gu
    import oracle
    # the multi-source BFS benchmark graph and the first sources of its source list
    hg = gu.HostGraph.rmat(args.scale, 16, 0.57, 0.19, 0.19, seed=1, permute=True)
    srcs = gu.sources(hg.n, 512, seed=2)[:args.sources]
    with tempfile.TemporaryDirectory() as d:
        pre = os.path.join(d, "g")
        np.asarray(hg.R, np.int32).tofile(pre + ".R")
        np.asarray(hg.C, np.int32).tofile(pre + ".C")
        with open(pre + ".meta", "w") as f:
            f.write(f"{hg.n} {hg.m} 0\n")
        np.asarray(srcs, np.int32).tofile(os.path.join(d, "s.i32"))
        out = subprocess.run([ref, "time_bfs", pre, os.path.join(d, "s.i32")], check=True,
                             capture_output=True, text=True).stdout.split()
    t_ref, e_ref = float(out[0]), int(out[1])
    t0 = time.perf_counter()
    _, e_port = oracle.bfs_multi(hg.R, hg.C, hg.n, srcs, nthreads=1)
    t_port = time.perf_counter() - t0
    if e_port != e_ref:
        sys.exit(f"scanned entries differ: port {e_port}, reference {e_ref}")
    r_ref, r_port = e_ref / 2 / t_ref / 1e9, e_port / 2 / t_port / 1e9
    print(json.dumps({"graph": f"rmat{args.scale}_ef16", "sources": len(srcs), "threads": 1,
                      "reference_gteps": r_ref, "port_gteps": r_port, "port_over_reference": r_port / r_ref,
                      "reference_s": t_ref, "port_s": t_port}))


if __name__ == "__main__":
    main()

"""Regenerate the golden vectors in tests/golden/ from the reference's own code.

Run in a container that has the reference tree (default /root/reference, or
$GU_REFERENCE): it builds oracle/_ref/ref_oracle from the reference sources
(oracle/build_ref.sh), parses the reference's graph fixtures with the
reference parser (parse.cpp), runs the reference CPU checkers on them and on
small seeded synthetic graphs, and writes one compressed .npz per case:

  R, C, n, directed          CSR as parsed / generated
  sources                    the sources the checkers ran from
  dist                       examples/multi_search/multi_search_test.cu:17-38
  sigma                      examples/counting_shortest_paths/shortest_paths.cu:11-39
  delta_f32                  examples/betweenness_centrality/bc.cu:11-57
  diameter                   examples/diameter_sampling/diameter_sampling_test.cu:9-38
  dag_pairs (DAG cases)      graph-utils/dag_reachability.cpp:36-65
and lbs_*.npz with counts, scanned, result (examples/load_balanced_search/lbs.cu:18-31),
and parse_<case>.{graph,txt,mtx} + parse_<case>.npz: small graph files in the
reference's three text formats, written with the quirks its parser has to cope
with (comments, double separators, '\r' line ends, extra fields, unsorted
lines), and the CSR the reference parser (parse.cpp:88-441) builds from them.

    python tests/golden/make_golden.py [--only parse]
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "graph-utils_gb300"))
REF = os.environ.get("GU_REFERENCE", "/root/reference")
REF_ORACLE = os.path.join(ROOT, "oracle", "_ref", "ref_oracle")


def run(*args):
    subprocess.run([REF_ORACLE] + [str(a) for a in args], check=True)


def write_csr(prefix, R, C, n, directed):
    np.asarray(R, np.int32).tofile(prefix + ".R")
    np.asarray(C, np.int32).tofile(prefix + ".C")
    with open(prefix + ".meta", "w") as f:
        f.write(f"{n} {len(C)} {int(directed)}\n")


def read_csr(prefix):
    R = np.fromfile(prefix + ".R", np.int32)
    C = np.fromfile(prefix + ".C", np.int32)
    n, m, d = map(int, open(prefix + ".meta").read().split())
    return R, C, n, bool(d)


def golden_case(tmp, name, R, C, n, directed, sources, dag=False):
    pre = os.path.join(tmp, name)
    write_csr(pre, R, C, n, directed)
    src = np.asarray(sources, np.int32)
    src.tofile(pre + ".src")
    run("run", pre, pre + ".src", pre + ".out")
    k = len(src)
    out = dict(R=np.asarray(R, np.int32), C=np.asarray(C, np.int32), n=np.int32(n), directed=np.bool_(directed),
               sources=src,
               dist=np.fromfile(pre + ".out.dist", np.int32).reshape(k, n),
               sigma=np.fromfile(pre + ".out.sigma", np.uint64).reshape(k, n),
               delta_f32=np.fromfile(pre + ".out.delta_f32", np.float32).reshape(k, n),
               diameter=np.fromfile(pre + ".out.diameter", np.int32)[0])
    if dag:
        run("dag", pre, pre + ".dag")
        out["dag_pairs"] = np.fromfile(pre + ".dag.pairs", np.int64)[0]
    np.savez_compressed(os.path.join(HERE, f"graph_{name}.npz"), **out)
    print(f"graph_{name}: n={n} m={len(C)} k={k} diameter={out['diameter']}")


def write_metis(path, R, C, n, rng):
    """METIS text with comments, a header, and per-line quirks: double spaces
    (the reference drops the field that follows), tabs, trailing blanks and
    '\r' line ends (the reference drops a field ending in '\r')."""
    lines = ["% written for the parser parity fixtures", f"{n} {len(C) // 2} "]
    for v in range(n):
        nb = [str(int(c) + 1) for c in C[R[v]:R[v + 1]]]
        sep = [" "] * max(len(nb) - 1, 0)
        for i in range(len(sep)):
            u = rng.random()
            sep[i] = "  " if u < 0.05 else ("\t" if u < 0.15 else " ")
        line = "".join(x + y for x, y in zip(nb, sep + [""]))
        u = rng.random()
        if u < 0.1:
            line += " "
        elif u < 0.15:
            line += "\r"
        lines.append(line)
        if rng.random() < 0.02:
            lines.append("% a comment between vertex lines")
    with open(path, "w", newline="") as f:
        f.write("\n".join(lines) + "\n")


def write_snap(path, R, C, n, rng, shuffle_some=False):
    """SNAP edge list, 0-based, '#' comments, tabs or spaces, some extra fields;
    optionally a few lines out of source order (the reference induces R as if
    sorted, and the parity covers that too)."""
    rows = [(v, int(c)) for v in range(n) for c in C[R[v]:R[v + 1]]]
    if shuffle_some:
        for _ in range(3):
            i, j = rng.integers(0, len(rows), 2)
            rows[i], rows[j] = rows[j], rows[i]
    lines = ["# Directed graph written for the parser parity fixtures", "# FromNodeId\tToNodeId"]
    for u, v in rows:
        sep = "\t" if rng.random() < 0.5 else " "
        extra = " 1.0" if rng.random() < 0.05 else ""
        lines.append(f"{u}{sep}{v}{extra}")
    with open(path, "w", newline="") as f:
        f.write("\n".join(lines) + "\n")


def write_market(path, R, C, n, rng):
    """MatrixMarket pattern matrix: one entry per undirected edge, in random order."""
    ent = [(v + 1, int(c) + 1) for v in range(n) for c in C[R[v]:R[v + 1]] if v < c]
    rng.shuffle(ent)
    lines = ["%%MatrixMarket matrix coordinate pattern symmetric", "% parser parity fixture", f"{n} {n} {len(ent)}"]
    lines += [f"{a} {b}" for a, b in ent]
    with open(path, "w", newline="") as f:
        f.write("\n".join(lines) + "\n")


def parse_cases(tmp):
    import gu
    rng = np.random.default_rng(17)
    g = gu.HostGraph.rmat(8, 8, seed=23)
    d = gu.HostGraph.dag(200, 900, seed=29)
    cases = [("metis_rmat8", "graph", "dimacs", lambda p: write_metis(p, g.R, g.C, g.n, rng)),
             ("snap_dag200", "txt", "edgelist", lambda p: write_snap(p, d.R, d.C, d.n, rng)),
             ("snap_unsorted", "txt", "edgelist", lambda p: write_snap(p, d.R, d.C, d.n, rng, True)),
             ("snap_h_dag200", "txt", "edgelist_h", lambda p: write_snap(p, d.R, d.C, d.n, rng)),
             ("market_rmat8", "mtx", "market", lambda p: write_market(p, g.R, g.C, g.n, rng))]
    for name, ext, fmt, writer in cases:
        path = os.path.join(HERE, f"parse_{name}.{ext}")
        writer(path)
        pre = os.path.join(tmp, "parse_" + name)
        run("parse", path, fmt, pre)
        R, C, n, directed = read_csr(pre)
        C = C[: R[n]]  # the reference sizes C from the header; only R[n] entries are the graph
        np.savez_compressed(os.path.join(HERE, f"parse_{name}.npz"), R=R, C=C, n=np.int32(n),
                            directed=np.bool_(directed), format=np.str_(fmt), input=np.str_(os.path.basename(path)))
        print(f"parse_{name}: {fmt} n={n} m={R[n]}")


def main():
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    if sys.argv[1:] == ["--only", "parse"]:
        with tempfile.TemporaryDirectory() as tmp:
            parse_cases(tmp)
        return
    import gu
    with tempfile.TemporaryDirectory() as tmp:
        parse_cases(tmp)
        # the reference's own fixtures, parsed by the reference parser
        files = [(f"test{i}", f"test{i}.graph", "dimacs") for i in range(1, 7)]
        files += [("jazz", "jazz.graph", "dimacs"), ("test7", "test7.txt", "edgelist")]
        for name, fn, fmt in files:
            pre = os.path.join(tmp, name + "_parsed")
            run("parse", os.path.join(REF, "graphs", fn), fmt, pre)
            R, C, n, directed = read_csr(pre)
            golden_case(tmp, name, R, C, n, directed, np.arange(n), dag=(name == "test7"))
        # seeded synthetic graphs (generators of this library)
        g = gu.HostGraph.er(198, 2742, seed=1)
        golden_case(tmp, "er198", g.R, g.C, g.n, False, np.arange(g.n))
        g = gu.HostGraph.rmat(9, 16, seed=5)
        golden_case(tmp, "rmat9", g.R, g.C, g.n, False, gu.sources(g.n, 70, seed=2))
        g = gu.HostGraph.grid(24, 20, 0.05, seed=7)
        golden_case(tmp, "grid24x20", g.R, g.C, g.n, False, gu.sources(g.n, 40, seed=2))
        g = gu.HostGraph.dag(300, 2400, seed=3)
        golden_case(tmp, "dag300", g.R, g.C, g.n, True, gu.sources(g.n, 50, seed=2), dag=True)
        # load-balanced search
        rng = np.random.default_rng(11)
        cases = {"random": rng.integers(0, 100, 5000), "zeros": np.zeros(64, np.int64),
                 "sparse": np.where(rng.random(3000) < 0.1, rng.integers(1, 2000, 3000), 0),
                 "single": np.array([37])}
        for cname, counts in cases.items():
            pre = os.path.join(tmp, "lbs_" + cname)
            counts = np.asarray(counts, np.int32)
            counts.tofile(pre + ".counts")
            run("lbs", pre + ".counts", pre)
            np.savez_compressed(os.path.join(HERE, f"lbs_{cname}.npz"), counts=counts,
                                scanned=np.fromfile(pre + ".scanned", np.int32),
                                result=np.fromfile(pre + ".result", np.int32))
            print(f"lbs_{cname}: N={len(counts)} total={int(counts.sum())}")


if __name__ == "__main__":
    main()

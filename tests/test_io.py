"""Graph files: the readers build the same CSR as the reference parser.

parse_<case>.* in tests/golden are small files in the reference's three text
formats, written with the quirks its parser copes with (comments, double
separators, '\\r' line ends, extra fields, out-of-order lines); parse_<case>.npz
holds the CSR the reference parser (parse.cpp:88-441) built from each
(tests/golden/make_golden.py).  Host code only: no GPU.
"""
import glob
import os
import sys

import numpy as np
import pytest

import gu
from conftest import GOLDEN

sys.path.insert(0, GOLDEN)


def parse_cases():
    return sorted(os.path.basename(p)[6:-4] for p in glob.glob(os.path.join(GOLDEN, "parse_*.npz")))


@pytest.mark.parametrize("case", parse_cases())
def test_reader_matches_reference_parser(case):
    ref = dict(np.load(os.path.join(GOLDEN, f"parse_{case}.npz")))
    g = gu.HostGraph.parse(os.path.join(GOLDEN, str(ref["input"])), str(ref["format"]))
    assert g.n == int(ref["n"])
    np.testing.assert_array_equal(g.R, ref["R"])
    np.testing.assert_array_equal(g.C, ref["C"])
    if str(ref["format"]) != "market":  # the reference leaves `directed` unset for MatrixMarket
        assert g.directed == bool(ref["directed"])


def test_quirks_are_reproduced():
    """The METIS fixture loses the fields that follow a double space or end in '\\r',
    exactly as the reference parser does; the MatrixMarket one keeps every entry."""
    metis = dict(np.load(os.path.join(GOLDEN, "parse_metis_rmat8.npz")))
    market = dict(np.load(os.path.join(GOLDEN, "parse_market_rmat8.npz")))
    assert int(metis["R"][-1]) < int(market["R"][-1])


def test_reference_fixture_files_when_present():
    """The reference's own graph files, where its tree is present, give the CSRs
    its parser gave (graph_<name>.npz)."""
    import make_golden
    root = os.path.join(make_golden.REF, "graphs")
    if not os.path.isdir(root):
        pytest.skip("reference tree not present")
    files = [(f"test{i}", f"test{i}.graph", "dimacs") for i in range(1, 7)]
    files += [("jazz", "jazz.graph", "dimacs"), ("test7", "test7.txt", "edgelist")]
    for name, fn, fmt in files:
        ref = dict(np.load(os.path.join(GOLDEN, f"graph_{name}.npz")))
        g = gu.HostGraph.parse(os.path.join(root, fn), fmt)
        np.testing.assert_array_equal(g.R, ref["R"], err_msg=name)
        np.testing.assert_array_equal(g.C, ref["C"][: ref["R"][-1]], err_msg=name)


def test_binary_cache_round_trip(tmp_path):
    g = gu.HostGraph.rmat(12, 16, seed=3)
    p = tmp_path / "g.csr"
    g.write_csr(p)
    h = gu.HostGraph.parse(p, "csrbin")
    assert (h.n, h.directed) == (g.n, g.directed)
    np.testing.assert_array_equal(h.R, g.R)
    np.testing.assert_array_equal(h.C, g.C)
    d = gu.HostGraph.dag(500, 3000, seed=4)
    d.write_csr(p)
    assert gu.HostGraph.parse(p, "csrbin").directed


def test_edgelist_writer_round_trip(tmp_path):
    """write_edgelist_to_file output reads back as the same directed CSR."""
    g = gu.HostGraph.grid(20, 30, 0.0, seed=1)  # no isolated vertex: every id appears
    p = tmp_path / "g.txt"
    g.write_edgelist(p)
    h = gu.HostGraph.parse(p, "edgelist")
    np.testing.assert_array_equal(h.R, g.R)
    np.testing.assert_array_equal(h.C, g.C)
    g.write_edgelist(p, header=True)
    first = open(p).readline().split()
    assert first == [str(g.n), str(g.m)]


def test_count_degree_zero():
    g = gu.HostGraph.rmat(10, 4, seed=3)
    assert g.count_degree_zero() == int((np.diff(g.R) == 0).sum()) > 0


@pytest.mark.parametrize("fmt,text,status", [
    ("dimacs", "3 2 1\n2\n1 3\n2\n", 7),              # weighted header
    ("dimacs", "2 1\n2\n1\n3\n", 1),                  # more vertex lines than n
    ("dimacs", "2 1\n2 3\n1\n", 1),                   # neighbour beyond n
    ("edgelist", "0 1\n5\n", 1),                      # a line with one field
    ("edgelist", "0 1\n1 7\n", 1),                    # ids not dense
    ("market", "3 3\n1 2\n", 1),                      # size line without nnz
    ("market", "3 3 1\n1 2 1.5\n", 1),                # not a pattern matrix
    ("nosuch", "1 0\n\n", 7),
])
def test_malformed_files_report_status(tmp_path, fmt, text, status):
    p = tmp_path / "bad"
    p.write_text(text)
    with pytest.raises(gu.GuError) as e:
        gu.HostGraph.parse(p, fmt)
    assert e.value.status == status


def test_missing_file():
    with pytest.raises(gu.GuError) as e:
        gu.HostGraph.parse("no/such/file.graph", "dimacs")
    assert e.value.status == 1


def test_convert_tool(tmp_path, capsys):
    """The convert example's flow: METIS in, edge list (or CSR cache) out."""
    import convert
    ref = dict(np.load(os.path.join(GOLDEN, "parse_metis_rmat8.npz")))
    src = os.path.join(GOLDEN, str(ref["input"]))
    out = tmp_path / "g.txt"
    assert convert.main(["-i", src, "-f", "dimacs", "-o", str(out)]) == 0
    assert f"Number of vertices: {int(ref['n'])}" in capsys.readouterr().out
    rows = np.loadtxt(out, dtype=np.int64).reshape(-1, 2)
    np.testing.assert_array_equal(rows[:, 1], ref["C"])
    np.testing.assert_array_equal(np.bincount(rows[:, 0], minlength=int(ref["n"])), np.diff(ref["R"]))
    csr = tmp_path / "g.csr"
    assert convert.main(["-i", src, "-f", "dimacs", "-o", str(csr), "--csr"]) == 0
    h = gu.HostGraph.parse(csr, "csrbin")
    np.testing.assert_array_equal(h.R, ref["R"])
    np.testing.assert_array_equal(h.C, ref["C"])
    assert convert.main(["-i", src, "-f", "dimacs"]) == 1


def test_multi_range_files_vs_reference_parser(tmp_path):
    """Where the reference checkers were built here: files of several MB, which the
    readers split into line ranges parsed by many threads, give the CSR the
    reference parser gives (parse.cpp:115-441), in every format, with the METIS
    quirks (double spaces, tabs, trailing blanks, '\\r') and unsorted SNAP lines."""
    import subprocess
    import make_golden as M
    if not os.path.exists(M.REF_ORACLE):
        pytest.skip("reference checkers not built (no reference tree)")
    rng = np.random.default_rng(31)
    g = gu.HostGraph.rmat(15, 16, seed=37)
    d = gu.HostGraph.dag(1 << 17, 1 << 20, seed=41)
    cases = [("metis", "graph", "dimacs", lambda p: M.write_metis(p, g.R, g.C, g.n, rng)),
             ("snap", "txt", "edgelist", lambda p: M.write_snap(p, d.R, d.C, d.n, rng, True)),
             ("market", "mtx", "market", lambda p: M.write_market(p, g.R, g.C, g.n, rng))]
    for name, ext, fmt, writer in cases:
        path = str(tmp_path / f"{name}.{ext}")
        writer(path)
        assert os.path.getsize(path) > (3 << 20), name  # several line ranges
        pre = str(tmp_path / f"ref_{name}")
        subprocess.run([M.REF_ORACLE, "parse", path, fmt, pre], check=True)
        R, C, n, directed = M.read_csr(pre)
        ours = gu.HostGraph.parse(path, fmt)
        assert ours.n == n, name
        np.testing.assert_array_equal(ours.R, R, err_msg=name)
        np.testing.assert_array_equal(ours.C, C[: R[n]], err_msg=name)
        if fmt != "market":
            assert ours.directed == directed, name

"""Host-side tests of the C ABI: symbols, status handling, generators.  No GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

import gu
import oracle
from conftest import ROOT


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:[\w\*\s]+?)\b(gu_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = gu.lib()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_status_strings():
    L = gu.lib()
    assert L.gu_version() >= 10000
    assert L.gu_status_string(0) == b"ok"
    assert L.gu_status_string(6) == b"device wait timed out"


def test_invalid_arguments_report_status():
    L = gu.lib()
    h = ctypes.c_void_p()
    st = L.gu_hgraph_er(1, 5, 1, ctypes.byref(h))
    assert st == 1
    assert b"n >= 2" in L.gu_last_error()
    assert L.gu_hgraph_rmat(0, 16, 0.57, 0.19, 0.19, 1, 1, ctypes.byref(h)) == 1
    assert L.gu_hgraph_rmat(10, 16, 0.7, 0.2, 0.2, 1, 1, ctypes.byref(h)) == 1
    out = np.zeros(4, np.int32)
    assert L.gu_sources(3, 4, 1, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))) == 1


def _csr_ok(g):
    assert g.R[0] == 0 and g.R[-1] == g.m
    assert np.all(np.diff(g.R) >= 0)
    for v in range(min(g.n, 2000)):
        adj = g.C[g.R[v]:g.R[v + 1]]
        assert np.all(np.diff(adj) > 0), "sorted, no duplicates"
        assert not np.any(adj == v), "no self loops"


def test_rmat_deterministic_and_symmetric():
    a = gu.HostGraph.rmat(12, 16, seed=3)
    b = gu.HostGraph.rmat(12, 16, seed=3)
    c = gu.HostGraph.rmat(12, 16, seed=4)
    np.testing.assert_array_equal(a.R, b.R)
    np.testing.assert_array_equal(a.C, b.C)
    assert not np.array_equal(a.C, c.C)
    assert a.n == 4096 and not a.directed
    _csr_ok(a)
    src = np.repeat(np.arange(a.n), np.diff(a.R))
    fwd = set(zip(src.tolist(), a.C.tolist()))
    assert all((v, u) in fwd for (u, v) in list(fwd)[:5000])
    # skewed degrees (R-MAT), 16*4096 draws minus duplicates
    deg = a.degrees()
    assert deg.max() > 20 * deg.mean()
    assert 0.5 * 2 * 16 * 4096 < a.m <= 2 * 16 * 4096


def test_er_exact_edge_count():
    g = gu.HostGraph.er(198, 2742, seed=1)
    assert g.n == 198 and g.m == 2 * 2742
    _csr_ok(g)


def test_grid_structure():
    g = gu.HostGraph.grid(40, 30, 0.0, seed=7)
    assert g.n == 1200 and g.m == 2 * (40 * 29 + 39 * 30)
    h = gu.HostGraph.grid(40, 30, 0.05, seed=7)
    removed = (g.m - h.m) // 2
    assert 0 < removed < 0.12 * g.m / 2
    assert h.degrees().max() <= 4
    _csr_ok(h)


def test_dag_is_acyclic():
    g = gu.HostGraph.dag(500, 4000, seed=3)
    assert g.directed
    _csr_ok(g)
    # Kahn's algorithm consumes every vertex
    indeg = np.bincount(g.C, minlength=g.n)
    stack = list(np.nonzero(indeg == 0)[0])
    seen = 0
    while stack:
        v = stack.pop()
        seen += 1
        for w in g.C[g.R[v]:g.R[v + 1]]:
            indeg[w] -= 1
            if indeg[w] == 0:
                stack.append(w)
    assert seen == g.n


def test_sources_distinct_deterministic():
    a = gu.sources(1000, 300, seed=2)
    b = gu.sources(1000, 300, seed=2)
    np.testing.assert_array_equal(a, b)
    assert len(set(a.tolist())) == 300 and a.min() >= 0 and a.max() < 1000


def test_from_edges_matches_oracle_semantics():
    u = np.array([0, 1, 2, 2, 3, 3, 0], np.int32)
    v = np.array([1, 2, 0, 2, 4, 4, 1], np.int32)
    g = gu.HostGraph.from_edges(6, u, v, symmetric=True)
    assert g.m == 2 * 4  # (0,1),(1,2),(2,0),(3,4); self loop and duplicates dropped
    d = oracle.bfs(g.R, g.C, g.n, 0)
    assert d.tolist() == [0, 1, 1, oracle.INF, oracle.INF, oracle.INF]


def test_drop_in_header_compiles_and_links(tmp_path):
    """include/graph_utils.hpp (the reference's signatures) compiles and links
    against the library with g++, as a reference caller would build it; the GPU
    tests run the resulting program."""
    import subprocess
    lib_dir = os.path.join(ROOT, "graph-utils_gb300", "lib")
    if not os.path.exists(os.path.join(lib_dir, "libgu_gb300.so")):
        pytest.skip("library not built")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "oracle"), "-I/usr/local/cuda/include",
           os.path.join(ROOT, "tests", "cpp", "shim_check.cpp"), "-x", "c", os.path.join(ROOT, "oracle", "gu_oracle.c"),
           "-x", "none", "-L" + lib_dir, "-lgu_gb300", "-L/usr/local/cuda/lib64", "-lcudart", "-lpthread",
           "-o", str(tmp_path / "shim_check")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_wait_limit_and_alloc_hook_arguments_on_the_host():
    """gu_set_wait_limit / gu_debug_fail_allocations validate their arguments
    without touching a GPU; gu_choose_device without one reports a CUDA status."""
    L = gu.lib()
    L.gu_set_wait_limit.argtypes = [ctypes.c_double]
    L.gu_get_wait_limit.argtypes = [ctypes.POINTER(ctypes.c_double)]
    L.gu_debug_fail_allocations.argtypes = [ctypes.c_int64, ctypes.c_int64]
    v = ctypes.c_double()
    assert L.gu_get_wait_limit(ctypes.byref(v)) == 0 and v.value == pytest.approx(4.0)
    for bad in (0.0, -1.0, 5e-5, 4000.0, float("nan")):
        assert L.gu_set_wait_limit(bad) == 1
    assert L.gu_get_wait_limit(ctypes.byref(v)) == 0 and v.value == pytest.approx(4.0)
    assert L.gu_set_wait_limit(0.25) == 0
    assert L.gu_get_wait_limit(ctypes.byref(v)) == 0 and v.value == pytest.approx(0.25)
    assert L.gu_set_wait_limit(4.0) == 0
    assert L.gu_get_wait_limit(None) == 1
    assert L.gu_debug_fail_allocations(-1, 1) == 1
    assert L.gu_debug_fail_allocations(0, -1) == 1
    assert L.gu_debug_fail_allocations(0, 0) == 0
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        chosen = ctypes.c_int(-7)
        assert L.gu_choose_device(-1, ctypes.byref(chosen)) == 2  # GU_ERR_CUDA, no exit()
        assert chosen.value == -7
        assert L.gu_last_error()


def test_ctypes_structs_match_the_c_header(tmp_path):
    """gu.py's ctypes mirrors of the C structs (gu_tuning, gu_search_item) have the
    header's size and field offsets, as gcc lays them out from include/gu.h."""
    import ctypes
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc absent")
    structs = {"gu_tuning": gu.GuTuning, "gu_search_item": gu.SearchItem}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "gu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c11", "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include",
                        str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)

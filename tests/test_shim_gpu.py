"""The C++ drop-in (include/graph_utils.hpp) driven like the reference's examples.

Compiles tests/cpp/shim_check.cpp (g++) against the library and the oracle and
runs it: every reference *_setup signature, the reference's result-row
convention, and the oracle as the checker.
"""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def shim_exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("shim") / "shim_check")
    lib_dir = os.path.join(ROOT, "graph-utils_gb300", "lib")
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "oracle"),
           "-I/usr/local/cuda/include", os.path.join(ROOT, "tests", "cpp", "shim_check.cpp"),
           "-x", "c", os.path.join(ROOT, "oracle", "gu_oracle.c"), "-x", "none",
           "-L" + lib_dir, "-lgu_gb300", "-L/usr/local/cuda/lib64", "-lcudart", "-lpthread",
           "-Wl,-rpath," + lib_dir, "-Wl,-rpath,/usr/local/cuda/lib64", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("args", [("10", "8", "0", "1024"),     # n < #SMs * 8: all sources, rows = #SMs
                                  ("12", "16", "17", "500"),    # offset start, end - start > #SMs
                                  ("9", "4", "3", "100")])      # end - start < #SMs
def test_reference_signatures(shim_exe, args):
    r = subprocess.run([shim_exe, *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASSED" in r.stdout

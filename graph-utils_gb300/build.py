"""Build recipe for graph-utils GB300: the CUDA/C++ library and the C oracle.

    python graph-utils_gb300/build.py            # library + oracle
    python graph-utils_gb300/build.py --lib      # library only

The library is compiled for sm_103a only (one -gencode), translation units in
parallel, and linked as graph-utils_gb300/lib/libgu_gb300.so (static CUDA
runtime).  The oracle (oracle/gu_oracle.c, test infrastructure) becomes
oracle/liboracle.so.  No cmake; a minute or less on 8+ cores.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "libgu_gb300.so")
ORACLE_SRC = os.path.join(ROOT, "oracle", "gu_oracle.c")
ORACLE_LIB = os.path.join(ROOT, "oracle", "liboracle.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")] + ARCH
CXXFLAGS = ["-std=c++17", "-O3", "-fPIC", "-Wall", "-I" + os.path.join(ROOT, "include"),
            "-I/usr/local/cuda/include"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose=False, ptxas_verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "gu.h"))
    jobs = []
    objs = []
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        if f.endswith(".cu"):
            obj = os.path.join(OBJ, f + ".o")
            flags = CUFLAGS + (["-Xptxas", "-v"] if ptxas_verbose else [])
            cmd = [NVCC] + flags + ["-c", src, "-o", obj]
        elif f.endswith(".cpp"):
            obj = os.path.join(OBJ, f + ".o")
            cmd = ["g++"] + CXXFLAGS + ["-c", src, "-o", obj]
        else:
            continue
        objs.append(obj)
        if ptxas_verbose or _stale(obj, [src] + headers):
            jobs.append(cmd)
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if jobs or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread", "-ldl"])
    if verbose:
        for lg in logs:
            if lg.strip():
                print(lg)
    return LIB


def build_oracle():
    if _stale(ORACLE_LIB, [ORACLE_SRC, ORACLE_SRC.replace(".c", ".h")]):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
              ORACLE_SRC, "-o", ORACLE_LIB])
    return ORACLE_LIB


if __name__ == "__main__":
    ptx = "--ptxas" in sys.argv
    build_library(verbose=True, ptxas_verbose=ptx)
    if "--lib" not in sys.argv:
        build_oracle()
    print("built", LIB)

"""ctypes binding of the CPU oracle (oracle/gu_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py, always as the checker or the
timed CPU baseline, never as the product path.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_ORACLE = os.path.join(HERE, "_ref", "ref_oracle")
INF = 2147483647

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} missing: build it with graph-utils_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_bfs.argtypes = [_i32p, _i32p, ctypes.c_int32, ctypes.c_int32, _i32p]
        L.oracle_sigma.argtypes = [_i32p, _i32p, ctypes.c_int32, ctypes.c_int32, _i32p, _u64p]
        L.oracle_brandes_f32.argtypes = [_i32p, _i32p, ctypes.c_int32, ctypes.c_int32, _i32p, _u64p, _f32p]
        L.oracle_brandes_f64.argtypes = [_i32p, _i32p, ctypes.c_int32, ctypes.c_int32, _i32p, _u64p, _f64p]
        L.oracle_brandes_pull_f64.argtypes = [_i32p, _i32p, ctypes.c_int32, ctypes.c_int32, _i32p, _u64p, _f64p]
        L.oracle_bc.argtypes = [_i32p, _i32p, ctypes.c_int32, _i32p, ctypes.c_int32, ctypes.c_int, _f64p,
                                ctypes.c_int]
        L.oracle_diameter.argtypes = [_i32p, _i32p, ctypes.c_int32, _i32p, ctypes.c_int32, ctypes.c_int]
        L.oracle_diameter.restype = ctypes.c_int32
        L.oracle_reach_count.argtypes = [_i32p, _i32p, ctypes.c_int32, _i32p, ctypes.c_int32, ctypes.c_int]
        L.oracle_reach_count.restype = ctypes.c_int64
        L.oracle_bfs_multi.argtypes = [_i32p, _i32p, ctypes.c_int32, _i32p, ctypes.c_int32, _i32p, ctypes.c_int64,
                                       ctypes.c_int]
        L.oracle_bfs_multi.restype = ctypes.c_int64
        L.oracle_sigma_multi.argtypes = [_i32p, _i32p, ctypes.c_int32, _i32p, ctypes.c_int32, _i32p, _u64p,
                                         ctypes.c_int64, ctypes.c_int]
        L.oracle_lbs.argtypes = [_i32p, ctypes.c_int32, _i32p, _i32p, ctypes.c_int64, _i64p]
        L.oracle_lbs.restype = ctypes.c_int
        L.oracle_race_and_resolve.argtypes = [ctypes.c_uint32, ctypes.c_int32]
        L.oracle_race_and_resolve.restype = ctypes.c_int32
        L.oracle_dag_reach_pairs.argtypes = [_i32p, _i32p, ctypes.c_int32]
        L.oracle_dag_reach_pairs.restype = ctypes.c_int64
        L.oracle_dag_reach_counts.argtypes = [_i32p, _i32p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64)]
        L.oracle_dag_reach_counts.restype = ctypes.c_int64
        L.oracle_rmat.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(_i32p), ctypes.POINTER(_i32p),
                                  ctypes.POINTER(ctypes.c_int64)]
        L.oracle_rmat.restype = ctypes.c_int
        L.oracle_sources.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, _i32p]
        L.oracle_sources.restype = ctypes.c_int
        L.oracle_free.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _p(a, t=_i32p):
    return a.ctypes.data_as(t)


def _csr(R, C):
    R = np.ascontiguousarray(R, dtype=np.int32)
    C = np.ascontiguousarray(C, dtype=np.int32)
    if C.size == 0:
        C = np.zeros(1, np.int32)
    return R, C


def bfs(R, C, n, source):
    R, C = _csr(R, C)
    d = np.empty(n, np.int32)
    lib().oracle_bfs(_p(R), _p(C), n, source, _p(d))
    return d


def bfs_multi(R, C, n, sources, nthreads=1):
    """Returns (dist[k, n], scanned CSR entries)."""
    R, C = _csr(R, C)
    s = np.ascontiguousarray(sources, dtype=np.int32)
    d = np.empty((len(s), n), np.int32)
    scanned = lib().oracle_bfs_multi(_p(R), _p(C), n, _p(s), len(s), _p(d), n, nthreads)
    return d, scanned


def sigma_multi(R, C, n, sources, nthreads=1):
    R, C = _csr(R, C)
    s = np.ascontiguousarray(sources, dtype=np.int32)
    d = np.empty((len(s), n), np.int32)
    sg = np.empty((len(s), n), np.uint64)
    lib().oracle_sigma_multi(_p(R), _p(C), n, _p(s), len(s), _p(d), _p(sg, _u64p), n, nthreads)
    return d, sg


def brandes(R, C, n, source, kind="f64"):
    """kind: 'f32' (bc.cu exactly), 'f64' (FP64 restatement), 'pull' (successor pull, FP64)."""
    R, C = _csr(R, C)
    d = np.empty(n, np.int32)
    sg = np.empty(n, np.uint64)
    if kind == "f32":
        de = np.empty(n, np.float32)
        lib().oracle_brandes_f32(_p(R), _p(C), n, source, _p(d), _p(sg, _u64p), _p(de, _f32p))
    else:
        de = np.empty(n, np.float64)
        fn = lib().oracle_brandes_f64 if kind == "f64" else lib().oracle_brandes_pull_f64
        fn(_p(R), _p(C), n, source, _p(d), _p(sg, _u64p), _p(de, _f64p))
    return d, sg, de


def bc(R, C, n, sources, pull=False, nthreads=1):
    R, C = _csr(R, C)
    s = np.ascontiguousarray(sources, dtype=np.int32)
    out = np.empty(n, np.float64)
    lib().oracle_bc(_p(R), _p(C), n, _p(s), len(s), int(pull), _p(out, _f64p), nthreads)
    return out


def diameter(R, C, n, sources, nthreads=1):
    R, C = _csr(R, C)
    s = np.ascontiguousarray(sources, dtype=np.int32)
    return int(lib().oracle_diameter(_p(R), _p(C), n, _p(s), len(s), nthreads))


def reach_count(R, C, n, sources, nthreads=1):
    R, C = _csr(R, C)
    s = np.ascontiguousarray(sources, dtype=np.int32)
    return int(lib().oracle_reach_count(_p(R), _p(C), n, _p(s), len(s), nthreads))


def lbs(counts, capacity=None):
    """Returns (scanned, result, total) or raises ValueError on overflow."""
    c = np.ascontiguousarray(counts, dtype=np.int32)
    N = len(c)
    tot = int(np.sum(c, dtype=np.int64))
    cap = tot if capacity is None else capacity
    scanned = np.empty(max(N, 1), np.int32)
    result = np.empty(max(cap, 1), np.int32)
    total = ctypes.c_int64()
    rc = lib().oracle_lbs(_p(c) if N else None, N, _p(scanned), _p(result), cap, ctypes.byref(total))
    if rc != 0:
        raise ValueError("LBS total exceeds capacity or INT32_MAX")
    return scanned[:N], result[: total.value], total.value


def race_and_resolve(vote, lane):
    return int(lib().oracle_race_and_resolve(vote, lane))


def dag_reach_pairs(R, C, n):
    R, C = _csr(R, C)
    return int(lib().oracle_dag_reach_pairs(_p(R), _p(C), n))


def dag_reach_counts(R, C, n):
    """Per-vertex reachable-set sizes (self excluded) of a DAG; returns (counts, total)."""
    R, C = _csr(R, C)
    out = np.zeros(max(n, 1), np.int64)
    tot = lib().oracle_dag_reach_counts(_p(R), _p(C), n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    return out[:n], int(tot)


def rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, permute=True):
    """The benchmark's R-MAT graph, built by the oracle's own restatement of the
    generator: (R, C) int32 numpy arrays of the symmetrised CSR."""
    R, C, m = _i32p(), _i32p(), ctypes.c_int64()
    rc = lib().oracle_rmat(scale, edge_factor, a, b, c, seed, int(permute), ctypes.byref(R), ctypes.byref(C),
                           ctypes.byref(m))
    if rc != 0:
        raise ValueError(f"oracle_rmat failed ({rc})")
    n = 1 << scale
    Rn = np.ctypeslib.as_array(R, shape=(n + 1,)).copy()
    Cn = np.ctypeslib.as_array(C, shape=(max(m.value, 1),))[: m.value].copy()
    lib().oracle_free(ctypes.cast(R, ctypes.c_void_p))
    lib().oracle_free(ctypes.cast(C, ctypes.c_void_p))
    return Rn, Cn


def sources(n, k, seed):
    """k distinct sources of [0, n), as the benchmark draws them."""
    out = np.empty(max(k, 1), np.int32)
    if lib().oracle_sources(n, k, seed, _p(out)) != 0:
        raise ValueError("need 0 <= k <= n")
    return out[:k]

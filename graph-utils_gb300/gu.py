"""ctypes binding of the graph-utils GB300 C ABI (include/gu.h).

Host-side mirror of the reference's entry points for Python callers (tests,
bench).  Device buffers are torch CUDA tensors (PyTorch is used for device
memory and streams only); host buffers are numpy arrays.  The compute path is
libgu_gb300.so; there is no fallback: loading fails loudly when the library is
missing.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libgu_gb300.so")

OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "capacity exceeded",
          5: "overflow", 6: "device wait timed out", 7: "unsupported", 8: "internal error", 9: "pending"}

BFS_AUTO, BFS_LINEAR, BFS_EDGE, BFS_WARP, BFS_CTA_WARP, BFS_SCAN, BFS_SHUFFLE, BFS_BOTTOM_UP, BFS_PLAIN = range(9)
VARIANTS = {"auto": BFS_AUTO, "linear": BFS_LINEAR, "edge": BFS_EDGE, "warp": BFS_WARP,
            "cta_warp": BFS_CTA_WARP, "scan": BFS_SCAN, "shuffle": BFS_SHUFFLE, "bottom_up": BFS_BOTTOM_UP,
            "plain": BFS_PLAIN}
UNREACHABLE = 2147483647

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p


class GuTuning(ctypes.Structure):
    """gu_tuning: AUTO's engine choice and its measured kernel time."""
    _fields_ = [("engine", ctypes.c_int32), ("alpha", ctypes.c_float), ("beta", ctypes.c_float),
                ("words", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("rare_frac", ctypes.c_float),
                ("seconds", ctypes.c_double)]


ENGINES = {0: "batched", 1: "per-source", 2: "one-cta"}
RARE_FRAC = 0.15  # the batched engine's default rare-source fraction (gu_tuning.rare_frac)


def _tuning_dict(t):
    return {"engine": ENGINES[t.engine], "alpha": float(t.alpha), "beta": float(t.beta), "words": int(t.words),
            "ctas_per_sm": int(t.ctas_per_sm), "rare_frac": float(t.rare_frac), "seconds": float(t.seconds)}


class GuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def lib():
    """Load libgu_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
    L = ctypes.CDLL(LIB_PATH)
    sig = {
        "gu_version": ([], ctypes.c_int),
        "gu_last_error": ([], ctypes.c_char_p),
        "gu_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "gu_choose_device": ([ctypes.c_int, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "gu_timer_start": ([_vp, ctypes.POINTER(_vp)], ctypes.c_int),
        "gu_timer_stop": ([_vp, _vp, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "gu_hgraph_rmat": ([ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                            ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(_vp)], ctypes.c_int),
        "gu_hgraph_er": ([ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(_vp)], ctypes.c_int),
        "gu_hgraph_grid": ([ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_uint64, ctypes.POINTER(_vp)],
                           ctypes.c_int),
        "gu_hgraph_dag": ([ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(_vp)], ctypes.c_int),
        "gu_hgraph_from_edges": ([ctypes.c_int32, _i32p, _i32p, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(_vp)],
                                 ctypes.c_int),
        "gu_hgraph_arrays": ([_vp, ctypes.POINTER(_i32p), ctypes.POINTER(_i32p), _i32p, _i64p,
                              ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "gu_hgraph_destroy": ([_vp], ctypes.c_int),
        "gu_hgraph_from_csr": ([_i32p, _i32p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(_vp)],
                               ctypes.c_int),
        "gu_hgraph_parse": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_vp)], ctypes.c_int),
        "gu_hgraph_write_csr": ([_vp, ctypes.c_char_p], ctypes.c_int),
        "gu_hgraph_write_edgelist": ([_vp, ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
        "gu_hgraph_count_degree_zero": ([_vp, ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
        "gu_sources": ([ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, _i32p], ctypes.c_int),
        "gu_graph_create": ([_i32p, _i32p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int, _vp, ctypes.POINTER(_vp)],
                            ctypes.c_int),
        "gu_graph_destroy": ([_vp], ctypes.c_int),
        "gu_graph_info": ([_vp, _i32p, _i64p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_size_t)],
                          ctypes.c_int),
        "gu_graph_arrays": ([_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                             ctypes.POINTER(_vp)], ctypes.c_int),
        "gu_graph_last_launch": ([_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "gu_graph_launch_times": ([_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)],
                                  ctypes.c_int),
        "gu_graph_level_idle": ([_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "gu_graph_autotune": ([_vp, _vp, ctypes.c_int32, ctypes.POINTER(GuTuning), ctypes.POINTER(GuTuning),
                               ctypes.c_int, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "gu_graph_set_tuning": ([_vp, ctypes.POINTER(GuTuning)], ctypes.c_int),
        "gu_graph_level_profile": ([_vp, ctypes.c_int, _i32p, _i32p, _i32p, _i64p, _i64p,
                                    ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "gu_bfs": ([_vp, ctypes.c_int, _vp, ctypes.c_int32, _vp, ctypes.c_int64, _vp], ctypes.c_int),
        "gu_bfs_host": ([_vp, ctypes.c_int, _i32p, ctypes.c_int32, _i32p, ctypes.c_int64, _vp], ctypes.c_int),
        "gu_sigma": ([_vp, _vp, ctypes.c_int32, _vp, _vp, ctypes.c_int64, _vp], ctypes.c_int),
        "gu_bc": ([_vp, _vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp, ctypes.c_int64, _vp], ctypes.c_int),
        "gu_diameter": ([_vp, _vp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), _vp], ctypes.c_int),
        "gu_reach": ([_vp, _vp, ctypes.c_int32, _vp, _vp], ctypes.c_int),
        "gu_dag_reach": ([_vp, _vp, _i64p, _vp], ctypes.c_int),
        "gu_power_start": ([ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)], ctypes.c_int),
        "gu_power_stop": ([_vp, ctypes.POINTER(ctypes.c_double), _i64p], ctypes.c_int),
        "gu_lbs": ([_vp, ctypes.c_int32, _vp, _vp, ctypes.c_int64, _vp, _i64p, _vp], ctypes.c_int),
        "gu_lbs_last_ms": ([ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "gu_race_and_resolve": ([_vp, ctypes.c_int32, _vp, _vp], ctypes.c_int),
        "gu_server_create": ([ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)], ctypes.c_int),
        "gu_server_destroy": ([_vp], ctypes.c_int),
        "gu_server_submit": ([_vp, _vp, ctypes.c_int, _i32p, ctypes.c_int32, _vp, _i64p], ctypes.c_int),
        "gu_server_wait": ([_vp, ctypes.c_int64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "gu_server_stats": ([_vp, _i64p, _i64p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
        "gu_bfs_many": ([_vp, ctypes.c_int32, _vp], ctypes.c_int),
        "gu_bfs_noalloc": ([_vp, _vp, ctypes.c_int32, ctypes.c_int64, _vp, ctypes.c_int32, _vp, ctypes.c_int64, _vp],
                           ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def check(status):
    if status != OK:
        raise GuError(status, lib().gu_last_error().decode())


def _ptr(a):
    return a.ctypes.data_as(_i32p)


class HostGraph:
    """Host CSR (R, C as int32 numpy arrays), from a generator or arrays."""

    def __init__(self, R, C, n, directed=False):
        self.R = np.ascontiguousarray(R, dtype=np.int32)
        self.C = np.ascontiguousarray(C, dtype=np.int32)
        self.n = int(n)
        self.m = int(self.C.shape[0])
        self.directed = bool(directed)

    @staticmethod
    def _from_handle(h):
        L = lib()
        R, C = _i32p(), _i32p()
        n, m, d = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int()
        check(L.gu_hgraph_arrays(h, ctypes.byref(R), ctypes.byref(C), ctypes.byref(n), ctypes.byref(m),
                                 ctypes.byref(d)))
        Rn = np.ctypeslib.as_array(R, shape=(n.value + 1,)).copy()
        Cn = np.ctypeslib.as_array(C, shape=(max(m.value, 1),))[: m.value].copy() if m.value else \
            np.zeros(0, np.int32)
        L.gu_hgraph_destroy(h)
        return HostGraph(Rn, Cn, n.value, bool(d.value))

    @staticmethod
    def rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, permute=True):
        h = _vp()
        check(lib().gu_hgraph_rmat(scale, edge_factor, a, b, c, seed, int(permute), ctypes.byref(h)))
        return HostGraph._from_handle(h)

    @staticmethod
    def er(n, m, seed=1):
        h = _vp()
        check(lib().gu_hgraph_er(n, m, seed, ctypes.byref(h)))
        return HostGraph._from_handle(h)

    @staticmethod
    def grid(rows, cols, p_delete=0.05, seed=7):
        h = _vp()
        check(lib().gu_hgraph_grid(rows, cols, p_delete, seed, ctypes.byref(h)))
        return HostGraph._from_handle(h)

    @staticmethod
    def dag(n, m, seed=1):
        h = _vp()
        check(lib().gu_hgraph_dag(n, m, seed, ctypes.byref(h)))
        return HostGraph._from_handle(h)

    @staticmethod
    def from_edges(n, u, v, symmetric=True):
        u = np.ascontiguousarray(u, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.int32)
        h = _vp()
        check(lib().gu_hgraph_from_edges(n, _ptr(u), _ptr(v), len(u), int(symmetric), ctypes.byref(h)))
        return HostGraph._from_handle(h)

    def degrees(self):
        return np.diff(self.R)

    @staticmethod
    def parse(path, fmt):
        """Read a graph file: "dimacs"/"metis", "edgelist", "edgelist_h", "market" or "csrbin"."""
        h = _vp()
        check(lib().gu_hgraph_parse(os.fsencode(path), fmt.encode(), ctypes.byref(h)))
        return HostGraph._from_handle(h)

    def _handle(self):
        h = _vp()
        check(lib().gu_hgraph_from_csr(_ptr(self.R), _ptr(self.C) if self.m else None, self.n, self.m,
                                       int(self.directed), ctypes.byref(h)))
        return h

    def _with_handle(self, fn):
        h = self._handle()
        try:
            return fn(h)
        finally:
            lib().gu_hgraph_destroy(h)

    def write_csr(self, path):
        """Binary CSR cache (read back with parse(path, "csrbin"))."""
        self._with_handle(lambda h: check(lib().gu_hgraph_write_csr(h, os.fsencode(path))))

    def write_edgelist(self, path, header=False):
        """The reference's write_edgelist_to_file: optional "n m" line, "u v" per CSR entry."""
        self._with_handle(lambda h: check(lib().gu_hgraph_write_edgelist(h, os.fsencode(path), int(header))))

    def count_degree_zero(self):
        c = ctypes.c_uint64()
        self._with_handle(lambda h: check(lib().gu_hgraph_count_degree_zero(h, ctypes.byref(c))))
        return c.value


def sources(n, k, seed=2):
    out = np.zeros(k, dtype=np.int32)
    check(lib().gu_sources(n, k, seed, _ptr(out)))
    return out


def _stream_handle(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


class Graph:
    """Device-resident graph (the reference's device_graph)."""

    def __init__(self, hg, stream=None):
        self.host = hg
        self.n, self.m, self.directed = hg.n, hg.m, hg.directed
        self._h = _vp()
        check(lib().gu_graph_create(_ptr(hg.R), _ptr(hg.C) if hg.m else None, hg.n, hg.m, int(hg.directed),
                                    _stream_handle(stream), ctypes.byref(self._h)))

    def close(self):
        if self._h:
            lib().gu_graph_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_bytes(self):
        b = ctypes.c_size_t()
        check(lib().gu_graph_info(self._h, None, None, None, ctypes.byref(b)))
        return b.value

    def launch_times(self, max_entries=64):
        """Kernel seconds of the graph's last launches (up to 64), oldest first."""
        out = np.zeros(max_entries, np.float64)
        cnt = ctypes.c_int()
        check(lib().gu_graph_launch_times(self._h, max_entries, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                          ctypes.byref(cnt)))
        return [float(x) for x in out[: cnt.value]]

    def autotune(self, sources_dev, max_trials=32):
        """Times AUTO's candidate engines and settings on a sample of sources and makes the
        fastest this graph's AUTO choice.  Returns (best, trials) as dicts."""
        best = GuTuning()
        trials = (GuTuning * max_trials)()
        nt = ctypes.c_int()
        check(lib().gu_graph_autotune(self._h, sources_dev.data_ptr(), int(sources_dev.numel()), ctypes.byref(best),
                                      trials, max_trials, ctypes.byref(nt)))
        return _tuning_dict(best), [_tuning_dict(trials[i]) for i in range(nt.value)]

    def set_tuning(self, tuning):
        """Sets AUTO's choice explicitly (a dict as autotune returns; None: the built-in choice)."""
        if tuning is None:
            check(lib().gu_graph_set_tuning(self._h, None))
            return
        eng = {v: k for k, v in ENGINES.items()}[tuning["engine"]]
        t = GuTuning(eng, float(tuning.get("alpha", 2.0)), float(tuning.get("beta", 24.0)), int(tuning.get("words", 0)),
                     int(tuning.get("ctas_per_sm", 0)), float(tuning.get("rare_frac", RARE_FRAC)), 0.0)
        check(lib().gu_graph_set_tuning(self._h, ctypes.byref(t)))

    def last_launch(self):
        """(kernel seconds, top-down levels, bottom-up levels, max level) of the last launch."""
        t = ctypes.c_double()
        td, bu, ml = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib().gu_graph_last_launch(self._h, ctypes.byref(t), ctypes.byref(td), ctypes.byref(bu),
                                         ctypes.byref(ml)))
        return t.value, td.value, bu.value, ml.value

    def level_profile(self, max_entries=1024):
        """Per-phase timeline of the last batched search or BC / sigma pass: list of dicts."""
        b, lv, kd = (np.zeros(max_entries, np.int32) for _ in range(3))
        fv, fe = np.zeros(max_entries, np.int64), np.zeros(max_entries, np.int64)
        t = np.zeros(max_entries, np.float64)
        cnt = ctypes.c_int()
        check(lib().gu_graph_level_profile(self._h, max_entries, _ptr(b), _ptr(lv), _ptr(kd),
                                           fv.ctypes.data_as(_i64p), fe.ctypes.data_as(_i64p),
                                           t.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(cnt)))
        kinds = {0: "top-down", 1: "bottom-up", 2: "rows", 4: "init", 5: "bu-final", 6: "bu-light", 7: "bu-scan",
                 8: "bc-forward", 9: "bc-backward", 10: "bc-combine", 11: "bc-finish", 12: "bc-clear"}
        return [dict(batch=int(b[i]), level=int(lv[i]), kind=kinds.get(int(kd[i]), "?"),
                     frontier_vertices=int(fv[i]), frontier_edges=int(fe[i]), t_ms=float(t[i]))
                for i in range(cnt.value)]

    def level_idle(self, max_entries=1024):
        """(idle CTA-ms per timeline entry, CTAs of the launch) of the last batched search."""
        out = np.zeros(max_entries, np.float64)
        nb, cnt = ctypes.c_int(), ctypes.c_int()
        check(lib().gu_graph_level_idle(self._h, max_entries, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                        ctypes.byref(nb), ctypes.byref(cnt)))
        return out[:cnt.value].copy(), nb.value

    def bfs(self, sources_dev, dist_dev, variant="auto", ld=None, stream=None):
        """Device form: sources_dev (int32 cuda tensor, k), dist_dev (int32 cuda tensor, k x ld)."""
        k = int(sources_dev.numel())
        ld = self.n if ld is None else ld
        check(lib().gu_bfs(self._h, VARIANTS[variant] if isinstance(variant, str) else variant,
                           sources_dev.data_ptr(), k, dist_dev.data_ptr(), ld, _stream_handle(stream)))
        return dist_dev

    def sigma(self, sources_dev, sigma_dev, dist_dev=None, ld=None, stream=None):
        """Shortest-path counts (uint64 rows, int64 tensor view) and optional distances."""
        ld = self.n if ld is None else ld
        check(lib().gu_sigma(self._h, sources_dev.data_ptr(), int(sources_dev.numel()),
                             dist_dev.data_ptr() if dist_dev is not None else None, sigma_dev.data_ptr(), ld,
                             _stream_handle(stream)))
        return sigma_dev

    def bc(self, sources_dev, bc_dev, delta_dev=None, batch=0, ld=None, stream=None):
        """Betweenness (float64 tensor of n) from the given sources; optional delta rows."""
        ld = self.n if ld is None else ld
        check(lib().gu_bc(self._h, sources_dev.data_ptr(), int(sources_dev.numel()), batch, bc_dev.data_ptr(),
                          delta_dev.data_ptr() if delta_dev is not None else None, ld, _stream_handle(stream)))
        return bc_dev

    def diameter(self, sources_dev, stream=None):
        d = ctypes.c_int32()
        check(lib().gu_diameter(self._h, sources_dev.data_ptr(), int(sources_dev.numel()), ctypes.byref(d),
                                _stream_handle(stream)))
        return d.value

    def reach(self, sources_dev, counts_dev, stream=None):
        """counts_dev (int64 cuda tensor, k): vertices reachable from each source, itself included."""
        check(lib().gu_reach(self._h, sources_dev.data_ptr(), int(sources_dev.numel()), counts_dev.data_ptr(),
                             _stream_handle(stream)))

    def dag_reach(self, counts_dev, stream=None):
        """counts_dev (int64 cuda tensor, n): reachable-set size of every vertex of the DAG
        (itself excluded); returns the total number of reachable pairs."""
        tot = ctypes.c_int64()
        check(lib().gu_dag_reach(self._h, counts_dev.data_ptr(), ctypes.byref(tot), _stream_handle(stream)))
        return tot.value

    def bfs_host(self, sources_host, variant="auto", out=None, stream=None):
        """Host form: numpy sources in, numpy k x n int32 distances out."""
        s = np.ascontiguousarray(sources_host, dtype=np.int32)
        k = len(s)
        if out is None:
            out = np.empty((k, self.n), dtype=np.int32)
        check(lib().gu_bfs_host(self._h, VARIANTS[variant] if isinstance(variant, str) else variant, _ptr(s), k,
                                out.ctypes.data_as(_i32p), out.shape[1], _stream_handle(stream)))
        return out


class SearchItem(ctypes.Structure):
    """gu_search_item: one request of gu_bfs_many."""
    _fields_ = [("graph", _vp), ("sources_dev", _vp), ("k", ctypes.c_int32), ("dist_dev", _vp),
                ("ld", ctypes.c_int64), ("reach_dev", _vp)]


def bfs_many(requests, stream=None):
    """Many searches on many graphs in one work-queue launch.  requests: list of
    (Graph, sources int32 cuda tensor, dist int32 cuda tensor k x ld or None,
    reach int64 cuda tensor k or None)."""
    arr = (SearchItem * max(1, len(requests)))()
    for i, (g, s, d, r) in enumerate(requests):
        arr[i] = SearchItem(g._h, s.data_ptr(), int(s.numel()), d.data_ptr() if d is not None else None,
                            int(d.shape[1]) if d is not None else 0, r.data_ptr() if r is not None else None)
    check(lib().gu_bfs_many(arr, len(requests), _stream_handle(stream)))


def lbs(counts_dev, scanned_dev, result_dev, total_dev=None, stream=None):
    """Load-balanced search on device tensors; returns the total (int)."""
    tot = ctypes.c_int64()
    check(lib().gu_lbs(counts_dev.data_ptr(), int(counts_dev.numel()), scanned_dev.data_ptr(),
                       result_dev.data_ptr() if result_dev.numel() else None, int(result_dev.numel()),
                       total_dev.data_ptr() if total_dev is not None else None, ctypes.byref(tot),
                       _stream_handle(stream)))
    return tot.value


def lbs_last_ms():
    """Device time of the last lbs call on the current device (ms)."""
    ms = ctypes.c_double()
    check(lib().gu_lbs_last_ms(ctypes.byref(ms)))
    return ms.value


def race_and_resolve(pred_dev, winners_dev, stream=None):
    """Winner lane per group of 32 predicates (device tensors, int32)."""
    check(lib().gu_race_and_resolve(pred_dev.data_ptr(), int(pred_dev.numel()) // 32, winners_dev.data_ptr(),
                                    _stream_handle(stream)))
    return winners_dev


class PowerSampler:
    """Mean board power over a region (gu_power_*): `with PowerSampler(0) as p: ...; p.watts`."""

    def __init__(self, device=0, period_ms=10):
        self.device, self.period_ms = device, period_ms
        self.watts, self.samples = None, 0
        self._h = None

    def __enter__(self):
        h = _vp()
        check(lib().gu_power_start(self.device, self.period_ms, ctypes.byref(h)))
        self._h = h
        return self

    def __exit__(self, *exc):
        w, n = ctypes.c_double(), ctypes.c_int64()
        h, self._h = self._h, None
        check(lib().gu_power_stop(h, ctypes.byref(w), ctypes.byref(n)))
        self.watts, self.samples = w.value, n.value
        return False


QUERY_BFS, QUERY_BC, QUERY_REACH = 0, 1, 2
PENDING = 9


class Server:
    """Continuous-batching query server (gu_server_*)."""

    def __init__(self, hbm_budget_bytes=8 << 30, slots=4, max_batch=256):
        self._h = _vp()
        check(lib().gu_server_create(hbm_budget_bytes, slots, max_batch, ctypes.byref(self._h)))
        self._keep = {}

    def submit(self, graph, query, sources, out):
        """Queue a request; `out` (numpy) receives the result when it is waited for."""
        s = np.ascontiguousarray(sources, dtype=np.int32)
        rid = ctypes.c_int64()
        check(lib().gu_server_submit(self._h, graph._h, query, _ptr(s), len(s), out.ctypes.data_as(_vp),
                                     ctypes.byref(rid)))
        self._keep[rid.value] = (s, out)
        return rid.value

    def wait(self, rid, timeout=-1.0):
        lat = ctypes.c_double()
        st = lib().gu_server_wait(self._h, rid, timeout, ctypes.byref(lat))
        if st == PENDING:
            return None
        self._keep.pop(rid, None)
        check(st)
        return lat.value

    def stats(self):
        c, b = ctypes.c_int64(), ctypes.c_int64()
        p50, p99, mb = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().gu_server_stats(self._h, ctypes.byref(c), ctypes.byref(b), ctypes.byref(p50), ctypes.byref(p99),
                                    ctypes.byref(mb)))
        return dict(completed=c.value, batches=b.value, p50_s=p50.value, p99_s=p99.value,
                    mean_requests_per_batch=mb.value)

    def close(self):
        if self._h:
            lib().gu_server_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

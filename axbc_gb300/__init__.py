"""axbc_gb300: GB300-native sampled-Brandes betweenness centrality.

Python binding of the C ABI in ``include/axbc.h`` (``libaxbc_gb300.so``, built
in-tree by ``axbc_gb300.build``).  Every call goes to the CUDA library; there is
no CPU fallback: if the library is missing or no GPU is present the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libaxbc_gb300.so")
MAX_BATCH = 64
_LIB = None


class AxbcError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"axbc status {status}: {msg}")
        self.status = status


class PivotStats(C.Structure):
    _fields_ = [("nvisited", C.c_uint64), ("all", C.c_uint64), ("te", C.c_uint64),
                ("levels", C.c_int32), ("pad", C.c_int32)]

    def as_dict(self):
        return dict(nvisited=self.nvisited, all=self.all, te=self.te, levels=self.levels)


class RunParams(C.Structure):
    _fields_ = [("z", C.c_int32), ("bader_c", C.c_int32), ("nbfs", C.c_uint64),
                ("nchecks", C.c_uint32), ("H", C.c_int32), ("seed", C.c_int64),
                ("batch_width", C.c_int32), ("pad", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [("push_factor_single", C.c_double), ("push_factor_batch", C.c_double),
                ("batch_width", C.c_int32), ("pad", C.c_int32), ("batch_te_per_s", C.c_double),
                ("plain_te_per_s", C.c_double)]


class RunResult(C.Structure):
    _fields_ = [("nrounds", C.c_uint64), ("skipped", C.c_uint64), ("dropped", C.c_uint64),
                ("rounds", C.c_uint64), ("te", C.c_uint64), ("stopped", C.c_int32),
                ("batches", C.c_int32)]


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("result", RunResult),
                ("bytes", C.c_uint64), ("submit_ns", C.c_uint64), ("start_ns", C.c_uint64),
                ("finish_ns", C.c_uint64), ("error", C.c_char * 256)]


class ServerStats(C.Structure):
    _fields_ = [("budget", C.c_uint64), ("in_use", C.c_uint64), ("queued", C.c_uint64),
                ("admitted", C.c_uint64), ("completed", C.c_uint64), ("passes", C.c_uint64),
                ("lanes", C.c_uint64)]


REQ_STATES = ["queued", "running", "done", "failed"]


# name -> (restype, argtypes) of every entry point this binding uses
_P = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_SIGS = {
    "axbc_status_str": (C.c_char_p, [C.c_int]),
    "axbc_last_error": (C.c_char_p, []),
    "axbc_version": (C.c_char_p, []),
    "axbc_edges_to_csc": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_int, C.c_int,
                                    C.POINTER(_P), C.POINTER(_P), C.POINTER(C.c_uint64),
                                    C.POINTER(_P), C.POINTER(C.c_uint64)]),
    "axbc_host_free": (None, [_P]),
    "axbc_read_edge_file": (C.c_int, [C.c_char_p, C.c_uint64, C.POINTER(_P),
                                      C.POINTER(C.c_uint64)]),
    "axbc_graph_create": (C.c_int, [_P, _P, C.c_uint64, C.c_uint64, _P, C.POINTER(_P)]),
    "axbc_graph_generate_rmat": (C.c_int, [C.c_int, C.c_int, C.c_uint64, C.c_int, C.c_int,
                                           C.POINTER(_P)]),
    "axbc_graph_generate_grid": (C.c_int, [C.c_uint32, C.c_double, C.c_double, C.c_uint64,
                                           C.POINTER(_P)]),
    "axbc_graph_from_edges": (C.c_int, [_P, C.c_uint64, C.c_uint64, C.c_int, C.c_int,
                                        C.POINTER(_P)]),
    "axbc_kron_edges": (C.c_int, [C.c_int, C.c_int, C.c_uint64, C.c_uint64, _P, C.c_int, _P]),
    "axbc_graph_generate_kronecker": (C.c_int, [C.c_int, C.c_int, C.c_uint64, C.c_uint64, _P,
                                                C.c_int, C.POINTER(_P)]),
    "axbc_graph_destroy": (C.c_int, [_P]),
    "axbc_graph_info": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                  C.POINTER(C.c_uint64), C.POINTER(C.c_int)]),
    "axbc_graph_get_deg": (C.c_int, [_P, _P]),
    "axbc_graph_get_csc": (C.c_int, [_P, _P, _P, _P]),
    "axbc_graph_degree2": (C.c_int, [_P, _P]),
    "axbc_graph_sum_deg_neigh": (C.c_int, [_P, _P]),
    "axbc_graph_lcc": (C.c_int, [_P, _P]),
    "axbc_ctx_create": (C.c_int, [_P, _P, C.POINTER(_P)]),
    "axbc_ctx_destroy": (C.c_int, [_P]),
    "axbc_ctx_reset": (C.c_int, [_P]),
    "axbc_ctx_bytes": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "axbc_ctx_set_tuning": (C.c_int, [_P, C.c_double, C.c_double]),
    "axbc_run_pivot": (C.c_int, [_P, C.c_uint32, C.c_double, C.c_int, C.POINTER(PivotStats)]),
    "axbc_run_batch": (C.c_int, [_P, _P, _P, C.c_int, C.c_int, _P]),
    "axbc_run_sampled": (C.c_int, [_P, C.POINTER(RunParams), C.POINTER(RunResult)]),
    "axbc_get_pivots": (C.c_int, [_P, _P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "axbc_get_checks": (C.c_int, [_P, _P, C.c_uint32]),
    "axbc_get_bc": (C.c_int, [_P, _P]),
    "axbc_get_delta": (C.c_int, [_P, _P]),
    "axbc_get_sigma": (C.c_int, [_P, _P]),
    "axbc_get_levels": (C.c_int, [_P, _P]),
    "axbc_get_batch_source": (C.c_int, [_P, C.c_int, _P, _P, _P]),
    "axbc_bc_device_ptr": (C.c_int, [_P, C.POINTER(_P)]),
    "axbc_ctx_sync": (C.c_int, [_P]),
    "axbc_ctx_profile": (C.c_int, [_P, C.c_int]),
    "axbc_ctx_profile_read": (C.c_int, [_P, _P, _P, _P, C.c_int]),
    "axbc_ctx_launches": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "axbc_ctx_count": (C.c_int, [_P, C.c_int]),
    "axbc_ctx_set_persistent": (C.c_int, [_P, C.c_int, C.c_int]),
    "axbc_selftest_grid_barrier": (C.c_int, [C.c_int, C.c_int, C.c_longlong, C.c_int, C.POINTER(C.c_int),
                                             C.POINTER(C.c_uint32), C.POINTER(C.c_float)]),
    "axbc_ctx_count_read": (C.c_int, [_P, _P, C.c_int]),
    "axbc_autotune": (C.c_int, [_P, _P, C.c_int, C.c_int, C.POINTER(Tuning)]),
    "axbc_bc_pivot_static": (C.c_int, [_P, _P, _P, C.c_uint64, C.c_uint64, C.c_uint32,
                                       C.c_double, C.c_int, _P, _P, C.POINTER(PivotStats)]),
    "axbc_selftest_division": (C.c_int, [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64),
                                         C.POINTER(C.c_uint64)]),
    "axbc_ctx_level_stats": (C.c_int, [_P, _P, _P, _P, _P, _P, C.c_int, C.POINTER(C.c_int)]),
    "axbc_ctx_profile_records": (C.c_int, [_P, _P, _P, _P, _P, C.c_uint64, C.POINTER(C.c_uint64)]),
    "axbc_srand48": (C.c_uint64, [C.c_int64]),
    "axbc_inject_alloc_failures": (None, [C.c_int]),
    "axbc_inject_alloc_failure_after": (None, [C.c_int]),
    "axbc_device_bytes_live": (C.c_uint64, []),
    "axbc_sample": (C.c_int, [_P, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.c_int,
                              C.POINTER(C.c_uint32), C.POINTER(C.c_double)]),
    "axbc_bader_check": (C.c_int, [_P, _P, C.c_uint32, C.c_uint32, C.POINTER(C.c_int)]),
    "axbc_server_create": (C.c_int, [C.c_uint64, C.POINTER(_P)]),
    "axbc_server_add_graph": (C.c_int, [_P, _P, C.c_int, C.POINTER(C.c_int)]),
    "axbc_request_submit": (C.c_int, [_P, C.c_int, C.POINTER(RunParams), C.POINTER(C.c_uint64)]),
    "axbc_request_poll": (C.c_int, [_P, C.c_uint64, C.POINTER(RequestInfo)]),
    "axbc_request_wait": (C.c_int, [_P, C.c_uint64, C.c_int64, C.POINTER(RequestInfo)]),
    "axbc_request_result": (C.c_int, [_P, C.c_uint64, _P, _P, _P, C.c_uint64,
                                      C.POINTER(C.c_uint64)]),
    "axbc_request_release": (C.c_int, [_P, C.c_uint64]),
    "axbc_server_stats": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "axbc_server_destroy": (C.c_int, [_P]),
    "axbc_server_graph_stats": (C.c_int, [_P, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                          C.POINTER(C.c_uint64)]),
}

PROF_KINDS = ["batch_fwd_push", "batch_fwd_pull", "batch_level_stats", "batch_bwd",
              "batch_bwd_combine", "batch_update", "sampler", "plain_fwd", "plain_bwd",
              "plain_other", "batch_persistent"]
# work counters per kind (axbc_ctx_count_read)
WORK_FIELDS = ["bytes", "entries", "gathers", "pairs"]
# kernel names behind each profiling kind (for matching ncu launch lists)
PROF_KERNELS = {"batch_fwd_push": "k_fwd_push_step", "batch_fwd_pull": "k_fwd_pull_step",
                "batch_level_stats": "k_stats_step", "batch_bwd": "k_bwd_step",
                "batch_bwd_combine": "k_bwd_combine_step", "batch_update": "k_update_m",
                "sampler": "k_sampler", "plain_fwd": "k_fwd_push1", "plain_bwd": "k_bwd1",
                "plain_other": "k_update1", "batch_persistent": "k_traverse_persist"}


def lib():
    """Load libaxbc_gb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise AxbcError(-1, f"{LIB_PATH} is missing: run `python -m axbc_gb300.build` "
                                "(the CUDA library is required; there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _check(rc):
    if rc != 0:
        raise AxbcError(rc, lib().axbc_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def version() -> str:
    return lib().axbc_version().decode()


def edges_to_csc(edges, n, undirected=True, H=0):
    """Reference graph pipeline on the host: returns (col, row, reach, removed)."""
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.uint64).reshape(-1, 2))
    col, row, reach = _P(), _P(), _P()
    m, rem = C.c_uint64(), C.c_uint64()
    L = lib()
    _check(L.axbc_edges_to_csc(_ptr(e), len(e), n, int(undirected), H, C.byref(col),
                               C.byref(row), C.byref(m), C.byref(reach), C.byref(rem)))
    try:
        colv = np.ctypeslib.as_array(C.cast(col, _U32P), (n + 1,)).copy()
        rowv = (np.ctypeslib.as_array(C.cast(row, _U32P), (m.value,)).copy()
                if m.value else np.zeros(0, np.uint32))
        reachv = np.ctypeslib.as_array(C.cast(reach, _U32P), (n,)).copy()
    finally:
        for p in (col, row, reach):
            L.axbc_host_free(p)
    return colv, rowv, reachv, rem.value


def read_edge_file(path, n):
    out, ne = _P(), C.c_uint64()
    L = lib()
    _check(L.axbc_read_edge_file(path.encode(), n, C.byref(out), C.byref(ne)))
    try:
        if ne.value == 0:
            return np.zeros((0, 2), np.uint64)
        arr = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_uint64)), (2 * ne.value,)).copy()
    finally:
        L.axbc_host_free(out)
    return arr.reshape(-1, 2)


def kron_edges(scale, edgefactor=16, seed1=23, seed2=24, stage=2, initiator=None):
    """The Graph500 generator's edge list, generated on the device, as int64
    (source, target) pairs: stage 2 = make_graph's output, 1 = before the edge
    scramble, 0 = before the vertex permutation."""
    out = np.empty(2 * (1 << scale) * edgefactor, np.int64)
    ini = None if initiator is None else (C.c_double * 4)(*initiator)
    _check(lib().axbc_kron_edges(scale, edgefactor, seed1, seed2,
                                 C.cast(ini, _P) if ini is not None else None, stage, _ptr(out)))
    return out.reshape(-1, 2)


class Graph:
    """A graph resident on the current CUDA device (reference CSC layout)."""

    def __init__(self, handle):
        self._h = handle
        n, m, b, sym = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_int()
        _check(lib().axbc_graph_info(handle, C.byref(n), C.byref(m), C.byref(b), C.byref(sym)))
        self.n, self.m, self.bytes, self.symmetric = n.value, m.value, b.value, bool(sym.value)

    @classmethod
    def from_csc(cls, col, row, reach=None):
        col = np.ascontiguousarray(col, dtype=np.uint32)
        row = np.ascontiguousarray(row, dtype=np.uint32)
        rch = None if reach is None else np.ascontiguousarray(reach, dtype=np.uint32)
        h = _P()
        _check(lib().axbc_graph_create(_ptr(col), _ptr(row), len(col) - 1, len(row), _ptr(rch),
                                       C.byref(h)))
        return cls(h)

    @classmethod
    def rmat(cls, scale, edgefactor=16, seed=23, directed=False, H=0):
        h = _P()
        _check(lib().axbc_graph_generate_rmat(scale, edgefactor, seed, int(directed), H,
                                              C.byref(h)))
        return cls(h)

    @classmethod
    def from_edges(cls, edges, n, undirected=True, H=0):
        """Device ingest of an edge list (mirror, norm_graph, one-degree
        reduction, build_csc; src/axbc2d.c:333-351, 695-907)."""
        e = np.ascontiguousarray(np.asarray(edges, np.uint64).reshape(-1, 2))
        h = _P()
        _check(lib().axbc_graph_from_edges(_ptr(e) if len(e) else None, len(e), n, int(undirected), H,
                                           C.byref(h)))
        return cls(h)

    @classmethod
    def kronecker(cls, scale, edgefactor=16, seed1=23, seed2=24, H=0, initiator=None):
        """The reference's synthetic graph: the Graph500 generator's edges
        (gen_graph, src/axbc2d.c:518-527), generated and built on the device."""
        h = _P()
        ini = None if initiator is None else (C.c_double * 4)(*initiator)
        _check(lib().axbc_graph_generate_kronecker(scale, edgefactor, seed1, seed2,
                                                   C.cast(ini, _P) if ini is not None else None,
                                                   H, C.byref(h)))
        return cls(h)

    @classmethod
    def grid(cls, side, drop_prob=0.02, longrange_frac=1e-4, seed=7):
        h = _P()
        _check(lib().axbc_graph_generate_grid(side, drop_prob, longrange_frac, seed, C.byref(h)))
        return cls(h)

    def csc(self):
        col = np.empty(self.n + 1, np.uint32)
        row = np.empty(max(self.m, 1), np.uint32)
        reach = np.empty(self.n, np.uint32)
        _check(lib().axbc_graph_get_csc(self._h, _ptr(col), _ptr(row), _ptr(reach)))
        return col, row[:self.m], reach

    def deg(self):
        out = np.empty(self.n, np.uint32)
        _check(lib().axbc_graph_get_deg(self._h, _ptr(out)))
        return out

    def degree2(self):
        out = np.empty(self.n, np.uint32)
        _check(lib().axbc_graph_degree2(self._h, _ptr(out)))
        return out

    def sum_deg_neigh(self):
        out = np.empty(self.n, np.uint32)
        _check(lib().axbc_graph_sum_deg_neigh(self._h, _ptr(out)))
        return out

    def lcc(self):
        out = np.empty(self.n, np.float32)
        _check(lib().axbc_graph_lcc(self._h, _ptr(out)))
        return out

    def close(self):
        if self._h:
            lib().axbc_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """BC state for one graph: bc, per-pivot state, batch state, sampler."""

    def __init__(self, graph: Graph, stream=None):
        self.graph = graph
        h = _P()
        _check(lib().axbc_ctx_create(graph._h, stream, C.byref(h)))
        self._h = h
        self.n = graph.n

    @property
    def bytes(self):
        b = C.c_uint64()
        _check(lib().axbc_ctx_bytes(self._h, C.byref(b)))
        return b.value

    def set_tuning(self, push_factor_single=1.0, push_factor_batch=1.0):
        _check(lib().axbc_ctx_set_tuning(self._h, push_factor_single, push_factor_batch))

    def reset(self):
        _check(lib().axbc_ctx_reset(self._h))

    def run_pivot(self, v0, p, H=0):
        st = PivotStats()
        _check(lib().axbc_run_pivot(self._h, int(v0), float(p), H, C.byref(st)))
        return st.as_dict()

    def run_batch(self, v0s, ps, H=0, stats=True):
        v = np.ascontiguousarray(v0s, dtype=np.uint32)
        p = np.ascontiguousarray(ps, dtype=np.float64)
        k = len(v)
        st = (PivotStats * k)() if stats else None
        _check(lib().axbc_run_batch(self._h, _ptr(v), _ptr(p), k, H,
                                    C.cast(st, _P) if stats else None))
        return [s.as_dict() for s in st] if stats else None

    def run_sampled(self, z=0, nbfs=1, bader_c=1, nchecks=1, H=0, seed=4343543, W=1):
        prm = RunParams(z, bader_c, nbfs, nchecks, H, seed, W, 0)
        res = RunResult()
        _check(lib().axbc_run_sampled(self._h, C.byref(prm), C.byref(res)))
        cnt = C.c_uint64()
        _check(lib().axbc_get_pivots(self._h, None, None, 0, C.byref(cnt)))
        piv = np.zeros(cnt.value, np.uint32)
        pr = np.zeros(cnt.value, np.float64)
        _check(lib().axbc_get_pivots(self._h, _ptr(piv), _ptr(pr), cnt.value, C.byref(cnt)))
        chk = np.zeros(max(nchecks, 1), np.uint32)
        _check(lib().axbc_get_checks(self._h, _ptr(chk), nchecks))
        return dict(nrounds=res.nrounds, skipped=res.skipped, dropped=res.dropped,
                    ui_end=res.rounds, te=res.te, stopped=bool(res.stopped),
                    batches=res.batches, pivots=piv, probs=pr, checks=chk[:nchecks])

    def bc(self):
        out = np.empty(self.n, np.float32)
        _check(lib().axbc_get_bc(self._h, _ptr(out)))
        return out

    def delta(self):
        out = np.empty(self.n, np.float32)
        _check(lib().axbc_get_delta(self._h, _ptr(out)))
        return out

    def sigma(self):
        out = np.empty(self.n, np.uint32)
        _check(lib().axbc_get_sigma(self._h, _ptr(out)))
        return out

    def levels(self):
        out = np.empty(self.n, np.int32)
        _check(lib().axbc_get_levels(self._h, _ptr(out)))
        return out

    def batch_source(self, s):
        sig = np.empty(self.n, np.uint32)
        lvl = np.empty(self.n, np.int32)
        dl = np.empty(self.n, np.float32)
        _check(lib().axbc_get_batch_source(self._h, s, _ptr(sig), _ptr(lvl), _ptr(dl)))
        return sig, lvl, dl

    def bc_device_ptr(self) -> int:
        p = _P()
        _check(lib().axbc_bc_device_ptr(self._h, C.byref(p)))
        return p.value

    def sync(self):
        _check(lib().axbc_ctx_sync(self._h))

    def autotune(self, pivots, H=0):
        """Pick direction-switch factors and batch width on these pivots (bc is kept)."""
        v = np.ascontiguousarray(pivots, dtype=np.uint32)
        t = Tuning()
        _check(lib().axbc_autotune(self._h, _ptr(v), len(v), H, C.byref(t)))
        return dict(push_factor_single=t.push_factor_single,
                    push_factor_batch=t.push_factor_batch, batch_width=t.batch_width,
                    batch_te_per_s=t.batch_te_per_s, plain_te_per_s=t.plain_te_per_s)

    def level_stats(self, max_levels=1 << 16):
        """Per forward level of the last batch: dict of arrays count, te, push,
        list_count, list_cap (list_count > list_cap: the level was scanned)."""
        lv = C.c_int()
        _check(lib().axbc_ctx_level_stats(self._h, None, None, None, None, None, 0, C.byref(lv)))
        L = min(lv.value, max_levels)
        out = dict(count=np.zeros(L, np.uint64), te=np.zeros(L, np.uint64), push=np.zeros(L, np.int32),
                   list_count=np.zeros(L, np.uint32), list_cap=np.zeros(L, np.uint32))
        _check(lib().axbc_ctx_level_stats(self._h, _ptr(out["count"]), _ptr(out["te"]), _ptr(out["push"]),
                                          _ptr(out["list_count"]), _ptr(out["list_cap"]), L,
                                          C.byref(lv)))
        return out

    def sample(self, z, rng, mix=0, first=False):
        """One draw of heuristic z from this context's bc / last delta:
        (v0, p, rng', mix') -- rng is a drand48 state (see srand48)."""
        r, m = C.c_uint64(rng), C.c_uint32(mix)
        v, p = C.c_uint32(), C.c_double()
        _check(lib().axbc_sample(self._h, z, C.byref(r), C.byref(m), int(first), C.byref(v),
                                 C.byref(p)))
        return v.value, p.value, r.value, m.value

    def bader_check(self, checks, c):
        """True if every check vertex v has bc[v] / 2 >= c * n."""
        ch = np.ascontiguousarray(checks, dtype=np.uint32)
        out = C.c_int()
        _check(lib().axbc_bader_check(self._h, _ptr(ch), len(ch), c, C.byref(out)))
        return bool(out.value)

    def profile(self, enable=True):
        """Record CUDA events around every kernel launch of this context."""
        _check(lib().axbc_ctx_profile(self._h, int(enable)))

    def profile_records(self):
        """The timed launches since profile() / the last profile_read(), in order:
        list of (kind, forward level or -1, ms, model bytes)."""
        cnt = C.c_uint64()
        _check(lib().axbc_ctx_profile_records(self._h, None, None, None, None, 0, C.byref(cnt)))
        k = cnt.value
        kinds = np.zeros(k, np.int32)
        tags = np.zeros(k, np.int32)
        ms = np.zeros(k, np.float32)
        by = np.zeros(k, np.float64)
        _check(lib().axbc_ctx_profile_records(self._h, _ptr(kinds), _ptr(tags), _ptr(ms), _ptr(by), k,
                                              C.byref(cnt)))
        return [(PROF_KINDS[a], int(b), float(c), float(d)) for a, b, c, d in zip(kinds, tags, ms, by)]

    def profile_read(self):
        """{kind: (ms, launches, algorithmic bytes)} since profile() / the last read."""
        k = len(PROF_KINDS)
        ms = np.zeros(k, np.float64)
        cnt = np.zeros(k, np.uint64)
        by = np.zeros(k, np.float64)
        _check(lib().axbc_ctx_profile_read(self._h, _ptr(ms), _ptr(cnt), _ptr(by), k))
        return {PROF_KINDS[i]: (float(ms[i]), int(cnt[i]), float(by[i])) for i in range(k)}

    def set_persistent(self, mode=0, blocks_per_sm=0):
        """Batched passes as one persistent launch: 1 always, -1 never, 0 auto."""
        _check(lib().axbc_ctx_set_persistent(self._h, int(mode), int(blocks_per_sm)))

    def count(self, enable=True):
        """Run the counting builds of the traversal kernels (measurement only)."""
        _check(lib().axbc_ctx_count(self._h, int(enable)))

    def count_read(self):
        """{kind: {bytes, entries, gathers, pairs}} since count() / the last read:
        the bytes each kind of launch must move at least and the work behind them."""
        k = len(PROF_KINDS)
        out = np.zeros(k * WORK_FIELDS.__len__(), np.uint64)
        _check(lib().axbc_ctx_count_read(self._h, _ptr(out), k))
        out = out.reshape(k, len(WORK_FIELDS))
        return {PROF_KINDS[i]: {f: int(out[i, j]) for j, f in enumerate(WORK_FIELDS)}
                for i in range(k) if out[i].any()}

    @property
    def launches(self):
        v = C.c_uint64()
        _check(lib().axbc_ctx_launches(self._h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "_h", None):
            lib().axbc_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def srand48(seed):
    """The drand48 state that srand48(seed) sets."""
    return lib().axbc_srand48(seed)


class Server:
    """Request server over resident graphs (axbc_server_* / axbc_request_*).

    Requests are sampled runs (run_sampled's parameters, W <= 64); the server
    batches the rounds of concurrent requests on one graph into shared passes.
    """

    def __init__(self, hbm_budget=0):
        h = _P()
        _check(lib().axbc_server_create(int(hbm_budget), C.byref(h)))
        self._h = h
        self._graphs = []

    def add_graph(self, graph, H=0):
        gid = C.c_int()
        _check(lib().axbc_server_add_graph(self._h, graph._h, H, C.byref(gid)))
        self._graphs.append(graph)  # keeps the graph alive as long as the server
        return gid.value

    def submit(self, graph_id, z=0, nbfs=1, bader_c=0, nchecks=1, H=0, seed=4343543, W=1):
        prm = RunParams(z, bader_c, nbfs, nchecks, H, seed, W, 0)
        rid = C.c_uint64()
        _check(lib().axbc_request_submit(self._h, graph_id, C.byref(prm), C.byref(rid)))
        return rid.value

    @staticmethod
    def _info(i):
        r = i.result
        return dict(state=REQ_STATES[i.state], status=i.status, bytes=i.bytes,
                    submit_ns=i.submit_ns, start_ns=i.start_ns, finish_ns=i.finish_ns,
                    error=i.error.decode(), nrounds=r.nrounds, skipped=r.skipped,
                    dropped=r.dropped, ui_end=r.rounds, te=r.te, stopped=bool(r.stopped),
                    batches=r.batches)

    def poll(self, rid):
        i = RequestInfo()
        _check(lib().axbc_request_poll(self._h, rid, C.byref(i)))
        return self._info(i)

    def wait(self, rid, timeout_ms=-1):
        i = RequestInfo()
        _check(lib().axbc_request_wait(self._h, rid, int(timeout_ms), C.byref(i)))
        return self._info(i)

    def result(self, rid, n):
        """(bc, pivots, probs) of a done request on an n-vertex graph."""
        cnt = C.c_uint64()
        _check(lib().axbc_request_result(self._h, rid, None, None, None, 0, C.byref(cnt)))
        bc = np.zeros(n, np.float32)
        piv = np.zeros(cnt.value, np.uint32)
        pr = np.zeros(cnt.value, np.float64)
        _check(lib().axbc_request_result(self._h, rid, _ptr(bc), _ptr(piv), _ptr(pr), cnt.value,
                                         C.byref(cnt)))
        return bc, piv, pr

    def release(self, rid):
        _check(lib().axbc_request_release(self._h, rid))

    def stats(self):
        st = ServerStats()
        _check(lib().axbc_server_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def graph_stats(self, graph_id):
        p, l, b = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(lib().axbc_server_graph_stats(self._h, graph_id, C.byref(p), C.byref(l), C.byref(b)))
        return dict(passes=p.value, lanes=l.value, busy_s=b.value / 1e9)

    def close(self):
        if getattr(self, "_h", None):
            lib().axbc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def selftest_grid_barrier(blocks_per_sm=2, rounds=1000, budget_cycles=1 << 33, absent_block=-1):
    """(failed barrier site or 0, barriers completed, ms) of the persistent loop's grid barrier."""
    site, leads, ms = C.c_int(), C.c_uint32(), C.c_float()
    _check(lib().axbc_selftest_grid_barrier(blocks_per_sm, rounds, budget_cycles, absent_block,
                                            C.byref(site), C.byref(leads), C.byref(ms)))
    return site.value, leads.value, ms.value


def selftest_division(n=1 << 26, seed=1):
    """(mismatches, exact-path count) of the update's division fast path."""
    bad, slow = C.c_uint64(), C.c_uint64()
    _check(lib().axbc_selftest_division(n, seed, C.byref(bad), C.byref(slow)))
    return bad.value, slow.value


def exported_symbols():
    """Names declared in include/*.h (read from the headers next to the package)."""
    import re
    names = []
    inc = os.path.join(os.path.dirname(_HERE), "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", txt)
    skip = {"if", "for", "while", "return", "sizeof", "defined"}
    return sorted({n for n in names if n not in skip and not n.isupper()})

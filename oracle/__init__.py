"""CPU oracle for the AxBC sampled-Brandes path -- test infrastructure only.

ctypes wrapper around ``oracle/liboracle.so`` (a plain-C restatement of the
reference's single-GPU path, see ``oracle/oracle.c``) and, when it was built,
``oracle/_ref/libkron_ref.so`` (the reference's own Graph500 generator compiled
from its sources).  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg import this package; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None


class Graph(C.Structure):
    _fields_ = [
        ("n", C.c_uint64),
        ("m", C.c_uint64),
        ("col", C.c_void_p),
        ("row", C.c_void_p),
        ("reach", C.c_void_p),
    ]


class PivotStats(C.Structure):
    _fields_ = [
        ("nvisited", C.c_uint64),
        ("all", C.c_uint64),
        ("te", C.c_uint64),
        ("levels", C.c_int32),
        ("pad", C.c_int32),
    ]


class RunParams(C.Structure):
    _fields_ = [
        ("z", C.c_int32),
        ("bader_c", C.c_int32),
        ("nbfs", C.c_uint64),
        ("nchecks", C.c_uint32),
        ("H", C.c_int32),
        ("seed", C.c_int64),
        ("W", C.c_int32),
        ("order", C.c_int32),
    ]


class RunResult(C.Structure):
    _fields_ = [
        ("nrounds", C.c_uint64),
        ("skipped", C.c_uint64),
        ("dropped", C.c_uint64),
        ("ui_end", C.c_uint64),
        ("te", C.c_uint64),
        ("stopped", C.c_int32),
        ("pad", C.c_int32),
    ]


def reference_dir():
    """The reference's source tree, when present on this machine: the
    AXBC_REFERENCE_DIR environment variable, else a `reference` directory
    beside the repository.  None where it does not exist (the GPU machine)."""
    d = os.environ.get("AXBC_REFERENCE_DIR") or os.path.join(_HERE, "..", "..", "reference")
    d = os.path.abspath(d)
    return d if os.path.isdir(os.path.join(d, "generator")) else None


def build(force: bool = False, ref: bool = False) -> None:
    """Compile liboracle.so (and the reference generator shim if asked)."""
    target = os.path.join(_HERE, "liboracle.so")
    newest = max(os.path.getmtime(os.path.join(_HERE, f)) for f in ("oracle.c", "oracle.h", "kron.c"))
    if force or not os.path.exists(target) or os.path.getmtime(target) < newest:
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    rd = reference_dir() if ref else None
    if rd:
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={rd}"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        build()
        L = C.CDLL(os.path.join(_HERE, "liboracle.so"))
        P = C.c_void_p
        L.orc_pipeline.argtypes = [P, C.c_uint64, C.c_uint64, C.c_int, C.c_int,
                                   C.POINTER(P), C.POINTER(P), C.POINTER(C.c_uint64),
                                   C.POINTER(P), C.POINTER(C.c_uint64)]
        L.orc_free.argtypes = [P]
        L.orc_bc_pivot.argtypes = [C.POINTER(Graph), C.c_uint32, C.c_double, C.c_int, C.c_int,
                                   P, P, P, P, C.POINTER(PivotStats)]
        L.orc_bc_pivots.argtypes = [C.POINTER(Graph), P, P, C.c_uint64, C.c_int, C.c_int, P, P,
                                    C.POINTER(C.c_uint64)]
        L.orc_bc_pivots_omp.argtypes = [C.POINTER(Graph), P, P, C.c_uint64, C.c_int, C.c_int, P,
                                        C.POINTER(C.c_uint64)]
        L.orc_degree2.argtypes = [C.POINTER(Graph), P]
        L.orc_sum_deg_neigh.argtypes = [C.POINTER(Graph), P]
        L.orc_lcc.argtypes = [C.POINTER(Graph), P]
        L.orc_hprefix.argtypes = [P, C.c_uint64, P, P]
        L.orc_hsearch.argtypes = [P, P, C.c_uint64, C.c_double, C.POINTER(C.c_int)]
        L.orc_hsearch.restype = C.c_uint64
        L.orc_lrand48_seq.argtypes = [C.c_int64, C.c_int64, P]
        L.orc_run.argtypes = [C.POINTER(Graph), C.POINTER(RunParams), P, P, P, P, C.c_uint64, P,
                              C.POINTER(RunResult)]
        L.orc_kron_edges.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_uint64, P, C.c_int, P]
        L.orc_kron_edges.restype = C.c_int64
        L.orc_kron_perm_key.argtypes = [C.c_uint64] * 5
        L.orc_kron_perm_key.restype = C.c_uint64
        _LIB = L
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class CSC:
    """A graph in the reference's CSC layout (col offsets, row ids, reach)."""

    def __init__(self, col, row, reach=None, rem_ed=0):
        self.col = np.ascontiguousarray(col, dtype=np.uint32)
        self.row = np.ascontiguousarray(row, dtype=np.uint32)
        self.n = len(self.col) - 1
        self.m = len(self.row)
        self.reach = (np.zeros(self.n, np.uint32) if reach is None
                      else np.ascontiguousarray(reach, dtype=np.uint32))
        self.rem_ed = rem_ed
        self._g = Graph(self.n, self.m, _ptr(self.col), _ptr(self.row), _ptr(self.reach))

    @property
    def deg(self):
        return np.diff(self.col.astype(np.int64)).astype(np.uint32)

    def graph(self):
        return C.byref(self._g)


def pipeline(edges, n, undirected=True, H=0) -> CSC:
    """mirror -> norm_graph -> [degree_reduction] -> norm_graph -> build_csc."""
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.uint64).reshape(-1, 2))
    L = lib()
    col, row, reach = C.c_void_p(), C.c_void_p(), C.c_void_p()
    m, rem = C.c_uint64(), C.c_uint64()
    rc = L.orc_pipeline(_ptr(e), len(e), n, int(undirected), H, C.byref(col), C.byref(row),
                        C.byref(m), C.byref(reach), C.byref(rem))
    if rc:
        raise ValueError(f"oracle pipeline failed ({rc})")
    colv = np.ctypeslib.as_array(C.cast(col, C.POINTER(C.c_uint32)), (n + 1,)).copy()
    rowv = (np.ctypeslib.as_array(C.cast(row, C.POINTER(C.c_uint32)), (m.value,)).copy()
            if m.value else np.zeros(0, np.uint32))
    reachv = (np.ctypeslib.as_array(C.cast(reach, C.POINTER(C.c_uint32)), (n,)).copy()
              if n else np.zeros(0, np.uint32))
    for p in (col, row, reach):
        L.orc_free(p)
    return CSC(colv, rowv, reachv, rem.value)


def bc_pivot(g: CSC, v0, p, H=0, order=0, bc=None):
    """One pivot; returns (bc, lvl, sigma, delta, stats dict)."""
    n = g.n
    bc = np.zeros(n, np.float32) if bc is None else bc
    lvl = np.empty(n, np.int32)
    sigma = np.empty(n, np.uint32)
    delta = np.empty(n, np.float32)
    st = PivotStats()
    rc = lib().orc_bc_pivot(g.graph(), v0, p, H, order, _ptr(bc), _ptr(lvl), _ptr(sigma),
                            _ptr(delta), C.byref(st))
    if rc:
        raise ValueError("bad pivot")
    return bc, lvl, sigma, delta, dict(nvisited=st.nvisited, all=st.all, te=st.te,
                                       levels=st.levels)


def bc_pivots(g: CSC, pivots, probs, H=0, order=0):
    piv = np.ascontiguousarray(pivots, dtype=np.uint32)
    pr = np.ascontiguousarray(probs, dtype=np.float64)
    bc = np.zeros(g.n, np.float32)
    dl = np.zeros(g.n, np.float32)
    te = C.c_uint64()
    rc = lib().orc_bc_pivots(g.graph(), _ptr(piv), _ptr(pr), len(piv), H, order, _ptr(bc),
                             _ptr(dl), C.byref(te))
    if rc:
        raise ValueError("bad pivot list")
    return bc, dl, te.value


def bc_pivots_omp(g: CSC, pivots, probs, H=0, threads=0):
    piv = np.ascontiguousarray(pivots, dtype=np.uint32)
    pr = np.ascontiguousarray(probs, dtype=np.float64)
    bc = np.zeros(g.n, np.float32)
    te = C.c_uint64()
    rc = lib().orc_bc_pivots_omp(g.graph(), _ptr(piv), _ptr(pr), len(piv), H, threads, _ptr(bc),
                                 C.byref(te))
    if rc:
        raise ValueError("bad pivot list")
    return bc, te.value


def degree2(g: CSC):
    out = np.empty(g.n, np.uint32)
    lib().orc_degree2(g.graph(), _ptr(out))
    return out


def sum_deg_neigh(g: CSC):
    out = np.empty(g.n, np.uint32)
    lib().orc_sum_deg_neigh(g.graph(), _ptr(out))
    return out


def lcc(g: CSC):
    out = np.empty(g.n, np.float32)
    lib().orc_lcc(g.graph(), _ptr(out))
    return out


def hprefix(w):
    w = np.ascontiguousarray(w, dtype=np.float32)
    n = len(w)
    local = np.empty(n, np.float64)
    csum = np.empty((n + 1023) // 1024, np.float64)
    lib().orc_hprefix(_ptr(w), n, _ptr(local), _ptr(csum))
    return local, csum


def hsearch(local, csum, r):
    f = C.c_int()
    i = lib().orc_hsearch(_ptr(local), _ptr(csum), len(local), r, C.byref(f))
    return int(i), bool(f.value)


def lrand48_seq(seed, count):
    out = np.empty(count, np.int64)
    lib().orc_lrand48_seq(seed, count, _ptr(out))
    return out


def run(g: CSC, z=0, nbfs=1, bader_c=1, nchecks=1, H=0, seed=4343543, W=1, order=0):
    """The reference's sampling loop; returns dict with bc, pivots, probs, ..."""
    n = g.n
    prm = RunParams(z, bader_c, nbfs, nchecks, H, seed, W, order)
    bc = np.zeros(n, np.float32)
    dl = np.zeros(n, np.float32)
    cap = min(nbfs, n) + 1
    piv = np.zeros(cap, np.uint32)
    pr = np.zeros(cap, np.float64)
    chk = np.zeros(max(nchecks, 1), np.uint32)
    res = RunResult()
    lib().orc_run(g.graph(), C.byref(prm), _ptr(bc), _ptr(dl), _ptr(piv), _ptr(pr), cap,
                  _ptr(chk), C.byref(res))
    k = res.nrounds
    return dict(bc=bc, delta_last=dl, pivots=piv[:k].copy(), probs=pr[:k].copy(),
                checks=chk[:nchecks].copy(), nrounds=res.nrounds, skipped=res.skipped,
                dropped=res.dropped, ui_end=res.ui_end, te=res.te, stopped=bool(res.stopped))


GRAPH500_INITIATOR = (.57, .19, .19, .05)


def kron_edges(scale, edgef, seed1=23, seed2=24, stage=2, initiator=GRAPH500_INITIATOR):
    """The Graph500 generator restated in oracle/kron.c, as int64 (src, tgt)
    pairs.  stage 0: before the vertex permutation; 1: permuted, (min, max)
    pairs; 2: scrambled (the reference make_graph's output order)."""
    L = lib()
    ne = (1 << scale) * edgef
    out = np.empty(2 * ne, np.int64)
    ini = (C.c_double * 4)(*initiator)
    got = L.orc_kron_edges(scale, edgef, seed1, seed2, ini, stage, _ptr(out))
    if got < 0:
        raise MemoryError("orc_kron_edges")
    return out.reshape(-1, 2)


def kron_perm_key(seed1, seed2, skip_hi, i, T):
    return int(lib().orc_kron_perm_key(seed1, seed2, skip_hi, i, T))


def ref_kron_available() -> bool:
    return os.path.exists(os.path.join(_HERE, "_ref", "libkron_ref.so"))


def ref_kron_edges(scale, edgef, seed1=23, seed2=24, initiator=GRAPH500_INITIATOR):
    """Edges from the reference's own generator (oracle/_ref), as int64 pairs."""
    global _REF
    if _REF is None:
        _REF = C.CDLL(os.path.join(_HERE, "_ref", "libkron_ref.so"))
        _REF.ref_kron_edges_ini.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_uint64,
                                            C.c_void_p, C.POINTER(C.c_void_p)]
        _REF.ref_kron_edges_ini.restype = C.c_int64
        _REF.ref_kron_free.argtypes = [C.c_void_p]
    out = C.c_void_p()
    ini = (C.c_double * 4)(*initiator)
    ned = _REF.ref_kron_edges_ini(scale, edgef, seed1, seed2, C.cast(ini, C.c_void_p), C.byref(out))
    arr = np.ctypeslib.as_array(C.cast(out, C.POINTER(C.c_int64)), (2 * ned,)).copy()
    _REF.ref_kron_free(out)
    return arr.reshape(-1, 2)

"""ctypes wrapper of the CPU oracle (``gtc_oracle.c``).

TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA library and the
timed CPU baseline in ``bench.py``.  Nothing in the product imports this
module.  The C file restates graph-tool-rs's centrality power iteration
(crates/gt-algo/src/centrality.rs:141-497) and its adjacency storage
(crates/gt-core/src/adj/{block,list,alloc}.rs); its header lists the exact
lines each function follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libgtc_oracle.so")
_lib = None

_u8p = C.POINTER(C.c_uint8)
_u32p = C.POINTER(C.c_uint32)
_u64p = C.POINTER(C.c_uint64)
_f64p = C.POINTER(C.c_double)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    src = os.path.join(_HERE, "gtc_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "libgtc_oracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.ora_graph_new.restype = C.c_void_p
        L.ora_graph_new.argtypes = [C.c_uint64]
        L.ora_graph_free.argtypes = [C.c_void_p]
        L.ora_add_edge.restype = C.c_int64
        L.ora_add_edge.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64]
        L.ora_remove_edge.restype = C.c_int
        L.ora_remove_edge.argtypes = [C.c_void_p, C.c_uint64]
        L.ora_add_edges.restype = C.c_int
        L.ora_add_edges.argtypes = [C.c_void_p, C.c_uint64, _u32p, _u32p]
        for f in ("ora_num_vertices", "ora_edge_bound", "ora_num_edges"):
            getattr(L, f).restype = C.c_uint64
            getattr(L, f).argtypes = [C.c_void_p]
        L.ora_export.argtypes = [C.c_void_p, _u64p, _u32p, _u32p, _u64p, _u32p, _u32p]
        L.ora_pagerank.restype = C.c_int64
        L.ora_pagerank.argtypes = [C.c_void_p, C.c_int, _u8p, _u8p, _f64p, _f64p, C.c_double,
                                   C.c_double, C.c_uint64, C.c_uint64, C.c_uint64, _f64p,
                                   C.c_uint64, C.c_int]
        L.ora_eigenvector.restype = C.c_int64
        L.ora_eigenvector.argtypes = [C.c_void_p, C.c_int, _u8p, _u8p, _f64p, C.c_double,
                                      C.c_uint64, C.c_uint64, C.c_uint64, _f64p, C.c_uint64,
                                      C.c_int, _f64p]
        L.ora_betweenness.restype = C.c_int
        L.ora_betweenness.argtypes = [C.c_void_p, C.c_int, C.c_int, _u8p, _u8p, _f64p, _f64p,
                                      C.c_int]
        L.ora_last_error.restype = C.c_char_p
        L.ora_max_threads.restype = C.c_int
        L.ora_plan_range.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, _u64p, _u64p]
        _lib = L
    return _lib


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


def plan_chunks(n: int, grain: int) -> int:
    """Plan::new(n, grain).chunks() (crates/gt-core/src/par/plan.rs:55-61)."""
    if grain <= 0:
        raise ValueError("Plan::new: grain must be non-zero")
    return max(-(-n // grain), 1)


class OracleError(RuntimeError):
    pass


class Graph:
    """The reference's AdjList, restated: edges added in call order."""

    def __init__(self, n: int, edges=None):
        self._h = lib().ora_graph_new(n)
        if not self._h:
            raise MemoryError("ora_graph_new")
        self.n = n
        if edges is not None:
            self.add_edges(edges)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.ora_graph_free(h)
            self._h = None

    def add_edge(self, s: int, t: int) -> int:
        r = lib().ora_add_edge(self._h, s, t)
        if r < 0:
            raise OracleError(lib().ora_last_error().decode())
        return r

    def remove_edge(self, e: int) -> None:
        if lib().ora_remove_edge(self._h, e) != 0:
            raise OracleError(lib().ora_last_error().decode())

    def add_edges(self, edges) -> None:
        e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
        src = np.ascontiguousarray(e[:, 0], dtype=np.uint32)
        tgt = np.ascontiguousarray(e[:, 1], dtype=np.uint32)
        self.add_edge_arrays(src, tgt)

    def add_edge_arrays(self, src: np.ndarray, tgt: np.ndarray) -> None:
        src = np.ascontiguousarray(src, dtype=np.uint32)
        tgt = np.ascontiguousarray(tgt, dtype=np.uint32)
        if src.size and (int(src.max()) >= self.n or int(tgt.max()) >= self.n):
            raise OracleError("add_edge: no such vertex")
        if lib().ora_add_edges(self._h, src.size, _ptr(src, _u32p), _ptr(tgt, _u32p)) != 0:
            raise OracleError(lib().ora_last_error().decode())

    def num_edges(self) -> int:
        return lib().ora_num_edges(self._h)

    def edge_bound(self) -> int:
        return lib().ora_edge_bound(self._h)

    def export(self):
        """(out_off, out_other, out_idx, in_off, in_other, in_idx): every
        block's out-half and in-half in storage order."""
        n, m = self.n, self.num_edges()
        oo = np.zeros(n + 1, np.uint64)
        io = np.zeros(n + 1, np.uint64)
        ot = np.zeros(max(m, 1), np.uint32)
        oi = np.zeros(max(m, 1), np.uint32)
        it = np.zeros(max(m, 1), np.uint32)
        ii = np.zeros(max(m, 1), np.uint32)
        lib().ora_export(self._h, _ptr(oo, _u64p), _ptr(ot, _u32p), _ptr(oi, _u32p),
                         _ptr(io, _u64p), _ptr(it, _u32p), _ptr(ii, _u32p))
        return oo, ot[:m], oi[:m], io, it[:m], ii[:m]

    def pagerank(self, weight=None, pers=None, damping=0.85, epsilon=1e-6, max_iter=0,
                 grain=4096, rank=None, had=None, reversed=False, vmask=None, emask=None,
                 threads=1, plan_len=None, plan_chunks_=None):
        """pagerank / pagerank_with (centrality.rs:234-384).  Returns
        (rank f64[n], iterations).  ``rank``/``had`` give a warm start."""
        n = self.n
        out = np.zeros(n, np.float64)
        if rank is not None:
            r = np.asarray(rank, np.float64)
            k = min(r.size, n)
            out[:k] = r[:k]
            had = k if had is None else had
        else:
            had = 0 if had is None else had
        w = None if weight is None else np.ascontiguousarray(weight, np.float64)
        p = None if pers is None else np.ascontiguousarray(pers, np.float64)
        vm = None if vmask is None else np.ascontiguousarray(vmask, np.uint8)
        em = None if emask is None else np.ascontiguousarray(emask, np.uint8)
        pl = n if plan_len is None else plan_len
        ch = plan_chunks(pl, grain) if plan_chunks_ is None else plan_chunks_
        it = lib().ora_pagerank(self._h, int(reversed), _ptr(vm, _u8p), _ptr(em, _u8p),
                                _ptr(w, _f64p), _ptr(p, _f64p), damping, epsilon, max_iter, pl,
                                ch, _ptr(out, _f64p), had, threads)
        if it < 0:
            raise OracleError(lib().ora_last_error().decode())
        return out, it

    def eigenvector(self, weight=None, epsilon=1e-6, max_iter=0, grain=4096, x=None, had=None,
                    reversed=False, vmask=None, emask=None, threads=1, plan_len=None):
        """eigenvector (centrality.rs:405-497).  Returns (x f64[n], eig, iters)."""
        n = self.n
        out = np.zeros(n, np.float64)
        if x is not None:
            r = np.asarray(x, np.float64)
            k = min(r.size, n)
            out[:k] = r[:k]
            had = k if had is None else had
        else:
            had = 0 if had is None else had
        w = None if weight is None else np.ascontiguousarray(weight, np.float64)
        vm = None if vmask is None else np.ascontiguousarray(vmask, np.uint8)
        em = None if emask is None else np.ascontiguousarray(emask, np.uint8)
        pl = n if plan_len is None else plan_len
        eig = C.c_double(0.0)
        it = lib().ora_eigenvector(self._h, int(reversed), _ptr(vm, _u8p), _ptr(em, _u8p),
                                   _ptr(w, _f64p), epsilon, max_iter, pl, plan_chunks(pl, grain),
                                   _ptr(out, _f64p), had, threads, C.byref(eig))
        if it < 0:
            raise OracleError(lib().ora_last_error().decode())
        return out, eig.value, it

    def betweenness(self, undirected=False, reversed=False, vmask=None, emask=None, threads=1):
        """betweenness (centrality.rs:633-689) of the view (Und when
        ``undirected``).  Returns (vertex f64[n], edge f64[edge bound])."""
        vb = np.zeros(max(self.n, 1), np.float64)
        eb = np.zeros(max(self.edge_bound(), 1), np.float64)
        vm = None if vmask is None else np.ascontiguousarray(vmask, np.uint8)
        em = None if emask is None else np.ascontiguousarray(emask, np.uint8)
        st = lib().ora_betweenness(self._h, int(reversed), int(undirected), _ptr(vm, _u8p),
                                   _ptr(em, _u8p), _ptr(vb, _f64p), _ptr(eb, _f64p), threads)
        if st != 0:
            raise OracleError("betweenness: out of memory")
        return vb[:self.n], eb[:self.edge_bound()]


def max_threads() -> int:
    return lib().ora_max_threads()

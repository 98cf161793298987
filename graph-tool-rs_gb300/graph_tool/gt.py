"""``graph_tool.load_graph`` for the native binary .gt format.

The document is parsed by libgtc (``gtc_gt_open``: header, one record per
vertex, property table) and its adjacency is decoded on the GPU straight into
the graph handle (``gtc_gt_graph``), which replays add_edge(v, u) for every
vertex v and every entry u of v's list in file order -- the call sequence of
the reference's reader, crates/gt-io/src/gt.rs:628-678 of graph-tool-rs --
so edge k is the file's k-th list entry and every block is the reference's.

Property columns come back keyed the way the reference keys them
(gt.rs:88-107): a graph column holds one value, a vertex column one per
vertex, an edge column one per edge id.  Numeric scalar columns (bool,
int16/32/64, double) become ``PropertyMap`` objects of that type; the other
kinds are returned as Python lists (str, numpy arrays for numeric vectors,
bytes for long double and pickled objects).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _ffi
from ._rust import Graph, PropertyMap

KINDS = ["bool", "int16_t", "int32_t", "int64_t", "double", "long double", "string",
         "vector<bool>", "vector<int16_t>", "vector<int32_t>", "vector<int64_t>",
         "vector<double>", "vector<long double>", "vector<string>", "python::object"]
_NUMERIC = {0: "u1", 1: "i2", 2: "i4", 3: "i8", 4: "f8"}
_VEC = {8: "i2", 9: "i4", 10: "i8", 11: "f8"}
GRAPH, VERTEX, EDGE = 0, 1, 2


class GtFile:
    """A parsed .gt document (gtc_gt_open); ``bytes`` or a path."""

    def __init__(self, source):
        if isinstance(source, (str, os.PathLike)):
            with open(source, "rb") as fh:
                source = fh.read()
        data = bytes(source)
        h = C.c_void_p()
        _ffi.check(_ffi.lib().gtc_gt_open(data, len(data), C.byref(h)))
        self._h = h.value
        n, m, nprops = C.c_uint64(), C.c_uint64(), C.c_uint64()
        directed, big = C.c_int32(), C.c_int32()
        _ffi.check(_ffi.lib().gtc_gt_info(self._h, C.byref(n), C.byref(m), C.byref(directed),
                                          C.byref(big), C.byref(nprops)))
        self.n, self.m, self.nprops = n.value, m.value, nprops.value
        self.directed, self.big_endian = bool(directed.value), bool(big.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _ffi._lib is not None:
            _ffi._lib.gtc_gt_close(h)
            self._h = None

    def comment(self) -> str:
        p, ln = C.c_void_p(), C.c_uint64()
        _ffi.check(_ffi.lib().gtc_gt_comment(self._h, C.byref(p), C.byref(ln)))
        return C.string_at(p.value, ln.value).decode() if ln.value else ""

    def properties(self) -> list[tuple[str, int, int, int]]:
        """(name, domain, kind, count) of every column, in file order."""
        out = []
        for i in range(self.nprops):
            p, ln, dom, kind, cnt = (C.c_void_p(), C.c_uint64(), C.c_int32(), C.c_int32(),
                                     C.c_uint64())
            _ffi.check(_ffi.lib().gtc_gt_property(self._h, i, C.byref(p), C.byref(ln),
                                                  C.byref(dom), C.byref(kind), C.byref(cnt)))
            name = C.string_at(p.value, ln.value).decode() if ln.value else ""
            out.append((name, dom.value, kind.value, cnt.value))
        return out

    def raw(self, i: int) -> bytes:
        """The column's bytes as stored."""
        p, ln = C.c_void_p(), C.c_uint64()
        _ffi.check(_ffi.lib().gtc_gt_property_bytes(self._h, i, C.byref(p), C.byref(ln)))
        return C.string_at(p.value, ln.value) if ln.value else b""

    def values(self, i: int):
        """The values of column i: a numpy array for a numeric scalar
        column, else a list."""
        _, _, kind, count = self.properties()[i]
        b = self.raw(i)
        e = ">" if self.big_endian else "<"
        if kind in _NUMERIC:
            return np.frombuffer(b, dtype=e + _NUMERIC[kind], count=count).astype(
                np.dtype(_NUMERIC[kind]).newbyteorder("="))
        out, pos = [], 0

        def u64():
            nonlocal pos
            v = int(np.frombuffer(b, dtype=e + "u8", count=1, offset=pos)[0])
            pos += 8
            return v

        def run(k):
            nonlocal pos
            r = b[pos:pos + k]
            pos += k
            return r

        for _ in range(count):
            if kind == 5:
                x = run(16)
                out.append(x[::-1] if self.big_endian else x)
            elif kind == 6:
                out.append(run(u64()).decode())
            elif kind in (7, 14):
                out.append(run(u64()))
            elif kind in _VEC:
                k = u64()
                w = int(_VEC[kind][1])
                out.append(np.frombuffer(run(k * w), dtype=e + _VEC[kind]).astype(_VEC[kind]))
            elif kind == 12:
                k = u64()
                out.append([(lambda x: x[::-1] if self.big_endian else x)(run(16))
                            for _ in range(k)])
            else:  # vector<string>
                k = u64()
                out.append([run(u64()).decode() for _ in range(k)])
        return out

    def graph(self) -> Graph:
        """The document's graph, built on the GPU (gtc_gt_graph)."""
        h = C.c_void_p()
        _ffi.check(_ffi.lib().gtc_gt_graph(self._h, C.byref(h)))
        return Graph._from_handle(h.value, self.n, self.m)


_SCALAR_NAME = {0: "bool", 1: "int16_t", 2: "int32_t", 3: "int64_t", 4: "double"}


def load_graph(source) -> Graph:
    """Read a .gt document (a path or its bytes) into a Graph.

    The graph carries ``directed`` and the columns as ``gp`` / ``vp`` /
    ``ep`` dictionaries (graph-tool's names): numeric scalar vertex and edge
    columns as PropertyMaps of their type, everything else as the values
    themselves."""
    f = GtFile(source)
    g = f.graph()
    g.directed = f.directed
    g.gp, g.vp, g.ep = {}, {}, {}
    for i, (name, dom, kind, _) in enumerate(f.properties()):
        vals = f.values(i)
        if dom == GRAPH:
            g.gp[name] = vals[0]
            continue
        if kind in _SCALAR_NAME:
            pm = (g.new_vertex_property if dom == VERTEX else g.new_edge_property)(
                _SCALAR_NAME[kind])
            pm.a[:] = vals
            (g.vp if dom == VERTEX else g.ep)[name] = pm
        else:
            (g.vp if dom == VERTEX else g.ep)[name] = vals
    return g


__all__ = ["GtFile", "load_graph", "KINDS", "PropertyMap"]

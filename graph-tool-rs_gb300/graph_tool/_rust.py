"""``graph_tool._rust`` -- the reference's Python module surface, on libgtc.

Mirrors crates/gt-py/src/module.rs of graph-tool-rs: a ``Graph`` (:392-506),
a ``PropertyMap`` (:578-650) and ``value_types`` (:806-809), and adds the two
centrality entry points the reference does not bind yet, ``Graph.pagerank``
and ``Graph.eigenvector``, in the module's three-step shape (module.rs:1-17):
borrow the graph and the maps, size every map to the graph's bound
(``DenseProp::sized_for``, crates/gt-core/src/prop/dense.rs:88-125), then run
the kernel -- here on the GPU through the C ABI, with the interpreter lock
released by ctypes for the duration of the call.

Errors use the reference's translation table (module.rs:78-114): a bad
vertex or edge index and a bad argument are ValueError, a key outside the
index bound is IndexError, the rest RuntimeError.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi

_SCALARS = {
    "bool": np.uint8,
    "int16_t": np.int16,
    "int32_t": np.int32,
    "int64_t": np.int64,
    "double": np.float64,
    "long double": np.longdouble,
}

MAX_INDEX = 0xFFFFFFFE  # crates/gt-core/src/ids.rs:32 (Raw = u32)


def value_types() -> list[str]:
    """The scalar member names this module stores, graph-tool's spelling
    (crates/gt-core/src/prop/value.rs:100-116)."""
    return list(_SCALARS)


class PropertyMap:
    """A vertex ("v") or edge ("e") property map of one scalar type.

    The store grows to the graph's index bound whenever it is used and never
    shrinks (``sized_for``); a never-written key inside the bound reads as
    the type's zero."""

    def __init__(self, graph: "Graph", key_type: str, value_type: str):
        if value_type not in _SCALARS:
            raise ValueError(f"Invalid property type: {value_type}")
        self._g = graph
        self._key = key_type
        self._vt = value_type
        self._a = np.zeros(0, dtype=_SCALARS[value_type])

    def value_type(self) -> str:
        return self._vt

    def key_type(self) -> str:
        return self._key

    def allocated(self) -> int:
        return int(self._a.size)

    def _bound(self) -> int:
        return self._g.num_vertices() if self._key == "v" else self._g.edge_index_range()

    def sized_for(self) -> np.ndarray:
        """Grow to the bound (never shrink) and return the live view."""
        b = self._bound()
        if self._a.size < b:
            grown = np.zeros(b, dtype=self._a.dtype)
            grown[: self._a.size] = self._a
            self._a = grown
        return self._a[:b]

    def __getitem__(self, key: int):
        b = self._bound()
        if not 0 <= key < b:
            raise IndexError(f"{'vertex' if self._key == 'v' else 'edge'} index {key} is "
                             f"outside this graph's index bound of {b}")
        return self.sized_for()[key].item()

    def __setitem__(self, key: int, value) -> None:
        b = self._bound()
        if not 0 <= key < b:
            raise IndexError(f"{'vertex' if self._key == 'v' else 'edge'} index {key} is "
                             f"outside this graph's index bound of {b}")
        self.sized_for()[key] = value

    @property
    def a(self) -> np.ndarray:
        """The sized array (a view: writes go to the map)."""
        return self.sized_for()

    fa = a


class Graph:
    """A directed graph, edges added in call order (AdjList::add_edge,
    crates/gt-core/src/adj/list.rs:258-280).  The GPU copy of its adjacency is
    built on first use and rebuilt after a mutation."""

    def __init__(self):
        self._n = 0
        self._src: list[np.ndarray] = []
        self._tgt: list[np.ndarray] = []
        self._m = 0
        self._handle = None
        self._flat = None
        self._lazy = False  # edges live only in the handle (a graph read by load_graph)
        self.directed = True

    @classmethod
    def from_blocks(cls, n: int, edge_bound: int, block_off, out_len, entries) -> "Graph":
        """A graph from the reference's adjacency blocks as stored
        (gtc_graph_create_blocks): vertex v's Block is entries[block_off[v] ..
        block_off[v+1]) of (other, idx) pairs, out-half first (out_len[v]
        entries).  Edge ids below ``edge_bound`` that no entry uses are
        removed edges; edge maps are indexed up to ``edge_bound``.  The graph
        is read-only here (its history of removals has no edge-list form)."""
        block_off = np.ascontiguousarray(block_off, dtype=np.uint64)
        out_len = np.ascontiguousarray(out_len, dtype=np.uint32)
        entries = np.ascontiguousarray(entries, dtype=np.uint32).reshape(-1)
        if block_off.size != n + 1 or out_len.size != n:
            raise ValueError("block_off needs n + 1 entries and out_len n")
        if entries.size != 2 * int(block_off[-1] if n else 0):
            raise ValueError("entries must hold 2 uint32 per block entry")
        h = C.c_void_p()
        _ffi.check(_ffi.lib().gtc_graph_create_blocks(
            int(n), int(edge_bound), _ffi.ptr(block_off, _ffi.u64p), _ffi.ptr(out_len, _ffi.u32p),
            _ffi.ptr(entries, _ffi.u32p), C.byref(h)))
        nv, eb, live = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _ffi.check(_ffi.lib().gtc_graph_info(h, C.byref(nv), C.byref(eb), C.byref(live)))
        g = cls._from_handle(h.value, nv.value, live.value)
        g._bound = int(eb.value)
        g._frozen = True
        return g

    @classmethod
    def _from_handle(cls, handle, n: int, m: int) -> "Graph":
        """Adopt a gtc_graph built elsewhere (the .gt reader); its edge list
        is copied back from the device only when asked for."""
        g = cls()
        g._n, g._m, g._handle, g._lazy = int(n), int(m), handle, True
        return g

    # ---- size ---------------------------------------------------------
    def num_vertices(self) -> int:
        return self._n

    def num_edges(self) -> int:
        return self._m

    def edge_index_range(self) -> int:
        return getattr(self, "_bound", self._m)

    # ---- mutation -----------------------------------------------------
    def _dirty(self):
        if getattr(self, "_frozen", False):
            raise RuntimeError("a graph built from blocks is read-only")
        if self._lazy:
            self.edges()  # the handle is the only copy of the edges so far
        self._flat = None
        if self._handle is not None:
            _ffi.check(_ffi.lib().gtc_graph_destroy(self._handle))
            self._handle = None

    def add_vertex(self, n: int = 1) -> int:
        """Append ``n`` isolated vertices; return the index of the first."""
        if n < 0:
            raise ValueError("negative vertex count")
        if self._n + n > MAX_INDEX:
            raise RuntimeError(f"vertex index space exhausted (max {MAX_INDEX})")
        first = self._n
        self._n += n
        self._dirty()
        return first

    def add_edge(self, s: int, t: int) -> int:
        """Add an edge and return its index."""
        for x in (s, t):
            if not isinstance(x, (int, np.integer)) or x < 0 or x > MAX_INDEX:
                raise ValueError(f"Invalid vertex index: {x}")
            if x >= self._n:
                raise ValueError(f"no such vertex: VertexId({x})")
        return self.add_edges(np.array([s], np.uint32), np.array([t], np.uint32))

    def add_edges(self, src, tgt) -> int:
        """Bulk add_edge in array order; return the index of the first edge."""
        src = np.ascontiguousarray(src).astype(np.int64, copy=False).ravel()
        tgt = np.ascontiguousarray(tgt).astype(np.int64, copy=False).ravel()
        if src.shape != tgt.shape:
            raise ValueError("src and tgt differ in length")
        if src.size:
            lo = min(int(src.min()), int(tgt.min()))
            hi = max(int(src.max()), int(tgt.max()))
            if lo < 0:
                raise ValueError(f"Invalid vertex index: {lo}")
            if hi >= self._n:
                raise ValueError(f"no such vertex: VertexId({hi})")
        if self._m + src.size > MAX_INDEX:
            raise RuntimeError(f"edge index space exhausted (max {MAX_INDEX})")
        first = self._m
        self._src.append(src.astype(np.uint32))
        self._tgt.append(tgt.astype(np.uint32))
        self._m += src.size
        self._dirty()
        return first

    def edges(self):
        """(src, tgt) arrays indexed by edge index."""
        if self._lazy:
            # every out-half entry (other, idx) of vertex v is edge idx: v -> other
            oo, ot, oi, _, _, _ = self.blocks()
            src = np.empty(self._m, np.uint32)
            tgt = np.empty(self._m, np.uint32)
            src[oi] = np.repeat(np.arange(self._n, dtype=np.uint32), np.diff(oo).astype(np.int64))
            tgt[oi] = ot
            self._src, self._tgt, self._lazy = [src], [tgt], False
        if self._flat is None:
            if self._src:
                self._flat = (np.concatenate(self._src), np.concatenate(self._tgt))
                self._src, self._tgt = [self._flat[0]], [self._flat[1]]
            else:
                self._flat = (np.zeros(0, np.uint32), np.zeros(0, np.uint32))
        return self._flat

    # ---- maps ---------------------------------------------------------
    def new_vertex_property(self, value_type: str) -> PropertyMap:
        return PropertyMap(self, "v", value_type)

    def new_edge_property(self, value_type: str) -> PropertyMap:
        return PropertyMap(self, "e", value_type)

    def sum_property(self, prop: PropertyMap) -> float:
        """Sum a scalar map over this graph's index space (module.rs:481-506)."""
        if prop._g is not self:
            raise ValueError("property map belongs to another graph")
        return float(np.sum(prop.sized_for(), dtype=np.float64))

    # ---- the device copy ----------------------------------------------
    def handle(self):
        """The gtc_graph handle (built on first use)."""
        if self._handle is None:
            src, tgt = self.edges()
            h = C.c_void_p()
            _ffi.check(_ffi.lib().gtc_graph_create(self._n, self._m, _ffi.ptr(src, _ffi.u32p),
                                                   _ffi.ptr(tgt, _ffi.u32p), C.byref(h)))
            self._handle = h.value
        return self._handle

    def blocks(self):
        """Every block's out-half and in-half as the GPU holds them:
        (out_off, out_other, out_idx, in_off, in_other, in_idx)."""
        h = self.handle()
        n, m = self._n, self._m
        oo = np.zeros(n + 1, np.uint64)
        io = np.zeros(n + 1, np.uint64)
        arrs = [np.zeros(max(m, 1), np.uint32) for _ in range(4)]
        _ffi.check(_ffi.lib().gtc_graph_export(
            h, _ffi.ptr(oo, _ffi.u64p), _ffi.ptr(arrs[0], _ffi.u32p), _ffi.ptr(arrs[1], _ffi.u32p),
            _ffi.ptr(io, _ffi.u64p), _ffi.ptr(arrs[2], _ffi.u32p), _ffi.ptr(arrs[3], _ffi.u32p)))
        return oo, arrs[0][:m], arrs[1][:m], io, arrs[2][:m], arrs[3][:m]

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and _ffi._lib is not None:
            _ffi._lib.gtc_graph_destroy(h)
            self._handle = None

    # ---- centrality ---------------------------------------------------
    def pagerank(self, rank: PropertyMap, weight: PropertyMap | None = None,
                 pers: PropertyMap | None = None, damping: float = 0.85,
                 epsilon: float = 1e-6, max_iter: int = 0, grain: int = 4096,
                 reversed: bool = False, vfilt=None, efilt=None,
                 precision: str = "f32", stream=None, result: bool = False,
                 plan_len: int | None = None, schedule: str = "auto"):
        """pagerank / pagerank_with (crates/gt-algo/src/centrality.rs:234-384)
        on this graph, its reversal or a filtered view.  ``rank`` is the
        initial iterate and the output; returns the number of sweeps (and the
        full gtc_result when ``result``).  ``schedule`` pins one FP32 sweep
        kernel (``_ffi.SCHEDULES``; "auto" lets the autotuner choose)."""
        return _solve(self, "pagerank", rank, weight, pers, damping, epsilon, max_iter, grain,
                      reversed, vfilt, efilt, precision, stream, result, plan_len, schedule)

    def eigenvector(self, x: PropertyMap, weight: PropertyMap | None = None,
                    epsilon: float = 1e-6, max_iter: int = 0, grain: int = 4096,
                    reversed: bool = False, vfilt=None, efilt=None, precision: str = "f32",
                    stream=None, result: bool = False, plan_len: int | None = None,
                    schedule: str = "auto"):
        """eigenvector (crates/gt-algo/src/centrality.rs:405-497); returns
        (eigenvalue, sweeps)."""
        r = _solve(self, "eigenvector", x, weight, None, 0.0, epsilon, max_iter, grain, reversed,
                   vfilt, efilt, precision, stream, True, plan_len, schedule)
        return r if result else (r.eigenvalue, r.iterations)

    def weighted_degree(self, weight: PropertyMap | None = None, direction: str = "out",
                        reversed: bool = False, vfilt=None, efilt=None) -> PropertyMap:
        """weighted_out_degree / weighted_in_degree (crates/gt-algo/src/degree.rs
        :122-160) of every vertex: the FP64 left fold of the weights over its
        out-edges (``direction="out"``) or in-edges (``"in"``) in storage
        order; ``weight=None`` is Unity (the degree)."""
        if direction not in ("out", "in"):
            raise ValueError("direction must be 'out' or 'in'")
        w = _f64_map(self, weight, "e", "weight")
        out = self.new_vertex_property("double")
        d = out.sized_for()
        vm = _mask(self, vfilt, self.num_vertices())
        em = _mask(self, efilt, self.edge_index_range())
        view = _ffi.View(int(bool(reversed)), 0, _ffi.ptr(vm, _ffi.u8p),
                         0 if vm is None else vm.size, _ffi.ptr(em, _ffi.u8p),
                         0 if em is None else em.size)
        _ffi.check(_ffi.lib().gtc_weighted_degree(
            self.handle(), C.byref(view), int(direction == "in"), _ffi.ptr(w, _ffi.f64p),
            0 if w is None else w.size, _ffi.ptr(d, _ffi.f64p), d.size, None))
        return out

    def betweenness(self, vertex_bc: PropertyMap | None = None,
                    edge_bc: PropertyMap | None = None, undirected: bool = False,
                    reversed: bool = False, vfilt=None, efilt=None, result: bool = False):
        """betweenness (crates/gt-algo/src/centrality.rs:633-689): Brandes
        from every vertex of the view, unnormalised; both maps are
        overwritten.  ``undirected`` runs on the undirected view (halved).
        Returns (vertex map, edge map)."""
        vb = vertex_bc if vertex_bc is not None else self.new_vertex_property("double")
        eb = edge_bc if edge_bc is not None else self.new_edge_property("double")
        for m_, key in ((vb, "v"), (eb, "e")):
            if not isinstance(m_, PropertyMap) or m_._g is not self or m_.key_type() != key \
                    or m_.value_type() != "double":
                raise ValueError("betweenness maps must be 'double' maps of this graph")
        va, ea = vb.sized_for(), eb.sized_for()
        vm = _mask(self, vfilt, self.num_vertices())
        em = _mask(self, efilt, self.edge_index_range())
        view = _ffi.View(int(bool(reversed)), 0, _ffi.ptr(vm, _ffi.u8p),
                         0 if vm is None else vm.size, _ffi.ptr(em, _ffi.u8p),
                         0 if em is None else em.size)
        res = _ffi.Result()
        _ffi.check(_ffi.lib().gtc_betweenness(
            self.handle(), C.byref(view), int(bool(undirected)), _ffi.ptr(va, _ffi.f64p), va.size,
            _ffi.ptr(ea, _ffi.f64p), ea.size, None, C.byref(res)))
        return (vb, eb, res) if result else (vb, eb)

    def ppr_batch(self, seeds, values=None, weight: PropertyMap | None = None,
                  damping: float = 0.85, epsilon: float = 1e-6, max_iter: int = 0,
                  reversed: bool = False, gather: str = "bulk"):
        """Personalised PageRank for many seed sets at once.

        ``seeds`` is a list of B vertex-index sequences (1 <= B <= 512);
        ``values`` (optional) the matching personalisation values (default
        1/|set|).  Every vector is pagerank_with (centrality.rs:261-384) with
        that sparse personalisation, started from it, to ``epsilon``.
        ``gather`` picks the batched sweep's gather kernel ("bulk": rows staged
        by cp.async.bulk, the default; "regs": rows loaded into registers).
        Returns (ranks float64 [B][n], sweeps uint64 [B])."""
        if gather not in ("bulk", "regs"):
            raise ValueError("gather must be 'bulk' or 'regs'")
        B = len(seeds)
        n = self.num_vertices()
        off = np.zeros(B + 1, np.uint64)
        off[1:] = np.cumsum([len(x) for x in seeds])
        verts = np.ascontiguousarray(np.concatenate([np.asarray(x, np.int64) for x in seeds])
                                     if B else np.zeros(0), dtype=np.uint32)
        vals = None
        if values is not None:
            vals = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64) for x in values]))
            if vals.size != verts.size:
                raise ValueError("values do not match the seed sets")
        w = _f64_map(self, weight, "e", "weight")
        ranks = np.zeros((B, n), np.float64)
        iters = np.zeros(B, np.uint64)
        view = _ffi.View(int(bool(reversed)), 0, None, 0, None, 0)
        params = _ffi.PowerIteration(float(epsilon), int(max_iter or 0), n, max(-(-n // 4096), 1))
        res = _ffi.Result()
        opt = _ffi.Options(_ffi.GTC_PREC_F32, 0, None, 0,
                           _ffi.GTC_PPR_REGS if gather == "regs" else _ffi.GTC_PPR_BULK)
        _ffi.check(_ffi.lib().gtc_ppr_batch(
            self.handle(), C.byref(view), _ffi.ptr(w, _ffi.f64p), 0 if w is None else w.size, B,
            _ffi.ptr(off, _ffi.u64p), _ffi.ptr(verts, _ffi.u32p), _ffi.ptr(vals, _ffi.f64p),
            float(damping), C.byref(params), _ffi.ptr(ranks, _ffi.f64p), _ffi.ptr(iters, _ffi.u64p),
            C.byref(opt), C.byref(res)))
        return ranks, iters


class GraphBatch:
    """Many graphs of uneven sizes, packed as one block-diagonal graph and
    solved together (no counterpart in the reference, which takes one graph
    per call).  ``graphs`` is a sequence of (n, src, tgt) with local vertex
    indices; the edges of each graph are added in array order."""

    def __init__(self, graphs):
        G = len(graphs)
        if G == 0:
            raise ValueError("a batch holds at least one graph")
        self._n = np.array([int(g[0]) for g in graphs], np.uint64)
        self._m = np.array([len(g[1]) for g in graphs], np.uint64)
        voff = np.zeros(G + 1, np.uint64)
        eoff = np.zeros(G + 1, np.uint64)
        voff[1:] = np.cumsum(self._n)
        eoff[1:] = np.cumsum(self._m)
        src = np.ascontiguousarray(np.concatenate([np.asarray(g[1], np.int64) for g in graphs])
                                   if eoff[-1] else np.zeros(0), dtype=np.uint32)
        tgt = np.ascontiguousarray(np.concatenate([np.asarray(g[2], np.int64) for g in graphs])
                                   if eoff[-1] else np.zeros(0), dtype=np.uint32)
        h = C.c_void_p()
        _ffi.check(_ffi.lib().gtc_graph_batch_create(G, _ffi.ptr(voff, _ffi.u64p),
                                                     _ffi.ptr(eoff, _ffi.u64p),
                                                     _ffi.ptr(src, _ffi.u32p),
                                                     _ffi.ptr(tgt, _ffi.u32p), C.byref(h)))
        self._h = h.value
        self.voff, self.eoff = voff, eoff

    def __len__(self):
        return len(self._n)

    def handle(self):
        return self._h

    def pagerank(self, weight=None, damping: float = 0.85, epsilon: float = 1e-6,
                 max_iter: int = 0, result: bool = False):
        """pagerank (centrality.rs:234-248) of every graph; ``weight`` per edge
        of the packed edge list.  Returns (ranks, iters): ranks per vertex of
        the packed vertex list (graph k is ranks[voff[k]:voff[k+1]])."""
        n, m = int(self.voff[-1]), int(self.eoff[-1])
        w = None
        if weight is not None:
            w = np.ascontiguousarray(weight, dtype=np.float64)
            if w.size < m:
                raise ValueError(f"weight holds {w.size} entries, the batch has {m} edges")
        ranks = np.zeros(max(n, 1), np.float64)
        iters = np.zeros(len(self), np.uint64)
        res = _ffi.Result()
        opt = _ffi.Options(_ffi.GTC_PREC_F32, 0, None, 0, 0)
        _ffi.check(_ffi.lib().gtc_pagerank_batch(
            self._h, _ffi.ptr(w, _ffi.f64p), 0 if w is None else w.size, float(damping),
            float(epsilon), int(max_iter or 0), _ffi.ptr(ranks, _ffi.f64p), n,
            _ffi.ptr(iters, _ffi.u64p), C.byref(opt), C.byref(res)))
        out = (ranks[:n], iters)
        return out + (res,) if result else out

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _ffi._lib is not None:
            _ffi.lib().gtc_graph_batch_destroy(h)
            self._h = None


_PRECISIONS = {"f32": _ffi.GTC_PREC_F32, "f64_exact": _ffi.GTC_PREC_F64_EXACT}


def _f64_map(g: Graph, m, key: str, what: str):
    if m is None:
        return None
    if isinstance(m, PropertyMap):
        if m._g is not g:
            raise ValueError(f"{what} map belongs to another graph")
        if m.key_type() != key:
            raise ValueError(f"{what} must be a {'vertex' if key == 'v' else 'edge'} map")
        if m.value_type() != "double":
            raise ValueError(f"{what} map holds {m.value_type()!r}, a 'double' map is required")
        return m.sized_for()
    a = np.ascontiguousarray(m, dtype=np.float64)
    bound = g.num_vertices() if key == "v" else g.edge_index_range()
    if a.size < bound:
        raise ValueError(f"{what} holds {a.size} entries, the graph's index bound is {bound}")
    return a


def _mask(g: Graph, m, bound: int):
    if m is None:
        return None
    if isinstance(m, PropertyMap):
        m = m.sized_for()
    a = np.ascontiguousarray(np.asarray(m) != 0, dtype=np.uint8)
    if a.size != bound:
        raise ValueError(f"filter mask holds {a.size} entries, the index bound is {bound}")
    return a


def _solve(g: Graph, kind, out_map, weight, pers, damping, epsilon, max_iter, grain, reversed,
           vfilt, efilt, precision, stream, want_result, plan_len=None, schedule="auto"):
    if not isinstance(out_map, PropertyMap):
        raise ValueError("the output must be a vertex PropertyMap of 'double'")
    if out_map._g is not g or out_map.key_type() != "v" or out_map.value_type() != "double":
        raise ValueError("the output must be a 'double' vertex map of this graph")
    if grain <= 0:
        raise ValueError("Plan::new: grain must be non-zero")
    if precision not in _PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}")
    if schedule not in _ffi.SCHEDULES:
        raise ValueError(f"schedule must be one of {sorted(_ffi.SCHEDULES)}")
    n = g.num_vertices()
    w = _f64_map(g, weight, "e", "weight")
    p = _f64_map(g, pers, "v", "pers")
    had = out_map.allocated()
    x = out_map.sized_for()  # step 2 of the module shape: size before the kernel
    vm = _mask(g, vfilt, n)
    em = _mask(g, efilt, g.edge_index_range())
    view = _ffi.View(int(bool(reversed)), 0, _ffi.ptr(vm, _ffi.u8p), 0 if vm is None else vm.size,
                     _ffi.ptr(em, _ffi.u8p), 0 if em is None else em.size)
    # PowerIteration.plan: Plan::new(plan_len, grain); plan_len must be n
    pl = n if plan_len is None else int(plan_len)
    params = _ffi.PowerIteration(float(epsilon), int(max_iter or 0), pl, max(-(-pl // grain), 1))
    opt = _ffi.Options(_PRECISIONS[precision], _ffi.SCHEDULES[schedule], stream, 0, 0)
    res = _ffi.Result()
    L = _ffi.lib()
    h = g.handle()
    if kind == "pagerank":
        st = L.gtc_pagerank(h, C.byref(view), _ffi.ptr(w, _ffi.f64p), 0 if w is None else w.size,
                            _ffi.ptr(p, _ffi.f64p), 0 if p is None else p.size, float(damping),
                            C.byref(params), _ffi.ptr(x, _ffi.f64p), x.size, had, C.byref(opt),
                            C.byref(res))
    else:
        st = L.gtc_eigenvector(h, C.byref(view), _ffi.ptr(w, _ffi.f64p),
                               0 if w is None else w.size, C.byref(params),
                               _ffi.ptr(x, _ffi.f64p), x.size, had, C.byref(opt), C.byref(res))
    _ffi.check(st)
    return res if want_result else int(res.iterations)

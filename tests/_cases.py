"""The reference's centrality tests (crates/gt-algo/tests/u16_centrality.rs),
written once against a solver interface so the same cases pin the CPU oracle
and check the GPU library in both arithmetics.

A solver has ``pagerank``, ``eigenvector`` and ``blocks`` (see OracleSolver
and GpuSolver) and a ``tol(t)`` that widens a reference tolerance ``t`` to
what its arithmetic can meet (identity for FP64, FP32 rounding otherwise).
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KA = json.load(open(os.path.join(GOLDEN, "u16_known_answers.json")))


def edges_of(pairs):
    e = np.array(pairs, dtype=np.uint32).reshape(-1, 2)
    return e[:, 0].copy(), e[:, 1].copy()


# --------------------------------------------------------------------------
# solvers
# --------------------------------------------------------------------------

class OracleSolver:
    name = "oracle"
    exact = True

    def __init__(self, O, threads=1):
        self.O = O
        self.threads = threads

    def tol(self, t):
        return t

    def graph(self, n, src, tgt):
        g = self.O.Graph(n)
        g.add_edge_arrays(src, tgt)
        return g

    def pagerank(self, n, src, tgt, grain=64, **kw):
        g = self.graph(n, src, tgt)
        return g.pagerank(grain=grain, threads=self.threads, **kw)

    def eigenvector(self, n, src, tgt, grain=64, **kw):
        g = self.graph(n, src, tgt)
        return g.eigenvector(grain=grain, threads=self.threads, **kw)

    def blocks(self, n, src, tgt):
        return self.graph(n, src, tgt).export()

    def betweenness(self, n, src, tgt, undirected=False, reversed=False, vmask=None,
                    emask=None):
        return self.graph(n, src, tgt).betweenness(undirected=undirected, reversed=reversed,
                                                   vmask=vmask, emask=emask,
                                                   threads=self.threads)


class GpuSolver:
    """The GPU library through its C ABI (graph_tool._rust over ctypes)."""

    def __init__(self, gt, precision):
        self.gt = gt
        self.precision = precision
        self.exact = precision == "f64_exact"
        self.name = "gpu-" + precision

    def tol(self, t):
        return t if self.exact else max(t, 2e-6)

    def graph(self, n, src, tgt):
        g = self.gt.Graph()
        g.add_vertex(n)
        g.add_edges(src, tgt)
        return g

    def _maps(self, g, rank, had):
        r = g.new_vertex_property("double")
        if rank is not None:
            rank = np.asarray(rank, np.float64)
            k = rank.size if had is None else had
            r._a = rank[:k].copy()
        return r

    def pagerank(self, n, src, tgt, grain=64, weight=None, pers=None, rank=None, had=None,
                 vmask=None, emask=None, reversed=False, damping=0.85, epsilon=1e-6, max_iter=0,
                 plan_len=None):
        g = self.graph(n, src, tgt)
        r = self._maps(g, rank, had)
        res = g.pagerank(r, weight=weight, pers=pers, damping=damping, epsilon=epsilon,
                         max_iter=max_iter, grain=grain, reversed=reversed, vfilt=vmask,
                         efilt=emask, precision=self.precision, result=True, plan_len=plan_len)
        return r.a.copy(), int(res.iterations)

    def eigenvector(self, n, src, tgt, grain=64, weight=None, x=None, had=None, vmask=None,
                    emask=None, reversed=False, epsilon=1e-6, max_iter=0):
        g = self.graph(n, src, tgt)
        r = self._maps(g, x, had)
        res = g.eigenvector(r, weight=weight, epsilon=epsilon, max_iter=max_iter, grain=grain,
                            reversed=reversed, vfilt=vmask, efilt=emask,
                            precision=self.precision, result=True)
        return r.a.copy(), float(res.eigenvalue), int(res.iterations)

    def blocks(self, n, src, tgt):
        return self.graph(n, src, tgt).blocks()

    def betweenness(self, n, src, tgt, undirected=False, reversed=False, vmask=None,
                    emask=None):
        g = self.graph(n, src, tgt)
        vb, eb = g.new_vertex_property("double"), g.new_edge_property("double")
        g.betweenness(vb, eb, undirected=undirected, reversed=reversed, vfilt=vmask,
                      efilt=emask)
        return vb.a.copy(), eb.a.copy()


# --------------------------------------------------------------------------
# independent references used by the cases
# --------------------------------------------------------------------------

def dense_pagerank(n, edges_w, pers, d, sweeps):
    """u16_centrality.rs:138-175: explicit n x n transition matrix, fixed
    sweep count, zero-out-weight columns skipped."""
    deg = np.zeros(n)
    for s, _, w in edges_w:
        deg[s] += w
    M = np.zeros((n, n))
    for s, t, w in edges_w:
        if deg[s] != 0.0:
            M[t, s] += w / deg[s]
    r = np.array(pers, dtype=np.float64)
    pers = np.array(pers, dtype=np.float64)
    for _ in range(sweeps):
        p_sink = sum(r[i] for i in range(n) if deg[i] == 0.0)
        r = (1.0 - d) * pers + d * (p_sink * pers + M @ r)
    return r


def eigen_residual(n, src, tgt, w, eig, c):
    """u16_centrality.rs:474-490: max |(A c)[v] - eig * c[v]|."""
    ac = np.zeros(n)
    np.add.at(ac, tgt.astype(np.int64), w * c[src.astype(np.int64)])
    return float(np.max(np.abs(ac - eig * c)))


# --------------------------------------------------------------------------
# the cases
# --------------------------------------------------------------------------

def case_odd_sweep_pagerank(S):
    k = KA["odd_sweep_pagerank"]
    src, tgt = edges_of(k["edges"])
    r, it = S.pagerank(2, src, tgt, epsilon=k["epsilon"], max_iter=1)
    assert it == 1
    assert r[0] != 0.5, "the initial iterate was handed back"
    for a, b in zip(r, k["rank"]):
        assert abs(a - b) < S.tol(k["tol"]), (r, k["rank"])
    # two sweeps: the even case equals the dense iteration
    r2, it2 = S.pagerank(2, src, tgt, epsilon=k["epsilon"], max_iter=2)
    assert it2 == 2
    want = dense_pagerank(2, [(0, 1, 1.0)], [0.5, 0.5], 0.85, 2)
    assert np.max(np.abs(r2 - want)) < S.tol(1e-15)


def case_warm_start(S):
    k = KA["warm_start_pagerank"]
    src, tgt = edges_of(k["edges"])
    r, it = S.pagerank(2, src, tgt, rank=k["start"], epsilon=k["epsilon"], max_iter=1)
    want = [eval(e) for e in k["rank_expr"]]
    assert abs(r[0] - want[0]) < S.tol(k["tol"])
    assert abs(r[1] - want[1]) < S.tol(k["tol"])


def case_cycle_and_pers(S):
    k = KA["cycle4_uniform"]
    src, tgt = edges_of(k["edges"])
    r, _ = S.pagerank(4, src, tgt, epsilon=k["epsilon"], max_iter=k["max_iter"])
    assert np.max(np.abs(r - 0.25)) < S.tol(k["tol"])
    k = KA["cycle4_pers"]
    pers = np.array(k["pers"])
    r, _ = S.pagerank(4, src, tgt, pers=pers, epsilon=k["epsilon"], max_iter=k["max_iter"])
    assert r[0] > 0.25 and r[0] > r[1] > r[2] > r[3]
    assert abs(r.sum() - 1.0) < S.tol(k["mass_tol"])
    want = dense_pagerank(4, [(int(a), int(b), 1.0) for a, b in zip(src, tgt)], pers, 0.85, 400)
    assert np.max(np.abs(r - want)) < S.tol(k["dense_tol"])


def case_zero_weight_predecessor(S):
    k = KA["zero_weight_predecessor"]
    src, tgt = edges_of(k["edges"])
    r, _ = S.pagerank(3, src, tgt, weight=np.array(k["weight"]), epsilon=k["epsilon"],
                      max_iter=k["max_iter"])
    assert np.all(np.isfinite(r))
    s2, t2 = edges_of(k["alone_edges"])
    want, _ = S.pagerank(3, s2, t2, epsilon=k["epsilon"], max_iter=k["max_iter"])
    assert np.max(np.abs(r - want)) < S.tol(k["tol"])


def case_plan_must_cover(S):
    k = KA["plan_must_cover"]
    src, tgt = edges_of(k["edges"])
    try:
        S.pagerank(4, src, tgt, epsilon=1e-6, max_iter=10, plan_len=k["plan_len"])
    except Exception as e:  # noqa: BLE001
        assert k["message"] in str(e), str(e)
    else:
        raise AssertionError("a plan that does not cover the index space was accepted")


def case_dense_thousand(S, thousand):
    k = KA["dense_thousand"]
    n, src, tgt = thousand
    want = dense_pagerank(n, [(int(a), int(b), 1.0) for a, b in zip(src, tgt)],
                          [1.0 / n] * n, 0.85, k["dense_sweeps"])
    eps = k["epsilon"] if S.exact else 1e-7
    r, it = S.pagerank(n, src, tgt, epsilon=eps, max_iter=k["max_iter"])
    lo, hi = k["iters_range"]
    assert lo <= it < hi, it
    assert np.max(np.abs(r - want)) < S.tol(k["tol"]) / (1 if S.exact else 100)
    assert abs(r.sum() - 1.0) < S.tol(k["mass_tol"])
    if not S.exact:
        rel_l1 = np.abs(r - want).sum() / np.abs(want).sum()
        assert rel_l1 < 1e-6, rel_l1


def case_cycle7_eigen(S):
    k = KA["cycle7_eigen"]
    n = k["n"]
    src = np.arange(n, dtype=np.uint32)
    tgt = ((np.arange(n) + 1) % n).astype(np.uint32)
    x, eig, _ = S.eigenvector(n, src, tgt, epsilon=k["epsilon"], max_iter=k["max_iter"])
    assert abs(eig - 1.0) < S.tol(k["tol"])
    assert np.max(np.abs(x - 1.0 / math.sqrt(n))) < S.tol(k["tol"])
    x2, eig2, _ = S.eigenvector(n, src, tgt, weight=np.full(n, k["const_weight"]),
                                epsilon=k["epsilon"], max_iter=k["max_iter"])
    assert abs(eig2 - k["eig_const"]) < S.tol(k["tol"]) * k["eig_const"]


def case_edgeless_eigen(S):
    k = KA["edgeless_eigen"]
    x, eig, it = S.eigenvector(5, np.zeros(0, np.uint32), np.zeros(0, np.uint32),
                               epsilon=k["epsilon"], max_iter=k["max_iter"])
    assert eig == 0.0
    assert it >= 1
    assert np.all(np.isfinite(x)) and np.all(x == 0.0)


def case_odd_sweep_eigen(S):
    k = KA["odd_sweep_eigen"]
    src, tgt = edges_of(k["edges"])
    x, eig, it = S.eigenvector(3, src, tgt, epsilon=k["epsilon"], max_iter=1)
    assert it == 1
    assert abs(eig - math.sqrt(2.0) / 3.0) < S.tol(k["tol"])
    h = 1.0 / math.sqrt(2.0)
    assert abs(x[0]) < S.tol(k["tol"])
    assert abs(x[1] - h) < S.tol(k["tol"]) and abs(x[2] - h) < S.tol(k["tol"])


def case_eigen60(S, eigen60):
    k = KA["eigen60_equation"]
    n, src, tgt, w = eigen60
    eps = k["epsilon"] if S.exact else 1e-9
    x, eig, it = S.eigenvector(n, src, tgt, weight=w, epsilon=eps, max_iter=k["max_iter"])
    assert it > 1 and eig > 1.0
    res = eigen_residual(n, src, tgt, w, eig, x)
    assert res < (k["residual"] if S.exact else 1e-5), res
    assert abs(np.sqrt((x * x).sum()) - 1.0) < S.tol(k["norm_tol"])


def case_push_swap(S):
    # vertex 0: in(e0) from 1, in(e1) from 2, then out(e2) to 1
    src = np.array([1, 2, 0], np.uint32)
    tgt = np.array([0, 0, 1], np.uint32)
    oo, ot, oi, io, it, ii = S.blocks(3, src, tgt)
    assert list(ii[io[0]:io[1]]) == KA["push_swap"]["inc"]
    assert list(oi[oo[0]:oo[1]]) == KA["push_swap"]["out"]


def case_unity_is_general(S, thousand):
    n, src, tgt = thousand
    eps = 1e-13 if S.exact else 1e-7
    a, ia = S.pagerank(n, src, tgt, epsilon=eps, max_iter=10_000)
    b, ib = S.pagerank(n, src, tgt, weight=np.ones(src.size), epsilon=eps, max_iter=10_000)
    if S.exact:
        assert ia == ib and a.tobytes() == b.tobytes()
    else:
        assert np.max(np.abs(a - b)) < 1e-7


# --------------------------------------------------------------------------
# betweenness (u16_centrality.rs:620-883)
# --------------------------------------------------------------------------

def brandes_flat(n, edges, directed):
    """u16_centrality.rs:628-691: an independent Brandes over a flat edge list
    (adjacency in edge order; an undirected edge listed at both endpoints),
    unnormalised, halved when undirected."""
    adj = [[] for _ in range(n)]
    for ei, (s_, t_) in enumerate(edges):
        adj[s_].append((t_, ei))
        if not directed and s_ != t_:
            adj[t_].append((s_, ei))
    vb = [0.0] * n
    eb = [0.0] * len(edges)
    for s_ in range(n):
        dist = [-1] * n
        sigma = [0.0] * n
        dep = [0.0] * n
        pred = [[] for _ in range(n)]
        order = [s_]
        dist[s_], sigma[s_] = 0, 1.0
        head = 0
        while head < len(order):
            u = order[head]
            head += 1
            for w, ei in adj[u]:
                if w == u:
                    continue
                if dist[w] < 0:
                    dist[w] = dist[u] + 1
                    sigma[w] = sigma[u]
                    pred[w].append((u, ei))
                    order.append(w)
                elif dist[w] == dist[u] + 1:
                    sigma[w] += sigma[u]
                    pred[w].append((u, ei))
        for u in reversed(order):
            for p, ei in pred[u]:
                f = (sigma[p] / sigma[u]) * (1.0 + dep[u])
                dep[p] += f
                eb[ei] += f
            if u != s_:
                vb[u] += dep[u]
    if not directed:
        vb = [x / 2.0 for x in vb]
        eb = [x / 2.0 for x in eb]
    return np.array(vb), np.array(eb)


def case_betweenness_random(S, cases=100):
    """u16_centrality.rs:707-760: 100 small multigraphs with self-loops,
    directed and undirected, within 1e-9 of the independent Brandes."""
    from graph_tool.synth import SplitMix64
    r = SplitMix64(0x0123_4567_89AB_CDEF)
    for case in range(cases):
        n = 3 + r.below(10)
        m = r.below(3 * n + 1)
        edges = [(r.below(n), r.below(n)) for _ in range(m)]
        src, tgt = edges_of(edges) if m else (np.zeros(0, np.uint32), np.zeros(0, np.uint32))
        for directed in (True, False):
            gv, ge = S.betweenness(n, src, tgt, undirected=not directed)
            wv, we = brandes_flat(n, edges, directed)
            assert np.all(np.abs(gv - wv) < 1e-9), (case, directed, gv, wv)
            assert np.all(np.abs(ge - we) < 1e-9), (case, directed, ge, we)


def case_betweenness_path(S):
    """u16_centrality.rs:767-792: on a 9-vertex path, vertex i has
    i (n-1-i) and edge (i, i+1) has (i+1)(n-1-i), exactly."""
    N = 9
    src, tgt = edges_of([(i, i + 1) for i in range(N - 1)])
    for undirected in (False, True):
        gv, ge = S.betweenness(N, src, tgt, undirected=undirected)
        assert gv.tolist() == [float(i * (N - 1 - i)) for i in range(N)]
        assert ge.tolist() == [float((i + 1) * (N - 1 - i)) for i in range(N - 1)]


def case_betweenness_back_edge(S):
    """u16_centrality.rs:794-831: a 4-cycle with a chord, and its relabelling."""
    edges = [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2)]
    gv, ge = S.betweenness(4, *edges_of(edges))
    wv, we = brandes_flat(4, edges, True)
    assert np.all(np.abs(gv - wv) < 1e-12) and np.all(np.abs(ge - we) < 1e-12)
    hv, _ = S.betweenness(4, *edges_of([(3 - s_, 3 - t_) for s_, t_ in edges]))
    assert np.all(np.abs(hv[::-1] - gv) < 1e-12)


def case_betweenness_unreachable(S):
    """u16_centrality.rs:870-883: no NaN from the unreachable half; the cut
    vertex and the lone edge of the second component are exact."""
    gv, ge = S.betweenness(6, *edges_of([(0, 1), (1, 2), (3, 4)]), undirected=True)
    assert np.all(np.isfinite(gv))
    assert gv[1] == 1.0 and gv[0] == 0.0 and gv[5] == 0.0
    assert ge[2] == 1.0


def ring_plus_chords(n=220, chords=600, seed=0xDEAD_BEEF_1234_5678):
    """u16_centrality.rs:846-853: a ring plus random chords."""
    from graph_tool.synth import SplitMix64
    r = SplitMix64(seed)
    edges = [(i, (i + 1) % n) for i in range(n)]
    edges += [(r.below(n), r.below(n)) for _ in range(chords)]
    return n, edges

"""Every FP32 sweep kernel (gtc_schedule), pinned one at a time, against the
oracle's f64 result and against each other.

The graph puts rows in all three in-degree tiers of the sweep: sliced rows
(<= 128 in-edges), medium rows (129 .. 2048, a warp per row) and long rows
cut into 2048-entry chunks (here 3, 4 and 5 chunks, folded by the last warp
to finish one).  It has more vertices than the largest shared-memory prefix
of the gathered vector (32,768 entries), so every prefix boundary of the
hot-prefix kernels falls inside the graph and the sources of every tier lie
on both sides of it.  A schedule changes where a gather is served from,
never a value: results and sweep counts must be bitwise equal across
schedules (the row sums and the reductions do not depend on the kernel).

The reference loop these kernels replace: crates/gt-algo/src/centrality.rs
:340-369 (pagerank_with) and :446-484 (eigenvector)."""
import numpy as np
import pytest

import _cases as K

pytestmark = pytest.mark.gpu

SCHEDULES = ["l1", "hot32k", "hot24k", "hot16k", "hot8k"]


@pytest.fixture(scope="module")
def tiers():
    rng = np.random.default_rng(2024)
    n = 50_000
    m0 = 450_000
    src = rng.integers(0, n, m0)
    tgt = rng.integers(0, n, m0)
    # medium rows: 60 rows with 200 .. 1900 in-edges
    med = rng.choice(n, 60, replace=False)
    ms, mt = [], []
    for r in med:
        k = int(rng.integers(200, 1900))
        ms.append(rng.integers(0, n, k))
        mt.append(np.full(k, r))
    # long rows of 3, 4 and 5 chunks of 2048
    for r, k in ((11, 4500), (40_001, 7000), (33_000, 9500)):
        ms.append(rng.integers(0, n, k))
        mt.append(np.full(k, r))
    src = np.concatenate([src] + ms)
    tgt = np.concatenate([tgt] + mt)
    order = rng.permutation(src.size)
    src, tgt = src[order], tgt[order]
    # 5% of the vertices lose their out-edges (dangling mass)
    sinks = rng.choice(n, n // 20, replace=False)
    keep = ~np.isin(src, sinks)
    src, tgt = src[keep].astype(np.uint32), tgt[keep].astype(np.uint32)
    indeg = np.bincount(tgt, minlength=n)
    assert (indeg > 2048 * 2).sum() >= 2 and ((indeg > 128) & (indeg <= 2048)).sum() >= 50
    return n, src, tgt


def _rel_l1(a, b):
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def _kwargs(kind, n, m, rng):
    if kind == "plain":
        return {}
    if kind == "weighted":
        return {"weight": rng.uniform(0.1, 1.0, m)}
    if kind == "reversed":
        return {"reversed": True}
    p = rng.uniform(0.0, 1.0, n)
    p[rng.choice(n, n // 3, replace=False)] = 0.0
    return {"pers": p / p.sum()}


def _gpu(gtc, n, src, tgt, schedule, solver, eps, **kw):
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    r = g.new_vertex_property("double")
    w = None
    if "weight" in kw:
        w = g.new_edge_property("double")
        w.a[:] = kw.pop("weight")
    if solver == "pagerank":
        p = None
        if "pers" in kw:
            p = g.new_vertex_property("double")
            p.a[:] = kw.pop("pers")
        res = g.pagerank(r, weight=w, pers=p, epsilon=eps, max_iter=1000, result=True,
                         schedule=schedule, **kw)
        return r.a.copy(), int(res.iterations), 0.0
    res = g.eigenvector(r, weight=w, epsilon=eps, max_iter=1000, result=True,
                        schedule=schedule, **kw)
    return r.a.copy(), int(res.iterations), float(res.eigenvalue)


@pytest.mark.parametrize("kind", ["plain", "weighted", "reversed", "pers"])
def test_pagerank_every_schedule(oracle, gtc, tiers, kind):
    n, src, tgt = tiers
    kw = _kwargs(kind, n, src.size, np.random.default_rng(7))
    want, iw = K.OracleSolver(oracle).pagerank(n, src, tgt, grain=4096, epsilon=1e-7,
                                               max_iter=1000, **kw)
    first = None
    for sched in SCHEDULES:
        got, ig, _ = _gpu(gtc, n, src, tgt, sched, "pagerank", 1e-7, **dict(kw))
        err = _rel_l1(got, want)
        print(f"pagerank {kind} {sched}: rel L1 {err:.3e}, max abs "
              f"{np.max(np.abs(got - want)):.3e}, sweeps {ig} vs {iw}")
        assert err <= 1e-6, (sched, err)
        assert abs(ig - iw) <= 2, (sched, ig, iw)
        if first is None:
            first = (got, ig)
        else:
            assert ig == first[1], (sched, ig, first[1])
            assert got.tobytes() == first[0].tobytes(), sched


@pytest.mark.parametrize("kind", ["plain", "weighted", "reversed"])
def test_eigenvector_every_schedule(oracle, gtc, tiers, kind):
    n, src, tgt = tiers
    kw = _kwargs(kind, n, src.size, np.random.default_rng(8))
    # epsilon 1e-5: above the FP32 floor of the L1 change of a normalised
    # vector of 50,000 entries (near 1e-6 the FP32 iterate's rounding noise
    # delays the stop by a few sweeps while the vector is already within
    # 1e-7 of the oracle's)
    want, ew, iw = K.OracleSolver(oracle).eigenvector(n, src, tgt, grain=4096, epsilon=1e-5,
                                                      max_iter=1000, **kw)
    first = None
    for sched in SCHEDULES:
        got, ig, eg = _gpu(gtc, n, src, tgt, sched, "eigenvector", 1e-5, **dict(kw))
        err = _rel_l1(got, want)
        print(f"eigenvector {kind} {sched}: rel L1 {err:.3e}, eigenvalue {eg!r} vs {ew!r}, "
              f"sweeps {ig} vs {iw}")
        assert err <= 1e-6, (sched, err)
        assert abs(eg - ew) <= 1e-6 * ew, (sched, eg, ew)
        assert abs(ig - iw) <= 2, (sched, ig, iw)
        if first is None:
            first = (got, ig, eg)
        else:
            assert (ig, eg) == first[1:], (sched, ig, eg, first[1:])
            assert got.tobytes() == first[0].tobytes(), sched

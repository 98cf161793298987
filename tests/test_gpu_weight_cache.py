"""The handle keeps the FP32 layouts of the last weight map it solved with
(the in-half and out-half orders, the sliced entries, the weighted
degrees).  A repeated solve reuses them and gives the same bits; a map whose
contents changed (in place, at the same address) is laid out again, so the
result follows the new weights; either orientation and the eigenvector reuse
the same cache.  Checked against the oracle's f64 solves
(crates/gt-algo/src/centrality.rs:261-384, :405-497)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def test_weight_cache_follows_the_map(oracle, gtc):
    from graph_tool import synth
    n, src, tgt = synth.rmat_cpu(13, edge_factor=12, seed=31)
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    og = oracle.Graph(n)
    og.add_edge_arrays(src, tgt)
    rng = np.random.default_rng(4)
    w = g.new_edge_property("double")
    w.a[:] = rng.uniform(0.1, 1.0, src.size)
    r1 = g.new_vertex_property("double")
    g.pagerank(r1, weight=w, epsilon=1e-7, max_iter=1000)
    want, _ = og.pagerank(weight=w.a.copy(), epsilon=1e-7, max_iter=1000, grain=4096)
    assert _rel(r1.a, want) < 1e-6
    r2 = g.new_vertex_property("double")
    g.pagerank(r2, weight=w, epsilon=1e-7, max_iter=1000)  # the cached layouts
    assert r2.a.tobytes() == r1.a.tobytes()
    # the same map, changed in place: laid out again
    w.a[:] = rng.uniform(0.1, 1.0, src.size) ** 3
    r3 = g.new_vertex_property("double")
    g.pagerank(r3, weight=w, epsilon=1e-7, max_iter=1000)
    want3, _ = og.pagerank(weight=w.a.copy(), epsilon=1e-7, max_iter=1000, grain=4096)
    assert _rel(r3.a, want3) < 1e-6
    assert _rel(r3.a, want) > 1e-3  # the new weights do change the result
    # the other orientation and the eigenvector on the same cache
    r4 = g.new_vertex_property("double")
    g.pagerank(r4, weight=w, epsilon=1e-7, max_iter=1000, reversed=True)
    want4, _ = og.pagerank(weight=w.a.copy(), epsilon=1e-7, max_iter=1000, grain=4096,
                           reversed=True)
    assert _rel(r4.a, want4) < 1e-6
    x = g.new_vertex_property("double")
    g.eigenvector(x, weight=w, epsilon=1e-5, max_iter=1000)
    wantx, _, _ = og.eigenvector(weight=w.a.copy(), epsilon=1e-5, max_iter=1000, grain=4096)
    assert _rel(x.a, wantx) < 1e-6

"""Bounded behaviour at the boundary: every refusal comes back as an error
status (the Python exception of the reference's module.rs:78-114), and the
GPU stays usable afterwards.

* a weight map holding a NaN or an infinity is GTC_ERR_ARG (ValueError) for
  every solver that takes weights;
* an uncapped solve (max_iter 0) with epsilon <= 0 could never stop: refused;
* the many-graph batch's device loop gives up after its sweep limit with
  GTC_ERR_TIMEOUT; the limit is lowered to a few sweeps through the
  library's test hook, and a solve afterwards on the same batch succeeds."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def small(gtc):
    from graph_tool import synth
    n, src, tgt = synth.rmat_cpu(10, edge_factor=8, seed=2)
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    return g


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_non_finite_weights_are_refused(small, bad):
    g = small
    w = g.new_edge_property("double")
    w.a[:] = 0.5
    w.a[3] = bad
    for prec in ("f32", "f64_exact"):
        with pytest.raises(ValueError, match="non-finite"):
            g.pagerank(g.new_vertex_property("double"), weight=w, precision=prec)
        with pytest.raises(ValueError, match="non-finite"):
            g.eigenvector(g.new_vertex_property("double"), weight=w, precision=prec)
    with pytest.raises(ValueError, match="non-finite"):
        g.ppr_batch([[0, 1], [2]], weight=w)
    # the GPU and the handle stay usable
    w.a[3] = 0.5
    assert g.pagerank(g.new_vertex_property("double"), weight=w, epsilon=1e-6) > 0


def test_uncapped_solve_without_a_stop_is_refused(small):
    g = small
    for eps in (0.0, -1.0):
        with pytest.raises(ValueError, match="never stop"):
            g.pagerank(g.new_vertex_property("double"), epsilon=eps, max_iter=0)
        with pytest.raises(ValueError, match="never stop"):
            g.eigenvector(g.new_vertex_property("double"), epsilon=eps, max_iter=0)


def test_batch_sweep_limit_gives_timeout_then_recovers(gtc):
    from graph_tool import _ffi, synth
    from graph_tool._rust import GraphBatch
    graphs = [synth.rmat_cpu(9, edge_factor=6, seed=s) for s in (1, 2, 3)]
    b = GraphBatch(graphs)
    L = _ffi.lib()
    try:
        _ffi.check(L.gtc_debug_set_batch_sweep_limit(3))
        with pytest.raises(_ffi.GtcError, match="did not converge within 3 sweeps"):
            b.pagerank(epsilon=1e-30, max_iter=0)
    finally:
        _ffi.check(L.gtc_debug_set_batch_sweep_limit(0))
    ranks, iters = b.pagerank(epsilon=1e-6, max_iter=0)
    assert (iters > 3).all()
    assert np.all(np.isfinite(ranks))

"""Host-side logic of the Python boundary (no GPU): graph construction
errors, property-map sizing, the module surface of crates/gt-py/src/module.rs."""
import numpy as np
import pytest


def test_value_types(gtc):
    from graph_tool import value_types
    assert "double" in value_types() and "int32_t" in value_types()


def test_add_edge_errors_are_value_errors(gtc):
    g = gtc.Graph()
    g.add_vertex(3)
    assert g.add_edge(0, 1) == 0
    assert g.add_edge(1, 2) == 1
    with pytest.raises(ValueError, match="no such vertex"):
        g.add_edge(0, 3)
    with pytest.raises(ValueError, match="Invalid vertex index"):
        g.add_edge(-1, 0)
    assert g.num_edges() == 2 and g.edge_index_range() == 2 and g.num_vertices() == 3


def test_property_map_grows_to_the_bound_and_never_shrinks(gtc):
    g = gtc.Graph()
    g.add_vertex(2)
    p = g.new_vertex_property("double")
    assert p.allocated() == 0
    assert p[1] == 0.0          # a never-written key inside the bound reads as zero
    assert p.allocated() == 2
    p[0] = 3.5
    g.add_vertex(2)
    assert p[3] == 0.0 and p[0] == 3.5 and p.allocated() == 4
    with pytest.raises(IndexError):
        p[4]
    with pytest.raises(ValueError, match="Invalid property type"):
        g.new_vertex_property("float128")


def test_edge_map_uses_the_edge_bound(gtc):
    g = gtc.Graph()
    g.add_vertex(2)
    g.add_edges(np.array([0, 1, 1]), np.array([1, 0, 1]))
    w = g.new_edge_property("double")
    w[2] = 1.5
    assert w.allocated() == 3 and g.sum_property(w) == 1.5


def test_centrality_map_type_checks(gtc):
    g = gtc.Graph()
    g.add_vertex(2)
    g.add_edge(0, 1)
    with pytest.raises(ValueError):
        g.pagerank(g.new_vertex_property("int32_t"))
    with pytest.raises(ValueError):
        g.pagerank(g.new_vertex_property("double"), weight=g.new_vertex_property("double"))
    with pytest.raises(ValueError, match="grain"):
        g.pagerank(g.new_vertex_property("double"), grain=0)


def test_synth_generators_are_deterministic(gtc):
    from graph_tool import synth
    a = synth.erdos_renyi_sinks(n=500, m=3000)
    b = synth.erdos_renyi_sinks(n=500, m=3000)
    assert a[0] == b[0] and (a[1] == b[1]).all() and (a[2] == b[2]).all()
    n, src, tgt, sinks = a
    assert not np.isin(src, sinks).any()            # sinks lost every out-edge
    assert (src != tgt).all()                        # no self-loops
    assert len(set(zip(src.tolist(), tgt.tolist()))) == src.size  # no duplicates
    n, s, t = synth.rmat_cpu(10)
    assert len(set(zip(s.tolist(), t.tolist()))) == s.size


def test_graph_batch_rejects_bad_input(gtc):
    """The batch's inputs are checked before any device work: endpoints
    beyond their own graph, decreasing offsets, an empty batch."""
    import pytest as _pt
    with _pt.raises(ValueError):
        gtc.GraphBatch([(3, [0, 3], [1, 2])])          # 3 is not a vertex of a 3-vertex graph
    with _pt.raises(ValueError):
        gtc.GraphBatch([(2, [0], [1]), (2, [0], [5])])  # local indices: 5 >= 2
    with _pt.raises(ValueError):
        gtc.GraphBatch([])


def test_graph_batch_uncapped_needs_positive_epsilon(gtc):
    """max_iter 0 with epsilon <= 0 would never stop on the device: refused
    before any device work."""
    import ctypes as C
    from graph_tool import _ffi
    L = _ffi.lib()
    r = _ffi.Result()
    st = L.gtc_pagerank_batch_device(C.c_void_p(1), None, 0.85, 0.0, 0, None, None, None,
                                     C.byref(r))
    assert st == _ffi.GTC_ERR_ARG
    assert b"epsilon" in L.gtc_last_error()

"""The CPU oracle against the reference's own known answers.

Every case here is a test of graph-tool-rs (crates/gt-algo/tests/
u16_centrality.rs and crates/gt-core/src/adj/block.rs), transcribed; passing
them is what pins the oracle before it is trusted to check the GPU."""
import numpy as np
import pytest

import _cases as K


@pytest.fixture(scope="module")
def S(oracle):
    return K.OracleSolver(oracle)


@pytest.fixture(scope="module")
def thousand():
    from graph_tool import synth
    return synth.thousand()


@pytest.fixture(scope="module")
def eigen60():
    from graph_tool import synth
    return synth.eigen60()


def test_odd_sweep_pagerank(S):
    K.case_odd_sweep_pagerank(S)


def test_warm_start(S):
    K.case_warm_start(S)


def test_cycle_and_personalisation(S):
    K.case_cycle_and_pers(S)


def test_zero_weight_predecessor(S):
    K.case_zero_weight_predecessor(S)


def test_plan_must_cover(S):
    K.case_plan_must_cover(S)


def test_dense_thousand(S, thousand):
    K.case_dense_thousand(S, thousand)


def test_cycle7_eigen(S):
    K.case_cycle7_eigen(S)


def test_edgeless_eigen(S):
    K.case_edgeless_eigen(S)


def test_odd_sweep_eigen(S):
    K.case_odd_sweep_eigen(S)


def test_eigen60_equation(S, eigen60):
    K.case_eigen60(S, eigen60)


def test_push_swap_layout(S):
    K.case_push_swap(S)


def test_unity_is_the_general_path(S, thousand):
    K.case_unity_is_general(S, thousand)


# ---- u16_centrality.rs:215-291, 594-617: thread counts and the plan -------

def test_pagerank_bit_identical_across_thread_counts(oracle, thousand):
    n, src, tgt = thousand
    runs = [K.OracleSolver(oracle, t).pagerank(n, src, tgt, epsilon=1e-13, max_iter=10_000)
            for t in (1, 4, 16)]
    for r, it in runs[1:]:
        assert it == runs[0][1]
        assert r.tobytes() == runs[0][0].tobytes()


def test_the_plan_fixes_the_fold_order(oracle, thousand):
    n, src, tgt = thousand
    S = K.OracleSolver(oracle)
    fine, _ = S.pagerank(n, src, tgt, grain=16, epsilon=1e-13, max_iter=10_000)
    coarse, _ = S.pagerank(n, src, tgt, grain=1000, epsilon=1e-13, max_iter=10_000)
    assert np.max(np.abs(fine - coarse)) < 1e-14
    assert fine.tobytes() != coarse.tobytes()


def test_eigenvector_bit_identical_across_thread_counts(oracle, thousand):
    n, src, tgt = thousand
    runs = [K.OracleSolver(oracle, t).eigenvector(n, src, tgt, epsilon=1e-13, max_iter=10_000)
            for t in (1, 4, 16)]
    for x, eig, it in runs[1:]:
        assert it == runs[0][2] and eig == runs[0][1]
        assert x.tobytes() == runs[0][0].tobytes()


# ---- block.rs:380-520: removal layouts, reached through the graph ----------

def test_remove_out_fills_the_hole_then_promotes(oracle):
    # block of vertex 0: out (10,e0) (11,e1) (12,e2), in (20,e3) (21,e4)
    g = oracle.Graph(22)
    for s, t in [(0, 10), (0, 11), (0, 12), (20, 0), (21, 0)]:
        g.add_edge(s, t)
    g.remove_edge(0)
    oo, ot, oi, io, it, ii = g.export()
    assert list(zip(ot[oo[0]:oo[1]], oi[oo[0]:oo[1]])) == [(12, 2), (11, 1)]
    assert list(zip(it[io[0]:io[1]], ii[io[0]:io[1]])) == [(21, 4), (20, 3)]


def test_remove_in_swaps_with_the_block_back(oracle):
    # block of vertex 0: out (10,e0), in (20,e1) (21,e2) (22,e3); remove e1
    g = oracle.Graph(23)
    for s, t in [(0, 10), (20, 0), (21, 0), (22, 0)]:
        g.add_edge(s, t)
    g.remove_edge(1)
    oo, ot, oi, io, it, ii = g.export()
    assert list(zip(it[io[0]:io[1]], ii[io[0]:io[1]])) == [(22, 3), (21, 2)]
    assert list(zip(ot[oo[0]:oo[1]], oi[oo[0]:oo[1]])) == [(10, 0)]


def test_self_loop_removal_relocates_its_own_in_entry(oracle):
    g = oracle.Graph(1)
    g.add_edge(0, 0)
    g.add_edge(0, 0)
    g.remove_edge(0)
    oo, ot, oi, io, it, ii = g.export()
    assert list(oi[oo[0]:oo[1]]) == [1]
    assert list(ii[io[0]:io[1]]) == [1]


def test_freed_ids_are_reused_lifo(oracle):
    g = oracle.Graph(4)
    for s, t in [(0, 1), (1, 2), (2, 3), (3, 0)]:
        g.add_edge(s, t)
    g.remove_edge(1)
    g.remove_edge(2)
    assert g.add_edge(0, 2) == 2 and g.add_edge(0, 3) == 1
    assert g.edge_bound() == 4 and g.num_edges() == 4


def test_insert_in_appends(oracle):
    # block.rs: insert_out then two insert_in -> inc == [(2,e1), (3,e2)]
    g = oracle.Graph(4)
    g.add_edge(0, 1)
    g.add_edge(2, 0)
    g.add_edge(3, 0)
    oo, ot, oi, io, it, ii = g.export()
    assert list(zip(it[io[0]:io[1]], ii[io[0]:io[1]])) == [(2, 1), (3, 2)]


def test_bad_vertex_is_an_error(oracle):
    g = oracle.Graph(2)
    with pytest.raises(oracle.OracleError, match="no such vertex"):
        g.add_edge(0, 5)


# ---- betweenness (u16_centrality.rs:620-883) ------------------------------

def test_betweenness_matches_an_independent_brandes(S):
    K.case_betweenness_random(S)


def test_betweenness_on_a_path_is_the_closed_form(S):
    K.case_betweenness_path(S)


def test_betweenness_back_edge_into_an_earlier_source(S):
    K.case_betweenness_back_edge(S)


def test_betweenness_unreachable_vertices_contribute_nothing(S):
    K.case_betweenness_unreachable(S)


def test_betweenness_bit_identical_across_thread_counts(oracle):
    n, edges = K.ring_plus_chords()
    g = oracle.Graph(n)
    g.add_edge_arrays(*K.edges_of(edges))
    base = g.betweenness(threads=1)
    for t in (2, 4, 16):
        got = g.betweenness(threads=t)
        assert got[0].tobytes() == base[0].tobytes() and got[1].tobytes() == base[1].tobytes()

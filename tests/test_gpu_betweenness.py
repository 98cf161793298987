"""Betweenness on the GPU (gtc_betweenness) against the reference's own
betweenness tests (crates/gt-algo/tests/u16_centrality.rs:620-883) and the
CPU oracle's restatement of centrality.rs:499-689: the 100 random
multigraphs within 1e-9 of an independent Brandes, the path's closed form
and the unreachable case exactly, run-to-run bit identity, and the oracle on
larger graphs, reversed and filtered views."""
import numpy as np
import pytest

import _cases as K

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(gtc):
    return K.GpuSolver(gtc, "f64_exact")


def test_matches_an_independent_brandes(S):
    K.case_betweenness_random(S)


def test_path_closed_form(S):
    K.case_betweenness_path(S)


def test_back_edge_into_an_earlier_source(S):
    K.case_betweenness_back_edge(S)


def test_unreachable_vertices_contribute_nothing(S):
    K.case_betweenness_unreachable(S)


def test_overwrites_the_maps_it_is_given(gtc):
    g = gtc.Graph()
    g.add_vertex(4)
    g.add_edges([0, 1, 2], [1, 2, 3])
    vb, eb = g.betweenness()
    first = (vb.a.copy(), eb.a.copy())
    g.betweenness(vb, eb)
    assert np.array_equal(vb.a, first[0]) and np.array_equal(eb.a, first[1])


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1.0)


def test_ring_with_chords_against_the_oracle_and_run_to_run(oracle, S):
    n, edges = K.ring_plus_chords()
    src, tgt = K.edges_of(edges)
    og = oracle.Graph(n)
    og.add_edge_arrays(src, tgt)
    for undirected in (False, True):
        wv, we = og.betweenness(undirected=undirected)
        gv, ge = S.betweenness(n, src, tgt, undirected=undirected)
        assert _rel(gv, wv) < 1e-12 and _rel(ge, we) < 1e-12
        hv, he = S.betweenness(n, src, tgt, undirected=undirected)
        assert gv.tobytes() == hv.tobytes() and ge.tobytes() == he.tobytes()


@pytest.mark.parametrize("seed", [1, 2])
def test_rmat_reversed_and_filtered_views(oracle, S, seed):
    from graph_tool import synth
    n, src, tgt = synth.rmat_cpu(10, edge_factor=8, seed=seed)
    og = oracle.Graph(n)
    og.add_edge_arrays(src, tgt)
    rng = np.random.default_rng(seed)
    vm = (rng.random(n) < 0.8).astype(np.uint8)
    em = (rng.random(len(src)) < 0.9).astype(np.uint8)
    for kw in (dict(), dict(reversed=True), dict(vmask=vm, emask=em),
               dict(undirected=True, vmask=vm)):
        wv, we = og.betweenness(**kw)
        gv, ge = S.betweenness(n, src, tgt, **kw)
        assert _rel(gv, wv) < 1e-12, kw
        assert _rel(ge, we) < 1e-12, kw
        if "vmask" in kw:
            assert np.all(gv[vm == 0] == 0.0)

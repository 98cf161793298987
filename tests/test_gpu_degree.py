"""gtc_weighted_degree against the reference's degree selectors
(crates/gt-algo/src/degree.rs:68-82, 122-160): the FP64 left fold from 0.0
of the weights over each vertex's out-half (in-half) in storage order, taken
here from the oracle's blocks, compared bit for bit -- with weights spread
over sixteen orders of magnitude, so any other summation order would show."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _folds(oracle, n, src, tgt, w, vmask=None, emask=None):
    og = oracle.Graph(n)
    og.add_edge_arrays(src, tgt)
    oo, ot, oi, io, it, ii = og.export()
    out = np.zeros(n)
    inn = np.zeros(n)
    keep_v = (lambda v: True) if vmask is None else (lambda v: bool(vmask[v]))
    keep_e = (lambda e: True) if emask is None else (lambda e: bool(emask[e]))
    for v in range(n):
        if not keep_v(v):
            continue
        for half, off, other, idx in ((out, oo, ot, oi), (inn, io, it, ii)):
            acc = 0.0
            for p in range(int(off[v]), int(off[v + 1])):
                if keep_e(int(idx[p])) and keep_v(int(other[p])):
                    acc = acc + (1.0 if w is None else float(w[idx[p]]))
            half[v] = acc
    return out, inn


@pytest.fixture(scope="module")
def graph():
    rng = np.random.default_rng(11)
    n, m = 300, 6000
    src = rng.integers(0, n, m).astype(np.uint32)
    tgt = rng.integers(0, n, m).astype(np.uint32)
    hub = rng.random(m) < 0.3
    src[hub & (rng.random(m) < 0.5)] = 0
    w = 10.0 ** rng.uniform(-8, 8, m)
    w[rng.random(m) < 0.05] = 0.0
    return n, src, tgt, w


def _gpu(gtc, n, src, tgt):
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    return g


def test_out_and_in_folds_are_bit_identical(oracle, gtc, graph):
    n, src, tgt, w = graph
    want_out, want_in = _folds(oracle, n, src, tgt, w)
    g = _gpu(gtc, n, src, tgt)
    got_out = g.weighted_degree(w, "out").a
    got_in = g.weighted_degree(w, "in").a
    assert got_out.tobytes() == want_out.tobytes()
    assert got_in.tobytes() == want_in.tobytes()
    # the reversed view swaps the halves
    assert g.weighted_degree(w, "out", reversed=True).a.tobytes() == want_in.tobytes()


def test_unity_is_the_degree(oracle, gtc, graph):
    n, src, tgt, _ = graph
    g = _gpu(gtc, n, src, tgt)
    assert np.array_equal(g.weighted_degree(None, "out").a, np.bincount(src, minlength=n))
    assert np.array_equal(g.weighted_degree(None, "in").a, np.bincount(tgt, minlength=n))


def test_filtered_view(oracle, gtc, graph):
    n, src, tgt, w = graph
    rng = np.random.default_rng(12)
    vm = (rng.random(n) < 0.7).astype(np.uint8)
    em = (rng.random(len(src)) < 0.8).astype(np.uint8)
    want_out, want_in = _folds(oracle, n, src, tgt, w, vm, em)
    g = _gpu(gtc, n, src, tgt)
    assert g.weighted_degree(w, "out", vfilt=vm, efilt=em).a.tobytes() == want_out.tobytes()
    assert g.weighted_degree(w, "in", vfilt=vm, efilt=em).a.tobytes() == want_in.tobytes()


def test_thousand_fixture(oracle, gtc):
    # the reference tests' fixed 1,000-vertex graph, weights U(0.1, 1)
    from graph_tool import synth
    n, src, tgt = synth.thousand()
    w = np.random.default_rng(3).uniform(0.1, 1.0, len(src))
    want_out, _ = _folds(oracle, n, src, tgt, w)
    assert _gpu(gtc, n, src, tgt).weighted_degree(w).a.tobytes() == want_out.tobytes()

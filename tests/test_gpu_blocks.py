"""gtc_graph_create_blocks: a graph handed over as the reference's blocks,
after removals and edge-id reuse.

The oracle replays a history of add_edge, remove_edge (the swap-remove of
crates/gt-core/src/adj/block.rs:241-291) and add_edge again (ids taken back
from the LIFO free list, crates/gt-core/src/adj/alloc.rs:58-90), so its
blocks are no add_edge replay of any edge list and its edge-id space has
holes.  Those blocks go through the C ABI as stored; the handle's blocks,
the FP64-exact PageRank and eigenvector (values, eigenvalue and sweep
counts) must then equal the oracle's bit for bit, and the FP32 solves must
be within 1e-6 relative L1."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _history(O, n, rounds, seed):
    rng = np.random.default_rng(seed)
    g = O.Graph(n)
    live = []
    for _ in range(rounds):
        k = int(rng.integers(n, 4 * n))
        s = rng.integers(0, n, k).astype(np.uint32)
        t = rng.integers(0, n, k).astype(np.uint32)
        t[: k // 10] = 3  # a hub with a long in-half
        for a, b in zip(s.tolist(), t.tolist()):
            live.append(g.add_edge(a, b))
        drop = rng.choice(len(live), len(live) // 3, replace=False)
        for j in sorted(drop.tolist(), reverse=True):
            g.remove_edge(live[j])
            live.pop(j)
    assert g.edge_bound() > g.num_edges()  # holes in the id space
    return g


def _blocks(og):
    """The oracle's blocks as the reference stores them: per vertex the
    out-half then the in-half, entries (other, idx)."""
    oo, ot, oi, io, it, ii = og.export()
    n = og.n
    oo, io = oo.astype(np.int64), io.astype(np.int64)
    out_len = np.diff(oo)
    in_len = np.diff(io)
    block_off = np.zeros(n + 1, np.uint64)
    block_off[1:] = np.cumsum(out_len + in_len)
    bo = block_off[:-1].astype(np.int64)
    ent = np.zeros((int(block_off[-1]), 2), np.uint32)
    vo = np.repeat(np.arange(n), out_len)
    po = bo[vo] + (np.arange(oo[-1]) - oo[vo])
    ent[po, 0], ent[po, 1] = ot, oi
    vi = np.repeat(np.arange(n), in_len)
    pi = bo[vi] + out_len[vi] + (np.arange(io[-1]) - io[vi])
    ent[pi, 0], ent[pi, 1] = it, ii
    return block_off, out_len.astype(np.uint32), ent


@pytest.fixture(scope="module")
def pair(oracle):
    og = _history(oracle, 3000, 3, 17)
    return og, _blocks(og)


def _graph(gtc, og, blk):
    return gtc.Graph.from_blocks(og.n, og.edge_bound(), *blk)


def test_blocks_round_trip(oracle, gtc, pair):
    og, blk = pair
    g = _graph(gtc, og, blk)
    assert g.num_edges() == og.num_edges() and g.edge_index_range() == og.edge_bound()
    for a, b in zip(g.blocks(), og.export()):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("kind", ["plain", "weighted", "reversed"])
def test_exact_solves_bit_identical(oracle, gtc, pair, kind):
    og, blk = pair
    g = _graph(gtc, og, blk)
    rng = np.random.default_rng(5)
    w = rng.uniform(0.1, 1.0, og.edge_bound()) if kind == "weighted" else None
    rev = kind == "reversed"
    wm = None
    if w is not None:
        wm = g.new_edge_property("double")
        wm.a[:] = w
    r = g.new_vertex_property("double")
    res = g.pagerank(r, weight=wm, epsilon=1e-12, max_iter=500, grain=256, reversed=rev,
                     precision="f64_exact", result=True)
    want, it = og.pagerank(weight=w, epsilon=1e-12, max_iter=500, grain=256, reversed=rev)
    assert int(res.iterations) == it
    assert r.a.tobytes() == want.tobytes()
    x = g.new_vertex_property("double")
    res = g.eigenvector(x, weight=wm, epsilon=1e-12, max_iter=300, grain=256, reversed=rev,
                        precision="f64_exact", result=True)
    wantx, eig, itx = og.eigenvector(weight=w, epsilon=1e-12, max_iter=300, grain=256,
                                     reversed=rev)
    assert int(res.iterations) == itx and float(res.eigenvalue) == eig
    assert x.a.tobytes() == wantx.tobytes()


def test_f32_pagerank_within_tolerance(oracle, gtc, pair):
    og, blk = pair
    g = _graph(gtc, og, blk)
    w = np.random.default_rng(6).uniform(0.1, 1.0, og.edge_bound())
    wm = g.new_edge_property("double")
    wm.a[:] = w
    r = g.new_vertex_property("double")
    it = g.pagerank(r, weight=wm, epsilon=1e-7, max_iter=1000)
    want, iw = og.pagerank(weight=w, epsilon=1e-7, max_iter=1000, grain=4096)
    err = float(np.abs(r.a - want).sum() / np.abs(want).sum())
    assert err < 1e-6, err
    assert abs(it - iw) <= 2


def test_inconsistent_blocks_are_refused(oracle, gtc, pair):
    og, (bo, ol, ent) = pair
    bad = ent.copy()
    k = int(bo[5]) + int(ol[5])  # first in-entry of some vertex with one
    while k >= int(bo[6]):
        k = int(bo[7]) + int(ol[7])
    bad[k, 0] = (bad[k, 0] + 1) % og.n  # an in-entry whose source disagrees
    with pytest.raises(ValueError):
        gtc.Graph.from_blocks(og.n, og.edge_bound(), bo, ol, bad)
    bad = ent.copy()
    bad[0, 1] = og.edge_bound()  # an id beyond the edge bound
    with pytest.raises(IndexError):
        gtc.Graph.from_blocks(og.n, og.edge_bound(), bo, ol, bad)

"""The .gt reader on the GPU: documents written by the oracle's restatement of
the reference's writer (crates/gt-io/src/gt.rs:865-940) are read by
gtc_gt_graph, which decodes the lists on the device and replays add_edge in
file order.  Every block must equal the oracle's blocks for the edge list the
reference's reader (gt.rs:628-678) produces, byte for byte, and a PageRank
weighted by the document's edge column must equal the oracle's bit for bit."""
import numpy as np
import pytest

import _cases as K
import gt_format as G

pytestmark = pytest.mark.gpu


def _doc(n, m, seed, big=False, weighted=True, directed=True):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, m)
    tgt = rng.integers(0, n, m)
    if n > 1:  # a hub with interleaved in- and out-edges and self-loops
        hub = rng.random(m) < 0.2
        side = rng.random(m) < 0.5
        src[hub & side] = 0
        tgt[hub & ~side] = 0
    edges = list(zip(src.tolist(), tgt.tolist()))
    props = []
    if weighted:
        props.append(("weight", G.EDGE, 4, (0.1 + 0.9 * rng.random(m)).tolist()))
    props.append(("label", G.VERTEX, 6, [f"v{i}" for i in range(n)]))
    return G.write(n, edges, directed, props, big_endian=big)


def _blocks_equal(oracle, g, n, src, tgt):
    want = K.OracleSolver(oracle).blocks(n, np.asarray(src, np.uint32), np.asarray(tgt, np.uint32))
    got = g.blocks()
    for name, a, b in zip(["out_off", "out_other", "out_idx", "in_off", "in_other", "in_idx"],
                          want, got):
        a = np.asarray(a, np.uint64)
        b = np.asarray(b, np.uint64)
        assert a.shape == b.shape, (name, a.shape, b.shape)
        assert np.array_equal(a, b), name


@pytest.mark.parametrize("n,m,big", [(40, 300, False), (40, 300, True), (300, 4000, False),
                                     (70_000, 250_000, True)])
def test_blocks_match_the_reference_reader(oracle, gtc, n, m, big):
    b = _doc(n, m, seed=n + m, big=big)
    d = G.read(b)
    g = gtc.load_graph(b)
    assert (g.num_vertices(), g.num_edges()) == (d["n"], len(d["src"]))
    _blocks_equal(oracle, g, d["n"], d["src"], d["tgt"])
    assert g.vp["label"][:3] == ["v0", "v1", "v2"]


def test_weighted_pagerank_from_the_document(oracle, gtc):
    b = _doc(500, 6000, seed=9)
    d = G.read(b)
    g = gtc.load_graph(b)
    w = g.ep["weight"]
    col = np.asarray({p[0]: p[3] for p in d["props"]}["weight"])
    assert np.array_equal(w.a, col)
    og = oracle.Graph(d["n"])
    og.add_edge_arrays(np.asarray(d["src"], np.uint32), np.asarray(d["tgt"], np.uint32))
    want, iw = og.pagerank(weight=col, epsilon=1e-10, max_iter=1000, grain=64)
    r = g.new_vertex_property("double")
    it = g.pagerank(r, weight=w, epsilon=1e-10, max_iter=1000, grain=64, precision="f64_exact")
    assert it == iw and r.a.tobytes() == want.tobytes()
    r32 = g.new_vertex_property("double")
    g.pagerank(r32, weight=w, epsilon=1e-7, max_iter=1000, grain=64)
    assert np.abs(r32.a - want).sum() / np.abs(want).sum() < 1e-6


def test_first_out_of_range_index_in_file_order(gtc):
    # two bad entries; the error names the first one of the file
    b = bytearray(G.write(300, [(0, 5), (2, 7), (2, 9)], True))
    raw = bytes(b)
    # n = 300: 2-byte indices; vertex 2's list holds 7 then 9
    hdr = 6 + 1 + 1 + 8 + int.from_bytes(raw[8:16], "little") + 1 + 8
    v0 = hdr + 8                 # vertex 0's single entry
    v2 = hdr + 8 + 2 + 8 + 8     # vertex 2's first entry (vertex 1 is empty)
    assert int.from_bytes(raw[v0:v0 + 2], "little") == 5
    assert int.from_bytes(raw[v2:v2 + 2], "little") == 7
    b[v2 + 2:v2 + 4] = (300).to_bytes(2, "little")
    b[v2:v2 + 2] = (301).to_bytes(2, "little")
    with pytest.raises(IndexError) as e:
        gtc.load_graph(bytes(b))
    assert "vertex index 301 is out of range (bound 300)" in str(e.value)


def test_edges_come_back_in_file_order_and_the_graph_stays_mutable(oracle, gtc):
    b = _doc(60, 500, seed=4, weighted=False, directed=False)
    d = G.read(b)
    g = gtc.load_graph(b)
    assert g.directed is False
    src, tgt = g.edges()
    assert src.tolist() == d["src"] and tgt.tolist() == d["tgt"]
    e = g.add_edge(3, 4)  # the handle is rebuilt with the file's edges first
    assert e == len(d["src"])
    _blocks_equal(oracle, g, 60, d["src"] + [3], d["tgt"] + [4])


def test_empty_and_edgeless_documents(gtc):
    g = gtc.load_graph(G.write(0, [], True))
    assert (g.num_vertices(), g.num_edges()) == (0, 0)
    g = gtc.load_graph(G.write(5, [], True))
    assert (g.num_vertices(), g.num_edges()) == (5, 0)
    r = g.new_vertex_property("double")
    g.pagerank(r, epsilon=1e-9, max_iter=100)
    assert np.allclose(r.a, 0.2)

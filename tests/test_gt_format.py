"""The .gt reader without a GPU: the oracle's restatement of the reference's
reader against the facts the reference's own tests assert
(crates/gt-io/tests/u27_gt.rs), and the library's host-side parser
(gtc_gt_open and the property accessors, no device involved) against the
oracle, on the reference's two data files and on documents of every value
kind in both byte orders.  Malformed input is refused, never read past
(u27_gt.rs:713-894)."""
import os
import struct

import numpy as np
import pytest

import gt_format as G

# The reference's own test documents (crates/gt-io/tests/data/{karate,lesmis}.gt),
# kept as fixtures beside the other reference-held vectors.
DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
needs_ref = pytest.mark.skipif(not os.path.exists(os.path.join(DATA, "karate.gt")),
                               reason="the reference's .gt fixtures are missing")


def _fixture(name):
    with open(os.path.join(DATA, name), "rb") as fh:
        return fh.read()


def _same(a, b):
    if hasattr(a, "dtype") or hasattr(b, "dtype"):
        return np.array_equal(np.asarray(a), np.asarray(b))
    if isinstance(a, list) and isinstance(b, list):
        return len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))
    return a == b


def _all_kinds_doc(n=5, big=False, seed=0):
    """A directed multigraph with self-loops and one column of every kind."""
    rng = np.random.default_rng(seed)
    m = 3 * n + 2
    edges = [(int(rng.integers(n)), int(rng.integers(n))) for _ in range(m)]
    edges[0] = (n - 1, n - 1)

    def col(kind, k):
        out = []
        for i in range(k):
            if kind == 0:
                out.append(i % 2)
            elif kind == 1:
                out.append(-3 * (i % 10000))
            elif kind == 2:
                out.append(-70000 * (i % 30000))
            elif kind == 3:
                out.append(-(1 << 40) * i - 7)
            elif kind == 4:
                out.append(0.1 * i - 2.5)
            elif kind == 5:
                out.append(bytes((i + j) % 256 for j in range(16)))
            elif kind == 6:
                out.append(f"v{i}é")
            elif kind == 7:
                out.append(bytes([1, 0, 1][: i % 4]))
            elif kind in (8, 9, 10):
                out.append([i % 9000, -(i % 9000), 2 * (i % 9000)][: i % 4])
            elif kind == 11:
                out.append([0.5 * i] * (i % 3))
            elif kind == 12:
                out.append([bytes([i % 256] * 16)] * (i % 3))
            elif kind == 13:
                out.append(["a", "βγ", ""][: i % 4])
            else:
                out.append(b"\x80\x05pickled" + bytes([i % 256]))
        return out

    props = [("g_" + str(k), G.GRAPH, k, col(k, 1)) for k in range(15)]
    props += [("v_" + str(k), G.VERTEX, k, col(k, n)) for k in range(15)]
    props += [("e_" + str(k), G.EDGE, k, col(k, m)) for k in range(15)]
    return G.write(n, edges, True, props, big_endian=big), n, edges, props


# ---- the oracle against the reference's own assertions ----------------------

@needs_ref
def test_oracle_reads_karate_as_the_reference_asserts():
    # u27_gt.rs:469-503
    b = _fixture("karate.gt")
    d = G.read(b)
    assert (d["n"], len(d["src"]), d["directed"]) == (34, 78, False)
    assert "34 vertices, 78 edges, undirected" in d["comment"]
    by = {p[0]: p for p in d["props"]}
    assert sorted(by) == ["description", "pos", "readme"]
    assert G.KINDS[by["description"][2]] == "string" and by["description"][1] == G.GRAPH
    assert by["readme"][1] == G.GRAPH
    assert G.KINDS[by["pos"][2]] == "vector<double>" and by["pos"][1] == G.VERTEX
    assert len(by["pos"][3]) == 34
    assert d["src"].count(0) + d["tgt"].count(0) == 16  # the instructor's degree
    edges = list(zip(d["src"], d["tgt"]))
    assert G.write(d["n"], edges, d["directed"], d["props"], d["comment"]) == b


@needs_ref
def test_oracle_reads_lesmis_as_the_reference_asserts():
    # u27_gt.rs:506-590
    b = _fixture("lesmis.gt")
    d = G.read(b)
    assert (d["n"], len(d["src"]), d["directed"]) == (77, 254, False)
    assert [(p[0], p[1], G.KINDS[p[2]]) for p in d["props"]] == [
        ("description", G.GRAPH, "string"), ("readme", G.GRAPH, "string"),
        ("label", G.VERTEX, "string"), ("pos", G.VERTEX, "vector<double>"),
        ("value", G.EDGE, "double")]
    assert len(d["props"][4][3]) == 254
    labels = d["props"][2][3]
    assert labels[0] == "Myriel" and "Valjean" in labels
    # the first list entry is Napoleon(1) -> Myriel(0), weight 1; vertex 0
    # has no out-edges and 10 in-edges
    assert (d["src"][0], d["tgt"][0], d["props"][4][3][0]) == (1, 0, 1.0)
    assert d["src"].count(0) == 0 and d["tgt"].count(0) == 10
    edges = list(zip(d["src"], d["tgt"]))
    assert G.write(d["n"], edges, d["directed"], d["props"], d["comment"]) == b


# ---- the library's host parser against the oracle ---------------------------

def _check_library_against_oracle(gtc, b):
    from graph_tool import gt as L
    d = G.read(b)
    f = L.GtFile(b)
    assert (f.n, f.m, f.directed, f.big_endian) == (d["n"], len(d["src"]), d["directed"],
                                                    d["big_endian"])
    assert f.comment() == d["comment"]
    props = f.properties()
    assert [(p[0], p[1], p[2]) for p in props] == [(p[0], p[1], p[2]) for p in d["props"]]
    for i, p in enumerate(d["props"]):
        assert props[i][3] == len(p[3])
        assert _same(list(f.values(i)), p[3]), p[0]


@needs_ref
@pytest.mark.parametrize("name", ["karate.gt", "lesmis.gt"])
def test_library_parses_the_reference_files(gtc, name):
    _check_library_against_oracle(gtc, _fixture(name))


@pytest.mark.parametrize("big", [False, True])
def test_four_byte_indices(gtc, big):
    # N > 65535: the lists use 4-byte indices (vint_width, gt.rs:689-699)
    n = 70_000
    rng = np.random.default_rng(3)
    src = rng.integers(0, n, 20_000)
    tgt = rng.integers(0, n, 20_000)
    edges = list(zip(src.tolist(), tgt.tolist()))
    props = [("w", G.EDGE, 4, (0.1 + rng.random(len(edges))).tolist()),
             ("deg", G.VERTEX, 2, rng.integers(-5, 5, n).tolist())]
    b = G.write(n, edges, True, props, big_endian=big)
    _check_library_against_oracle(gtc, b)


@pytest.mark.parametrize("big", [False, True])
@pytest.mark.parametrize("n", [5, 300])
def test_library_parses_every_kind_in_both_byte_orders(gtc, n, big):
    b, _, edges, props = _all_kinds_doc(n, big)
    d = G.read(b)
    # the oracle round trip: the file lists edges vertex by vertex (edge-id
    # order inside a vertex), and reading numbers them in that order
    order = sorted(range(len(edges)), key=lambda k: (edges[k][0], k))
    want = [p[3] if p[1] != G.EDGE else [p[3][k] for k in order] for p in props]
    assert [p[3] for p in d["props"]] == want
    assert list(zip(d["src"], d["tgt"])) == [edges[k] for k in order]
    _check_library_against_oracle(gtc, b)


@pytest.mark.parametrize("n,width", [(1, 1), (255, 1), (256, 2), (65_535, 2), (65_536, 4)])
def test_the_index_width_switches_at_the_boundaries(gtc, n, width):
    # u27_gt.rs:250-286: the narrowest unsigned width holding N (N <= 255 is
    # one byte); one edge 0 -> n-1
    from graph_tool import gt as L
    b = G.write(n, [(0, n - 1)], True)
    clen = struct.unpack("<Q", b[8:16])[0]
    lst = 16 + clen + 1 + 8
    assert struct.unpack("<Q", b[lst:lst + 8])[0] == 1
    assert int.from_bytes(b[lst + 8:lst + 8 + width], "little") == n - 1
    assert len(b) == lst + 8 + width + 8 * (n - 1) + 8  # the other lists are empty, then nprops
    f = L.GtFile(b)
    assert (f.n, f.m) == (n, 1)
    d = G.read(b)
    assert (d["src"], d["tgt"]) == ([0], [n - 1])


def test_empty_and_edgeless_documents_with_a_graph_property(gtc):
    # u27_gt.rs:1072-1102
    from graph_tool import gt as L
    f = L.GtFile(G.write(0, [], False))
    assert (f.n, f.m, f.directed, f.nprops) == (0, 0, False, 0)
    f = L.GtFile(G.write(4, [], True, [("name", G.GRAPH, 6, ["four dots"])]))
    assert (f.n, f.m, f.nprops) == (4, 0, 1)
    assert f.properties() == [("name", G.GRAPH, 6, 1)]
    assert f.values(0) == ["four dots"]


def test_an_undirected_document_lists_each_edge_once(gtc):
    # u27_gt.rs:1104-1120: the flag is metadata; the lists are the directed
    # adjacency, one entry per edge
    from graph_tool import gt as L
    f = L.GtFile(G.write(2, [(0, 1)], False))
    assert (f.n, f.m, f.directed) == (2, 1, False)


@needs_ref
def test_the_edge_column_of_lesmis_stays_with_its_edge(gtc):
    # u27_gt.rs:547-590: the first list entry is 1 -> 0 with weight 1; the
    # column is keyed by edge id, which is file order
    from graph_tool import gt as L
    f = L.GtFile(_fixture("lesmis.gt"))
    names = [p[0] for p in f.properties()]
    w = f.values(names.index("value"))
    assert w.dtype == np.float64 and w.size == 254 and w[0] == 1.0
    d = G.read(_fixture("lesmis.gt"))
    assert np.array_equal(w, np.asarray(d["props"][4][3]))


def test_big_endian_twin_reads_the_same(gtc):
    from graph_tool import gt as L
    le, *_ = _all_kinds_doc(7, False)
    be, *_ = _all_kinds_doc(7, True)
    assert le != be
    a, b = L.GtFile(le), L.GtFile(be)
    for i in range(a.nprops):
        assert _same(list(a.values(i)), list(b.values(i)))


def test_numeric_columns_as_doubles(gtc):
    from graph_tool import _ffi
    from graph_tool import gt as L
    b, n, edges, props = _all_kinds_doc(9)
    d = G.read(b)
    f = L.GtFile(b)
    for i, (name, dom, kind, count) in enumerate(f.properties()):
        out = np.zeros(max(count, 1))
        st = _ffi.lib().gtc_gt_property_f64(f._h, i, out.ctypes.data_as(_ffi.f64p), out.size)
        if kind <= 4:
            _ffi.check(st)
            assert np.array_equal(out[:count], np.asarray(d["props"][i][3], np.float64)), name
        else:
            assert st == _ffi.GTC_ERR_ARG
    short = np.zeros(1)
    vi = [p[0] for p in f.properties()].index("v_4")
    assert _ffi.lib().gtc_gt_property_f64(f._h, vi, short.ctypes.data_as(_ffi.f64p), 1) \
        == _ffi.GTC_ERR_ARG


# ---- malformed input --------------------------------------------------------

def _refused(b):
    from graph_tool import gt as L
    with pytest.raises(ValueError) as e:
        L.GtFile(b)
    return str(e.value)


def test_every_truncation_is_refused(gtc):
    # u27_gt.rs:713-742: every prefix is a bad magic or a parse error
    b, *_ = _all_kinds_doc(4)
    for cut in range(len(b)):
        msg = _refused(b[:cut])
        if cut < 6:
            assert "bad magic" in msg
        else:
            assert "at byte" in msg, (cut, msg)
        with pytest.raises(G.GtError) as e:
            G.read(b[:cut])
        assert e.value.kind == ("BadMagic" if cut < 6 else "Parse")


@needs_ref
def test_every_truncation_of_the_reference_files_is_refused(gtc):
    for name in ("karate.gt", "lesmis.gt"):
        b = _fixture(name)
        for cut in range(0, len(b), 7):
            _refused(b[:cut])


def test_foreign_empty_and_future_documents(gtc):
    assert "bad magic" in _refused(b'<?xml version="1.0"?>')
    assert "bad magic" in _refused(b"")
    b = bytearray(G.write(2, [], True))
    b[6] = 2
    assert "version 2" in _refused(bytes(b))


def test_unknown_value_type_and_domain(gtc):
    # u27_gt.rs:799-840
    b = G.write(2, [], True, [("p", G.VERTEX, 3, [1, 2])])
    at = len(b) - 2 * 8 - 1
    assert b[at] == 3
    for bad in (15, 16, 200, 255):
        x = bytearray(b)
        x[at] = bad
        assert f"value type index {bad}" in _refused(bytes(x))
    x = bytearray(b)
    dom_at = len(b) - 2 * 8 - 1 - 1 - 8 - 1
    assert x[dom_at] == G.VERTEX
    x[dom_at] = 3
    assert "invalid property domain 3" in _refused(bytes(x))


def test_non_utf8_strings_are_refused(gtc):
    b = G.write(1, [], True, [("s", G.VERTEX, 6, ["ok"])])
    x = bytearray(b)
    x[-2:] = b"\xff\xfe"
    assert "not UTF-8" in _refused(bytes(x))
    with pytest.raises(G.GtError) as e:
        G.read(bytes(x))
    assert e.value.kind == "MalformedProperty"
    # a property name that is not UTF-8 is a parse error
    b = G.write(1, [], True, [("nm", G.VERTEX, 0, [1])])
    x = bytearray(b)
    i = x.rindex(b"nm")
    x[i:i + 2] = b"\xc3\x28"
    assert "not valid UTF-8" in _refused(bytes(x))


def test_absurd_declared_lengths_do_not_allocate(gtc):
    # u27_gt.rs:863-894: a count near 2^64 is truncation, not an allocation
    b = bytearray(G.write(3, [(0, 1)], True))
    hdr = 6 + 1 + 1 + 8 + struct.unpack("<Q", b[8:16])[0]
    first_count = hdr + 1 + 8
    b[first_count:first_count + 8] = struct.pack("<Q", (1 << 64) - 1)
    assert "unexpected end of file" in _refused(bytes(b))
    b = bytearray(G.write(1, [], True, [("s", G.GRAPH, 6, ["x"])]))
    b[-9:-1] = struct.pack("<Q", (1 << 63))
    assert "declares" in _refused(bytes(b))


def test_an_absurd_vertex_count_is_refused_before_anything_is_sized(gtc):
    # u27_gt.rs:876-885: N = 2^40 is past the index space; N = 2^32 - 1 is
    # inside it but the document cannot hold that many records
    for n in ((1 << 40), (1 << 32) - 1):
        b = bytearray(G.MAGIC) + bytes([G.VERSION, 0]) + struct.pack("<Q", 0) + bytes([1])
        b += struct.pack("<Q", n)
        msg = _refused(bytes(b))
        assert "index space" in msg or "unexpected end of file" in msg, msg
        with pytest.raises(G.GtError) as e:
            G.read(bytes(b))
        assert e.value.kind in ("Parse", "IndexWidthExceeded")


def test_a_vector_count_that_would_wrap_is_refused(gtc):
    # a vector<double> value declaring 2^61 + 1 elements: 8 x that count wraps
    # around 2^64 to 8, which must not pass for a short remainder
    b = bytearray(G.write(1, [], True, [("v", G.VERTEX, 11, [[1.5]])]))
    at = len(b) - 8 - 8  # the element count, then the one element
    assert struct.unpack("<Q", b[at:at + 8])[0] == 1
    b[at:at + 8] = struct.pack("<Q", (1 << 61) + 1)
    assert "unexpected end of file" in _refused(bytes(b))


def test_out_of_range_index_is_left_to_the_device_check(gtc):
    # the framing is sound, so the host parse accepts it; gtc_gt_graph (on
    # the GPU) refuses the index -- the oracle refuses it while reading
    b = bytearray(G.write(3, [(0, 2)], True))
    idx = len(b) - 8 - 8 - 8 - 1  # vertex 0's single index (1 byte): before 2 empty lists
    assert b[idx] == 2
    b[idx] = 3
    from graph_tool import gt as L
    assert L.GtFile(bytes(b)).m == 1
    with pytest.raises(G.GtError) as e:
        G.read(bytes(b))
    assert e.value.kind == "IndexOutOfRange"

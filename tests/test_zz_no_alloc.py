"""gtc_pagerank_noalloc: PageRank for callers that cannot allocate device
memory while it runs (a runtime that reserved all GPU memory up front, or a
path where an allocation would stall).  It keeps its intermediate vectors in
a static device array inside the library, so this test hands it the graph
and the output only, and checks it against the ordinary entry point
(gtc_pagerank, FP32) to the FP32 tolerance the other tests use, on two calls
in a row: the second call starts from the contents the first one left in
the shared array.

Collected last on purpose (test_zz_*): a failure here stops a -x run only
after every other test has run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_pagerank_matches_the_allocating_entry_point(gtc):
    import torch

    from graph_tool import _ffi, synth

    n, src, tgt = synth.rmat_cpu(14, edge_factor=12, seed=5)
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    want = g.new_vertex_property("double")
    iw = g.pagerank(want, epsilon=1e-7, max_iter=1000)
    want = want.a.copy()

    # the graph as a caller would pass it: the in-halves (pull order) and
    # the out-degrees, in device memory owned by the caller
    oo, ot, oi, io, it, ii = g.blocks()
    dev = torch.device("cuda", 0)
    d_off = torch.from_numpy(io.astype(np.int64).astype(np.int32)).to(dev)
    d_src = torch.from_numpy(it.astype(np.int64).astype(np.int32)).to(dev)
    d_deg = torch.from_numpy(np.diff(oo).astype(np.int64).astype(np.int32)).to(dev)
    d_rank = torch.full((n,), -1.0, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    L = _ffi.lib()
    results = []
    for _ in range(2):
        iters = C.c_uint64(0)
        st = L.gtc_pagerank_noalloc(n, d_off.data_ptr(), d_src.data_ptr(), d_deg.data_ptr(), 0.85,
                                    1e-7, 1000, d_rank.data_ptr(), C.byref(iters), None)
        _ffi.check(st)
        got = d_rank.double().cpu().numpy()
        rel_l1 = np.abs(got - want).sum() / np.abs(want).sum()
        assert rel_l1 < 1e-6, rel_l1
        assert abs(int(iters.value) - iw) <= 2, (iters.value, iw)
        results.append(got)
        d_rank.fill_(-1.0)  # the second call must produce the result again
    assert np.array_equal(results[0], results[1])


def test_noalloc_rejects_a_graph_beyond_its_limit(gtc):
    from graph_tool import _ffi
    L = _ffi.lib()
    st = L.gtc_pagerank_noalloc((1 << 20) + 1, None, None, None, 0.85, 1e-6, 10, None, None, None)
    assert st == _ffi.GTC_ERR_ARG
    assert b"limit" in L.gtc_last_error()


def test_noalloc_odd_and_even_sweep_counts(gtc):
    """After an even number of sweeps the result is already in the caller's
    buffer; after an odd number it is copied back from the static array.
    Both returns are checked against the allocating entry point capped at
    the same sweep count."""
    import torch

    from graph_tool import _ffi, synth

    n, src, tgt = synth.rmat_cpu(12, edge_factor=8, seed=9)
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    oo, ot, oi, io, it, ii = g.blocks()
    dev = torch.device("cuda", 0)
    d_off = torch.from_numpy(io.astype(np.int64).astype(np.int32)).to(dev)
    d_src = torch.from_numpy(it.astype(np.int64).astype(np.int32)).to(dev)
    d_deg = torch.from_numpy(np.diff(oo).astype(np.int64).astype(np.int32)).to(dev)
    d_rank = torch.full((n,), -1.0, dtype=torch.float32, device=dev)
    L = _ffi.lib()
    for cap in (1, 2, 3, 4):
        want = g.new_vertex_property("double")
        assert g.pagerank(want, epsilon=1e-12, max_iter=cap) == cap
        d_rank.fill_(-1.0)
        torch.cuda.synchronize()
        iters = C.c_uint64(0)
        _ffi.check(L.gtc_pagerank_noalloc(n, d_off.data_ptr(), d_src.data_ptr(), d_deg.data_ptr(),
                                          0.85, 1e-12, cap, d_rank.data_ptr(), C.byref(iters),
                                          None))
        assert iters.value == cap
        got = d_rank.double().cpu().numpy()
        rel_l1 = np.abs(got - want.a).sum() / np.abs(want.a).sum()
        assert rel_l1 < 1e-6, (cap, rel_l1)


def test_noalloc_refuses_an_uncapped_solve_that_cannot_stop(gtc):
    from graph_tool import _ffi
    L = _ffi.lib()
    st = L.gtc_pagerank_noalloc(4, None, None, None, 0.85, 0.0, 0, None, None, None)
    assert st == _ffi.GTC_ERR_ARG
    assert b"never" in L.gtc_last_error()

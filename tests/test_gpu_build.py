"""The GPU CSR/CSC build against the oracle's blocks, byte for byte.

The oracle replays AdjList::add_edge (crates/gt-core/src/adj/list.rs:258-280)
with the push-swap of block.rs:171-209; the GPU must leave every vertex's
out-half and in-half in exactly that order."""
import numpy as np
import pytest

import _cases as K

pytestmark = pytest.mark.gpu


def _compare(oracle, gtc, n, src, tgt):
    want = K.OracleSolver(oracle).blocks(n, src, tgt)
    got = K.GpuSolver(gtc, "f32").blocks(n, src, tgt)
    names = ["out_off", "out_other", "out_idx", "in_off", "in_other", "in_idx"]
    for name, a, b in zip(names, want, got):
        a = np.asarray(a, np.uint64)
        b = np.asarray(b, np.uint64)
        assert a.shape == b.shape, (name, a.shape, b.shape)
        bad = np.nonzero(a != b)[0]
        assert bad.size == 0, f"{name} differs at {bad[:10]} (of {bad.size})"


def test_push_swap(oracle, gtc):
    K.case_push_swap(K.GpuSolver(gtc, "f32"))


def test_thousand(oracle, gtc):
    from graph_tool import synth
    _compare(oracle, gtc, *synth.thousand())


def test_empty_and_isolated(oracle, gtc):
    _compare(oracle, gtc, 0, np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    _compare(oracle, gtc, 7, np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    _compare(oracle, gtc, 5, np.array([4], np.uint32), np.array([0], np.uint32))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_multigraph_with_self_loops(oracle, gtc, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 40))
    m = int(rng.integers(1, 400))
    src = rng.integers(0, n, m).astype(np.uint32)
    tgt = rng.integers(0, n, m).astype(np.uint32)
    _compare(oracle, gtc, n, src, tgt)


def test_hub_rotations(oracle, gtc):
    # one vertex with long interleaved runs of in- and out-edges (the rotation
    # of its in-half is long), plus self-loops on it
    rng = np.random.default_rng(7)
    n, m = 500, 60_000
    src = rng.integers(0, n, m)
    tgt = rng.integers(0, n, m)
    hub = rng.random(m) < 0.5
    side = rng.random(m) < 0.5
    src[hub & side] = 0
    tgt[hub & ~side] = 0
    loops = rng.random(m) < 0.01
    src[loops] = 0
    tgt[loops] = 0
    _compare(oracle, gtc, n, src.astype(np.uint32), tgt.astype(np.uint32))


def test_rmat_scale_16(oracle, gtc):
    from graph_tool import synth
    n, src, tgt = synth.rmat_cpu(16, edge_factor=8, seed=3)
    _compare(oracle, gtc, n, src, tgt)


def test_bad_vertex_is_a_value_error(gtc):
    from graph_tool import _ffi
    import ctypes as C
    src = np.array([0, 3], np.uint32)
    tgt = np.array([1, 0], np.uint32)
    h = C.c_void_p()
    st = _ffi.lib().gtc_graph_create(3, 2, _ffi.ptr(src, _ffi.u32p), _ffi.ptr(tgt, _ffi.u32p),
                                     C.byref(h))
    assert st == _ffi.GTC_ERR_ARG and b"no such vertex" in _ffi.lib().gtc_last_error()


def test_first_handle_of_a_fresh_process_keeps_its_sizes(gtc):
    """The first gtc_graph of a process, built before anything else touched
    the GPU, reports the sizes it was built with and solves over all its
    edges (a solve over an edgeless graph would return the uniform vector)."""
    import subprocess
    import sys
    code = r'''
import ctypes as C, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from graph_tool import _ffi
L = _ffi.lib()
n, m = 6, 7
src = np.array([0, 1, 2, 3, 4, 5, 0], np.uint32)
tgt = np.array([1, 2, 0, 4, 5, 3, 3], np.uint32)
h = C.c_void_p()
_ffi.check(L.gtc_graph_create(n, m, _ffi.ptr(src, _ffi.u32p), _ffi.ptr(tgt, _ffi.u32p), C.byref(h)))
a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
_ffi.check(L.gtc_graph_info(h, C.byref(a), C.byref(b), C.byref(c)))
assert (a.value, b.value, c.value) == (n, m, m), (a.value, b.value, c.value)
r = np.full(n, 1.0 / n)
p = _ffi.PowerIteration(1e-10, 200, n, 1)
res = _ffi.Result()
_ffi.check(L.gtc_pagerank(h, None, None, 0, None, 0, 0.85, C.byref(p), _ffi.ptr(r, _ffi.f64p), n,
                          n, None, C.byref(res)))
assert abs(r.sum() - 1.0) < 1e-5 and r.max() - r.min() > 1e-3, r
print("ok", res.iterations)
'''
    import os
    pkg = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "graph-tool-rs_gb300")
    out = subprocess.run([sys.executable, "-c", code, pkg], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok")

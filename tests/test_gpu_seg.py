"""The segmented pull sweep of the FP32 PageRank path (gtc_seg.cu), pinned
on, against the oracle's f64 result: relative L1 <= 1e-6 and the sweep
count within 2, on graphs that exercise several source segments (32768
sources each), destination groups (1024 vertices each), pairs cut into
sub-pairs (a destination with thousands of in-edges from one segment) and
phase-1 units cut inside one (segment, group) key."""
import numpy as np
import pytest

import _cases as K

pytestmark = pytest.mark.gpu


@pytest.fixture
def seg_on(monkeypatch):
    monkeypatch.setenv("GTC_SWEEP_VARIANT", "2")


def _rel_l1(a, b):
    return float(np.abs(a - b).sum() / np.abs(b).sum())


@pytest.fixture(scope="module")
def rmat16():
    from graph_tool import synth
    return synth.rmat_cpu(16, edge_factor=16, seed=21)


@pytest.fixture(scope="module")
def hubby():
    # 3 segments; vertex 5 takes 20000 in-edges from sources all over the
    # graph (sub-pairs of 256 edges, keys of more than 4096 edges); sinks
    rng = np.random.default_rng(77)
    n = 70_000
    src = rng.integers(0, n, 400_000)
    tgt = rng.integers(0, n, 400_000)
    tgt[:20_000] = 5
    keep = ~np.isin(src, rng.choice(n, 2000, replace=False))  # sinks
    return n, src[keep].astype(np.uint32), tgt[keep].astype(np.uint32)


def _check(oracle, gtc, n, src, tgt, eps=1e-7, **kw):
    want, iw = K.OracleSolver(oracle).pagerank(n, src, tgt, grain=4096, epsilon=eps,
                                               max_iter=1000, **kw)
    got, ig = K.GpuSolver(gtc, "f32").pagerank(n, src, tgt, grain=4096, epsilon=eps,
                                               max_iter=1000, **kw)
    err = _rel_l1(got, want)
    print(f"seg n={n} m={src.size} {sorted(kw)}: rel L1 {err:.2e}, sweeps {ig} vs {iw}")
    assert err < 1e-6, (sorted(kw), err)
    assert abs(ig - iw) <= 2, (ig, iw)


def test_seg_rmat_unweighted(oracle, gtc, rmat16, seg_on):
    n, src, tgt = rmat16
    _check(oracle, gtc, n, src, tgt)


def test_seg_rmat_weighted_pers_reversed(oracle, gtc, rmat16, seg_on):
    n, src, tgt = rmat16
    rng = np.random.default_rng(3)
    w = rng.uniform(0.1, 1.0, src.size)
    p = rng.exponential(1.0, n)
    _check(oracle, gtc, n, src, tgt, weight=w)
    _check(oracle, gtc, n, src, tgt, pers=p / p.sum())
    _check(oracle, gtc, n, src, tgt, reversed=True, weight=w)


def test_seg_hub_subpairs(oracle, gtc, hubby, seg_on):
    n, src, tgt = hubby
    _check(oracle, gtc, n, src, tgt)
    w = np.random.default_rng(4).uniform(0.1, 1.0, src.size)
    _check(oracle, gtc, n, src, tgt, weight=w, reversed=True)


def test_seg_warm_start(oracle, gtc, hubby, seg_on):
    n, src, tgt = hubby
    r0 = np.random.default_rng(5).uniform(0.0, 2.0 / n, n)
    _check(oracle, gtc, n, src, tgt, rank=r0, had=n)


def test_seg_matches_pull_sweep(gtc, rmat16, monkeypatch):
    """The two FP32 sweeps agree to FP32 accuracy and take the same sweeps."""
    n, src, tgt = rmat16
    monkeypatch.setenv("GTC_SWEEP_VARIANT", "2")
    a, ia = K.GpuSolver(gtc, "f32").pagerank(n, src, tgt, grain=4096, epsilon=1e-7,
                                             max_iter=1000)
    monkeypatch.setenv("GTC_SWEEP_VARIANT", "0")
    b, ib = K.GpuSolver(gtc, "f32").pagerank(n, src, tgt, grain=4096, epsilon=1e-7,
                                             max_iter=1000)
    assert _rel_l1(a, b) < 5e-7
    assert abs(ia - ib) <= 1

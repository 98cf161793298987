"""Batched personalised PageRank (one SpMM over B right-hand sides) against
the oracle's pagerank_with, one call per seed set (the reference's way)."""
import numpy as np
import pytest

import _cases as K

pytestmark = pytest.mark.gpu


def _seed_sets(n, B, rng, max_size=8):
    sets = []
    for _ in range(B):
        k = int(rng.integers(1, max_size + 1))
        sets.append(rng.choice(n, k, replace=False))
    return sets


def _check(oracle, gtc, n, src, tgt, B, weight=None, reversed=False, eps=1e-7, seed=1,
           gather="bulk", sets=None):
    rng = np.random.default_rng(seed)
    if sets is None:
        sets = _seed_sets(n, B, rng)
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    wm = None
    if weight is not None:
        wm = g.new_edge_property("double")
        wm.a[:] = weight
    ranks, iters = g.ppr_batch(sets, weight=wm, epsilon=eps, max_iter=1000, reversed=reversed,
                               gather=gather)
    og = oracle.Graph(n)
    og.add_edge_arrays(src, tgt)
    worst = 0.0
    for b, st in enumerate(sets):
        pers = np.zeros(n)
        pers[st] = 1.0 / len(st)
        want, it = og.pagerank(weight=weight, pers=pers, epsilon=eps, max_iter=1000, grain=4096,
                               reversed=reversed)
        err = np.abs(ranks[b] - want).sum() / np.abs(want).sum()
        worst = max(worst, err)
        assert err < 1e-6, (b, err, iters[b], it)
        assert abs(int(iters[b]) - it) <= 3, (b, iters[b], it)
    print(f"ppr batch B={B}: worst rel L1 {worst:.2e}")


@pytest.fixture(params=["bulk", "regs"])
def variant(request):
    """Both gather variants of the batched sweep (bulk copies into shared
    memory, loads into registers) must give the oracle's results."""
    return request.param


def test_ppr_batch_matches_separate_solves(oracle, gtc, variant):
    from graph_tool import synth
    n, src, tgt, _ = synth.erdos_renyi_sinks(n=3000, m=24000)
    _check(oracle, gtc, n, src, tgt, 37, gather=variant)


def test_ppr_batch_padded_columns_weighted(oracle, gtc, variant):
    from graph_tool import synth
    n, src, tgt = synth.rmat_cpu(11, edge_factor=8, seed=4)
    w = np.random.default_rng(2).uniform(0.1, 1.0, src.size)
    _check(oracle, gtc, n, src, tgt, 130, weight=w, seed=3, gather=variant)


def test_ppr_batch_reversed_with_hubs(oracle, gtc, variant):
    # a hub with more in-edges than one warp row takes (a CTA row)
    rng = np.random.default_rng(5)
    n, m = 4000, 40000
    src = rng.integers(0, n, m)
    tgt = rng.integers(0, n, m)
    tgt[: 6000] = 7
    _check(oracle, gtc, n, src.astype(np.uint32), tgt.astype(np.uint32), 64, seed=6,
           gather=variant)
    _check(oracle, gtc, n, src.astype(np.uint32), tgt.astype(np.uint32), 64, seed=7, reversed=True,
           gather=variant)


def test_ppr_batch_seeds_without_in_edges(oracle, gtc, variant):
    # The sweeps skip rows without in-edges; seeds among them (sinks and
    # vertices with out-edges) are finished with an empty sum, and the
    # skipped rows must read as zero after the columns are repacked.
    from graph_tool import synth
    n, src, tgt = synth.rmat_cpu(10, edge_factor=8, seed=9)
    indeg = np.bincount(tgt, minlength=n)
    outdeg = np.bincount(src, minlength=n)
    no_in = np.flatnonzero(indeg == 0)
    no_in_src = np.flatnonzero((indeg == 0) & (outdeg > 0))
    assert no_in.size > 100 and no_in_src.size > 10
    rng = np.random.default_rng(11)
    sets = []
    for b in range(70):
        k = int(rng.integers(1, 6))
        pool = no_in_src if b % 3 == 0 else (no_in if b % 3 == 1 else np.arange(n))
        sets.append(rng.choice(pool, min(k, pool.size), replace=False))
    _check(oracle, gtc, n, src, tgt, len(sets), gather=variant, sets=sets)


def test_ppr_batch_zero_weights_make_sinks(oracle, gtc, variant):
    # a vertex whose out-edges all weigh 0 is a sink by weight although its
    # row is gathered (with weight 0); wide rows and narrow rows
    from graph_tool import synth
    n, src, tgt = synth.rmat_cpu(10, edge_factor=8, seed=17)
    w = np.random.default_rng(5).uniform(0.1, 1.0, src.size)
    zero_src = np.random.default_rng(6).choice(n, n // 10, replace=False)
    w[np.isin(src, zero_src)] = 0.0
    w[np.random.default_rng(7).random(src.size) < 0.05] = 0.0
    _check(oracle, gtc, n, src, tgt, 40, weight=w, seed=18, gather=variant)
    _check(oracle, gtc, n, src, tgt, 6, weight=w, seed=19, gather=variant)


def test_ppr_batch_widest(oracle, gtc, variant):
    # 512 columns: rows of 16 lines, then 12, 8, 6, 4 ... as columns converge
    from graph_tool import synth
    n, src, tgt, _ = synth.erdos_renyi_sinks(n=1500, m=12000)
    _check(oracle, gtc, n, src, tgt, 512, seed=21, gather=variant)


@pytest.mark.parametrize("B", [5, 12])
def test_ppr_batch_narrow_rows_from_the_start(oracle, gtc, B):
    # at most 16 columns: rows of 8 or 16 floats from the first sweep, a
    # group of lanes per row; weighted and reversed as well
    from graph_tool import synth
    n, src, tgt = synth.rmat_cpu(11, edge_factor=8, seed=12)
    w = np.random.default_rng(4).uniform(0.1, 1.0, src.size)
    _check(oracle, gtc, n, src, tgt, B, seed=13)
    _check(oracle, gtc, n, src, tgt, B, weight=w, reversed=True, seed=14)


def test_ppr_batch_max_iter_caps_every_column(oracle, gtc, variant):
    # a cap below convergence: every column stops at the cap with the
    # iterate of that sweep (also in the narrow rows of the last columns)
    from graph_tool import synth
    n, src, tgt, _ = synth.erdos_renyi_sinks(n=2000, m=16000)
    rng = np.random.default_rng(9)
    sets = _seed_sets(n, 20, rng)
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    ranks, iters = g.ppr_batch(sets, epsilon=1e-12, max_iter=5, gather=variant)
    assert (iters == 5).all()
    og = oracle.Graph(n)
    og.add_edge_arrays(src, tgt)
    for b in (0, 7, 19):
        pers = np.zeros(n)
        pers[sets[b]] = 1.0 / len(sets[b])
        want, it = og.pagerank(pers=pers, epsilon=1e-12, max_iter=5, grain=4096)
        assert it == 5
        err = np.abs(ranks[b] - want).sum() / np.abs(want).sum()
        assert err < 1e-6, (b, err)


def test_ppr_batch_rejects_bad_batches(gtc):
    g = gtc.Graph()
    g.add_vertex(3)
    g.add_edge(0, 1)
    with pytest.raises(ValueError):
        g.ppr_batch([[0]] * 513)
    with pytest.raises(IndexError):
        g.ppr_batch([[5]])

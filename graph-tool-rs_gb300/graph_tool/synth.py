"""Seeded synthetic graphs (CPU, numpy) in the shapes the reference's tests
and this project's benchmarks use.

* ``SplitMix64`` is the generator graph-tool-rs's own tests use for their
  fixtures (crates/gt-algo/tests/u16_centrality.rs:59-72), so ``thousand()``
  and ``eigen60()`` regenerate the reference's test graphs exactly
  (u16_centrality.rs:93-107 and :494-508).
* ``erdos_renyi_sinks()`` is the plain-PageRank workload: uniform directed
  pairs without self-loops or duplicates, with every out-edge of a random 5%
  of the vertices dropped before insertion.
* ``rmat_cpu()`` is a small-scale R-MAT for tests; the full-size generators
  run on the GPU (``graph_tool.synth_gpu``).

Edge lists are (src, tgt) uint32 arrays in insertion order.
"""
from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_MASK = (1 << 64) - 1


class SplitMix64:
    """The reference tests' Rng (u16_centrality.rs:59-72)."""

    def __init__(self, seed: int):
        self.s = seed & _MASK

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & _MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        return z ^ (z >> 31)

    def below(self, n: int) -> int:
        return self.next() % n

    def block(self, count: int) -> np.ndarray:
        """The next ``count`` outputs at once (uint64), advancing the state."""
        i = np.arange(1, count + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            z = np.uint64(self.s) + i * _GAMMA
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            z = z ^ (z >> np.uint64(31))
        self.s = (self.s + count * 0x9E3779B97F4A7C15) & _MASK
        return z


def thousand():
    """u16_centrality.rs:93-107: ring of 1000 + 4000 chords, then the 50
    sinks 17, 37, ..., 997 lose every out-edge (before insertion)."""
    N = 1000
    r = SplitMix64(0x243F6A8885A308D3)
    edges = [(i, (i + 1) % N) for i in range(N)]
    for _ in range(4000):
        s = r.below(N)
        t = r.below(N)
        edges.append((s, t))

    def sink(i):
        return i >= 17 and (i - 17) % 20 == 0 and i < 17 + 20 * 50

    edges = [(s, t) for (s, t) in edges if not sink(s)]
    e = np.array(edges, dtype=np.uint32)
    return N, e[:, 0].copy(), e[:, 1].copy()


def eigen60():
    """u16_centrality.rs:494-508: ring of 60 + 240 chords; weights
    1 + 0.25*(i % 5) by edge index."""
    n = 60
    r = SplitMix64(0xFEEDFACECAFEBEEF)
    edges = [(i, (i + 1) % n) for i in range(n)]
    for _ in range(240):
        s = r.below(n)
        t = r.below(n)
        edges.append((s, t))
    e = np.array(edges, dtype=np.uint32)
    w = np.array([1.0 + (i % 5) * 0.25 for i in range(len(edges))])
    return n, e[:, 0].copy(), e[:, 1].copy(), w


def erdos_renyi_sinks(n: int = 10_000, m: int = 100_000, sink_frac: float = 0.05,
                      seed: int = 0x5EED_0000_0000_0001):
    """Directed G(n, m): uniform (s, t) pairs, self-loops and duplicates
    rejected, in draw order; then ``sink_frac * n`` vertices drawn without
    replacement lose all out-edges (so m shrinks).  Returns (n, src, tgt,
    sinks)."""
    r = SplitMix64(seed)
    seen = set()
    out = np.empty((m, 2), np.int64)
    k = 0
    while k < m:
        z = r.block(2 * (m - k) + 64)
        s = (z[0::2] % np.uint64(n)).astype(np.int64)
        t = (z[1::2] % np.uint64(n)).astype(np.int64)
        for a, b in zip(s.tolist(), t.tolist()):
            if a == b or (a, b) in seen:
                continue
            seen.add((a, b))
            out[k] = (a, b)
            k += 1
            if k == m:
                break
    # partial Fisher-Yates for the sinks
    n_s = int(round(sink_frac * n))
    perm = np.arange(n)
    for i in range(n_s):
        j = i + r.below(n - i)
        perm[i], perm[j] = perm[j], perm[i]
    sinks = np.sort(perm[:n_s])
    is_sink = np.zeros(n, bool)
    is_sink[sinks] = True
    keep = ~is_sink[out[:, 0]]
    e = out[keep]
    return n, e[:, 0].astype(np.uint32), e[:, 1].astype(np.uint32), sinks


def rmat_cpu(scale: int, edge_factor: int = 16, abcd=(0.57, 0.19, 0.19, 0.05),
             seed: int = 1, permute: bool = True, dedup: bool = True):
    """R-MAT (small scales, tests): edge_factor * 2^scale draws, each bit of
    (src, tgt) chosen by quadrant probabilities; a random vertex relabelling;
    duplicates removed keeping the first draw (draw order kept).  Self-loops
    are kept."""
    n = 1 << scale
    m = edge_factor * n
    r = SplitMix64(seed)
    a, b, c, _ = abcd
    src = np.zeros(m, np.int64)
    tgt = np.zeros(m, np.int64)
    for lvl in range(scale):
        u = (r.block(m) >> np.uint64(11)).astype(np.float64) / float(1 << 53)
        sb = (u >= a + b).astype(np.int64)                    # quadrants c, d
        tb = (((u >= a) & (u < a + b)) | (u >= a + b + c)).astype(np.int64)  # b, d
        src |= sb << lvl
        tgt |= tb << lvl
    if permute:
        keys = r.block(n) >> np.uint64(1)  # 63-bit keys (the GPU sorts int64)
        perm = np.argsort(keys, kind="stable")
        relabel = np.empty(n, np.int64)
        relabel[perm] = np.arange(n)
        src, tgt = relabel[src], relabel[tgt]
    if dedup:
        key = src * n + tgt
        _, first = np.unique(key, return_index=True)
        first.sort()
        src, tgt = src[first], tgt[first]
    return n, src.astype(np.uint32), tgt.astype(np.uint32)


def sbm_batch(G: int, n_min: int = 100, n_max: int = 100_000, blocks: int = 4,
              k_in: float = 16.0, k_out: float = 2.0, seed: int = 3):
    """G directed stochastic-block-model graphs of log-uniform sizes in
    [n_min, n_max]: ``blocks`` equal blocks, edge probability k_in / n inside
    a block and k_out / n across (mean out-degree (k_in + (blocks - 1) k_out)
    / blocks).  Each block pair draws its edge count (binomial) and then its
    endpoints uniformly; duplicates and self-loops are dropped (first draw
    kept).  Returns a list of (n, src, tgt) with local indices."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(G):
        n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
        bounds = np.linspace(0, n, blocks + 1).round().astype(np.int64)
        srcs, tgts = [], []
        for a in range(blocks):
            for b in range(blocks):
                na, nb = bounds[a + 1] - bounds[a], bounds[b + 1] - bounds[b]
                p = (k_in if a == b else k_out) / n
                cnt = rng.binomial(int(na * nb), min(p, 1.0)) if na and nb else 0
                srcs.append(bounds[a] + rng.integers(0, max(na, 1), cnt))
                tgts.append(bounds[b] + rng.integers(0, max(nb, 1), cnt))
        s = np.concatenate(srcs) if srcs else np.zeros(0, np.int64)
        t = np.concatenate(tgts) if tgts else np.zeros(0, np.int64)
        keep = s != t
        s, t = s[keep], t[keep]
        key = s * n + t
        _, first = np.unique(key, return_index=True)
        first.sort()
        out.append((n, s[first].astype(np.uint32), t[first].astype(np.uint32)))
    return out

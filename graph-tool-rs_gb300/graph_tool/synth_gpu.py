"""Full-size synthetic graphs, generated on the GPU with torch tensor ops.

Same streams as ``graph_tool.synth`` (counter-based SplitMix64: output k of a
generator seeded ``s`` is mix(s + (k+1) * gamma)), so at small scale the GPU
and CPU generators produce identical edge lists.  torch is plumbing here: the
inputs it makes are handed to libgtc as device pointers.

* ``rmat``: R-MAT, (a, b, c, d) quadrant bits per level, random vertex
  relabelling, duplicates removed keeping the first draw (draw order kept),
  self-loops kept.
* ``chung_lu``: expected out- and in-degrees i.i.d. Pareto(exponent alpha,
  minimum x_min) capped, scaled to sum to m; sources and targets drawn
  independently by inverse CDF over the cumulative weights; self-loops
  dropped, multi-edges kept; FP32 edge weights U(lo, hi).
"""
from __future__ import annotations

import torch

_GAMMA = 0x9E3779B97F4A7C15
_M1 = 0xBF58476D1CE4E5B9
_M2 = 0x94D049BB133111EB


def _s64(x: int) -> int:
    """An unsigned 64-bit constant as the signed int64 torch stores."""
    x &= (1 << 64) - 1
    return x - (1 << 64) if x >= 1 << 63 else x


def _srl(z: torch.Tensor, k: int) -> torch.Tensor:
    """Logical right shift of int64 bit patterns."""
    return (z >> k) & ((1 << (64 - k)) - 1)


def splitmix(seed: int, k0: int, count: int, device) -> torch.Tensor:
    """Outputs k0 .. k0+count-1 of SplitMix64(seed), as int64 bit patterns."""
    k = torch.arange(k0 + 1, k0 + count + 1, dtype=torch.int64, device=device)
    z = k * _s64(_GAMMA) + _s64(seed)
    z = (z ^ _srl(z, 30)) * _s64(_M1)
    z = (z ^ _srl(z, 27)) * _s64(_M2)
    return z ^ _srl(z, 31)


def _unit(z: torch.Tensor) -> torch.Tensor:
    """Top 53 bits as a double in [0, 1)."""
    return _srl(z, 11).to(torch.float64) * (1.0 / float(1 << 53))


def rmat(scale: int, edge_factor: int = 16, abcd=(0.57, 0.19, 0.19, 0.05), seed: int = 1,
         permute: bool = True, dedup: bool = True, device="cuda"):
    """(n, src int32 tensor, tgt int32 tensor) on ``device``; ids < 2^31."""
    n = 1 << scale
    m = edge_factor * n
    a, b, c, _ = abcd
    src = torch.zeros(m, dtype=torch.int64, device=device)
    tgt = torch.zeros(m, dtype=torch.int64, device=device)
    for lvl in range(scale):
        u = _unit(splitmix(seed, lvl * m, m, device))
        sb = u >= a + b
        tb = ((u >= a) & (u < a + b)) | (u >= a + b + c)
        src |= sb.to(torch.int64) << lvl
        tgt |= tb.to(torch.int64) << lvl
        del u, sb, tb
    if permute:
        keys = _srl(splitmix(seed, scale * m, n, device), 1)
        perm = torch.argsort(keys, stable=True)
        relabel = torch.empty(n, dtype=torch.int64, device=device)
        relabel[perm] = torch.arange(n, dtype=torch.int64, device=device)
        src = relabel[src]
        tgt = relabel[tgt]
        del keys, perm, relabel
    if dedup:
        key = src * n + tgt
        sk, order = torch.sort(key, stable=True)
        first = torch.ones_like(sk, dtype=torch.bool)
        first[1:] = sk[1:] != sk[:-1]
        keep = torch.sort(order[first]).values
        del key, sk, order, first
        src = src[keep]
        tgt = tgt[keep]
    return n, src.to(torch.int32), tgt.to(torch.int32)


def chung_lu(n: int, m: int, alpha: float = 2.1, x_min: float = 2.0, cap: float = 100_000.0,
             seed: int = 2, w_lo: float = 0.1, w_hi: float = 1.0, device="cuda"):
    """(n, src, tgt, w) tensors on ``device`` (int32, int32, float32)."""
    k = 0

    def draw(count):
        nonlocal k
        u = _unit(splitmix(seed, k, count, device))
        k += count
        return u

    def pareto(count):
        u = 1.0 - draw(count)  # (0, 1]
        x = x_min * torch.pow(u, -1.0 / (alpha - 1.0))
        return torch.clamp(x, max=cap)

    cdf_out = torch.cumsum(pareto(n), 0)
    cdf_in = torch.cumsum(pareto(n), 0)
    cdf_out = cdf_out / cdf_out[-1]
    cdf_in = cdf_in / cdf_in[-1]
    src = torch.searchsorted(cdf_out, draw(m), right=True).clamp_(max=n - 1)
    tgt = torch.searchsorted(cdf_in, draw(m), right=True).clamp_(max=n - 1)
    w = (w_lo + (w_hi - w_lo) * draw(m)).to(torch.float32)
    keep = src != tgt
    return n, src[keep].to(torch.int32), tgt[keep].to(torch.int32), w[keep]

"""The adjoint formulas against FP64 central finite differences (no GPU).

L = c . pi for PageRank pi(w, p) on the 2,048-vertex R-MAT instance; the
dense adjoint gradients (tests/_dense.py, the formulas the GPU kernels
implement) must match (L(x + h) - L(x - h)) / 2h, h = 1e-6, on sampled edge
weights and personalisation entries."""
import numpy as np

import _dense as D


def test_adjoint_matches_central_differences():
    n, src, tgt, w, p, c = D.small_problem()
    d = 0.85
    pi, lam, gw, gp = D.gradients(n, src, tgt, w, p, d, c)
    rng = np.random.default_rng(3)
    h = 1e-6
    for e in rng.choice(src.size, 12, replace=False):
        wp, wm = w.copy(), w.copy()
        wp[e] += h
        wm[e] -= h
        fd = (c @ D.pagerank(n, src, tgt, wp, p, d) - c @ D.pagerank(n, src, tgt, wm, p, d)) / (2 * h)
        assert abs(fd - gw[e]) <= 1e-6 * max(1.0, abs(fd)) + 1e-7, (e, fd, gw[e])
    for v in rng.choice(n, 12, replace=False):
        pp, pm = p.copy(), p.copy()
        pp[v] += h
        pm[v] -= h
        fd = (c @ D.pagerank(n, src, tgt, w, pp, d) - c @ D.pagerank(n, src, tgt, w, pm, d)) / (2 * h)
        assert abs(fd - gp[v]) <= 1e-6 * max(1.0, abs(fd)) + 1e-7, (v, fd, gp[v])

"""Dense FP64 PageRank and its adjoint (independent references for the
gradient tests).  A[t, s] = w_e / deg_s summed over edges s -> t with
deg_s != 0; sinks (deg_s == 0) redistribute through the personalisation."""
import numpy as np


def matrices(n, src, tgt, w):
    src = np.asarray(src, np.int64)
    tgt = np.asarray(tgt, np.int64)
    deg = np.zeros(n)
    np.add.at(deg, src, w)
    A = np.zeros((n, n))
    ok = deg[src] != 0
    np.add.at(A, (tgt[ok], src[ok]), w[ok] / deg[src[ok]])
    sink = (deg == 0).astype(np.float64)
    return A, sink, deg


def pagerank(n, src, tgt, w, p, d):
    """pi = (1-d) p + d (A pi + p (s . pi)), solved exactly."""
    A, s, _ = matrices(n, src, tgt, w)
    M = np.eye(n) - d * (A + np.outer(p, s))
    return np.linalg.solve(M, (1 - d) * p)


def gradients(n, src, tgt, w, p, d, c):
    """dL/dw and dL/dp of L = c . pi by the adjoint (dense)."""
    A, s, deg = matrices(n, src, tgt, w)
    M = np.eye(n) - d * (A + np.outer(p, s))
    pi = np.linalg.solve(M, (1 - d) * p)
    lam = np.linalg.solve(M.T, c)
    gp = lam * ((1 - d) + d * (s @ pi))
    atl = A.T @ lam
    src = np.asarray(src, np.int64)
    tgt = np.asarray(tgt, np.int64)
    gw = np.where(deg[src] != 0, d * pi[src] / np.where(deg[src] != 0, deg[src], 1.0)
                  * (lam[tgt] - atl[src]), 0.0)
    return pi, lam, gw, gp


def small_problem(seed=11, scale=11):
    """The 2,048-vertex instance of the gradient workload: R-MAT scale 11,
    edge factor 16, weights U(0.1, 1), pers Dirichlet(1), c ~ N(0, 1)."""
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "graph-tool-rs_gb300"))
    from graph_tool import synth
    n, src, tgt = synth.rmat_cpu(scale, edge_factor=16, seed=seed)
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.1, 1.0, src.size)
    p = rng.exponential(1.0, n)
    p /= p.sum()
    c = rng.standard_normal(n)
    return n, src, tgt, w, p, c

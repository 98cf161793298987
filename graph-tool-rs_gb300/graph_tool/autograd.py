"""Differentiable PageRank for torch: ``pagerank(g, weight, pers, ...)``.

The forward is the FP32 GPU solve (gtc_pagerank_device); the backward is the
hand-written adjoint (gtc_pagerank_adjoint_device): it solves the transposed
fixed point lambda = dL/dpi + d (A^T lambda + s (p . lambda)) and forms
dL/dw and dL/dp per edge and per vertex.  Only the converged pi is saved
(implicit-function theorem); no iterate history is kept.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _ffi
from ._rust import Graph


def _stream(device) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class _PageRank(torch.autograd.Function):
    @staticmethod
    def forward(ctx, g: Graph, weight, pers, damping: float, epsilon: float, max_iter: int,
                adj_epsilon: float, adj_max_iter: int):
        h = g.handle()
        n = g.num_vertices()
        dev = weight.device if weight is not None else (pers.device if pers is not None else
                                                       torch.device("cuda", torch.cuda.current_device()))
        dtype = weight.dtype if weight is not None else (pers.dtype if pers is not None
                                                         else torch.float32)
        rank = torch.empty(n, dtype=dtype, device=dev)
        w = weight.contiguous() if weight is not None else None
        p = pers.contiguous() if pers is not None else None
        params = _ffi.PowerIteration(float(epsilon), int(max_iter), n, max(-(-n // 4096), 1))
        opt = _ffi.Options(_ffi.GTC_PREC_F32, 0, _stream(dev), 0, 0)
        res = _ffi.Result()
        rv = _ffi.DVec.of(rank)
        wv = _ffi.DVec.of(w)
        pv = _ffi.DVec.of(p)
        _ffi.check(_ffi.lib().gtc_pagerank_device(
            h, None, C.byref(wv) if wv else None, C.byref(pv) if pv else None, float(damping),
            C.byref(params), C.byref(rv), 0, C.byref(opt), C.byref(res)))
        ctx.g = g
        ctx.damping = float(damping)
        ctx.adj = (float(adj_epsilon), int(adj_max_iter))
        ctx.iterations = int(res.iterations)
        ctx.save_for_backward(w, p, rank)
        return rank

    @staticmethod
    def backward(ctx, grad_rank):
        w, p, rank = ctx.saved_tensors
        g = ctx.g
        n, m = g.num_vertices(), g.edge_index_range()
        dev = rank.device
        gr = grad_rank.contiguous().to(rank.dtype)
        gw = torch.empty(m, dtype=rank.dtype, device=dev) if (w is not None and ctx.needs_input_grad[1]) else None
        gp = torch.empty(n, dtype=rank.dtype, device=dev) if (p is not None and ctx.needs_input_grad[2]) else None
        eps, mi = ctx.adj
        params = _ffi.PowerIteration(eps, mi, n, max(-(-n // 4096), 1))
        opt = _ffi.Options(_ffi.GTC_PREC_F32, 0, _stream(dev), 0, 0)
        res = _ffi.Result()
        wv, pv = _ffi.DVec.of(w), _ffi.DVec.of(p)
        piv, gv = _ffi.DVec.of(rank), _ffi.DVec.of(gr)
        gwv, gpv = _ffi.DVec.of(gw), _ffi.DVec.of(gp)
        _ffi.check(_ffi.lib().gtc_pagerank_adjoint_device(
            g.handle(), None, C.byref(wv) if wv else None, C.byref(pv) if pv else None,
            ctx.damping, C.byref(params), C.byref(piv), C.byref(gv),
            C.byref(gwv) if gwv else None, C.byref(gpv) if gpv else None, C.byref(opt),
            C.byref(res)))
        return None, gw, gp, None, None, None, None, None


def pagerank(g: Graph, weight: torch.Tensor | None = None, pers: torch.Tensor | None = None,
             damping: float = 0.85, epsilon: float = 1e-7, max_iter: int = 0,
             adj_epsilon: float | None = None, adj_max_iter: int = 0) -> torch.Tensor:
    """PageRank of ``g`` as a differentiable function of the edge weights
    (a CUDA tensor indexed by edge index) and the personalisation vector (by
    vertex index).  Returns the rank vector (same dtype, float32 or float64
    storage; the arithmetic is the FP32 path)."""
    return _PageRank.apply(g, weight, pers, damping, epsilon, max_iter,
                           epsilon if adj_epsilon is None else adj_epsilon, adj_max_iter)

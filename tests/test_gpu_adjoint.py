"""The PageRank adjoint on the GPU against the dense FP64 adjoint (itself
checked against FP64 central differences in test_adjoint_math.py), through
torch.autograd and through the host C ABI."""
import ctypes as C

import numpy as np
import pytest

import _dense as D

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def problem():
    return D.small_problem()


def test_autograd_matches_dense_fp64(gtc, problem):
    import torch

    from graph_tool import autograd

    n, src, tgt, w, p, c = problem
    d = 0.85
    pi_ref, lam_ref, gw_ref, gp_ref = D.gradients(n, src, tgt, w, p, d, c)
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    dev = torch.device("cuda", 0)
    wt = torch.tensor(w, dtype=torch.float32, device=dev, requires_grad=True)
    pt = torch.tensor(p, dtype=torch.float32, device=dev, requires_grad=True)
    ct = torch.tensor(c, dtype=torch.float32, device=dev)
    pi = autograd.pagerank(g, wt, pt, damping=d, epsilon=1e-7, max_iter=2000)
    assert _rel(pi.detach().double().cpu().numpy(), pi_ref) < 1e-5
    loss = (ct * pi).sum()
    loss.backward()
    gw = wt.grad.double().cpu().numpy()
    gp = pt.grad.double().cpu().numpy()
    print(f"adjoint: rel err dL/dw {_rel(gw, gw_ref):.2e}, dL/dp {_rel(gp, gp_ref):.2e}")
    assert _rel(gw, gw_ref) < 1e-4
    assert _rel(gp, gp_ref) < 1e-4


def test_host_abi_adjoint(gtc, problem):
    from graph_tool import _ffi

    n, src, tgt, w, p, c = problem
    d = 0.85
    pi_ref, lam_ref, gw_ref, gp_ref = D.gradients(n, src, tgt, w, p, d, c)
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    gw = np.zeros(src.size)
    gp = np.zeros(n)
    params = _ffi.PowerIteration(1e-7, 2000, n, 1)
    res = _ffi.Result()
    _ffi.check(_ffi.lib().gtc_pagerank_adjoint(
        g.handle(), None, _ffi.ptr(w, _ffi.f64p), w.size, _ffi.ptr(p, _ffi.f64p), n, d,
        C.byref(params), _ffi.ptr(pi_ref, _ffi.f64p), _ffi.ptr(c, _ffi.f64p),
        _ffi.ptr(gw, _ffi.f64p), _ffi.ptr(gp, _ffi.f64p), None, C.byref(res)))
    assert res.iterations > 5
    assert _rel(gw, gw_ref) < 1e-4
    assert _rel(gp, gp_ref) < 1e-4


def test_unweighted_uniform_adjoint(gtc, problem):
    """Unity weights and uniform pers: dL/dw is the derivative with respect
    to implicit unit weights."""
    from graph_tool import _ffi

    n, src, tgt, _, _, c = problem
    d = 0.85
    ones = np.ones(src.size)
    unif = np.full(n, 1.0 / n)
    pi_ref, lam_ref, gw_ref, gp_ref = D.gradients(n, src, tgt, ones, unif, d, c)
    g = gtc.Graph()
    g.add_vertex(n)
    g.add_edges(src, tgt)
    gw = np.zeros(src.size)
    gp = np.zeros(n)
    params = _ffi.PowerIteration(1e-7, 2000, n, 1)
    _ffi.check(_ffi.lib().gtc_pagerank_adjoint(
        g.handle(), None, None, 0, None, 0, d, C.byref(params), _ffi.ptr(pi_ref, _ffi.f64p),
        _ffi.ptr(c, _ffi.f64p), _ffi.ptr(gw, _ffi.f64p), _ffi.ptr(gp, _ffi.f64p), None, None))
    assert _rel(gw, gw_ref) < 1e-4
    assert _rel(gp, gp_ref) < 1e-4

"""The C ABI without a GPU: the library builds for sm_103a, loads, exports
every entry point include/*.h declares, and refuses to compute (no CPU
fallback) when no CUDA device is present."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(gtc_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for want in ("gtc_graph_create", "gtc_pagerank", "gtc_eigenvector", "gtc_graph_destroy"):
        assert want in names


def test_library_exports_every_declared_symbol(gtc):
    from graph_tool import _ffi
    L = C.CDLL(_ffi.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing
    # and the binding knows every one of them
    assert set(declared_symbols()) <= set(_ffi.SIGNATURES), \
        set(declared_symbols()) - set(_ffi.SIGNATURES)


def test_version_and_last_error(gtc):
    from graph_tool import _ffi
    assert b"sm_103a" in _ffi.lib().gtc_version()
    assert isinstance(_ffi.lib().gtc_last_error(), bytes)


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # noqa: BLE001
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_no_device_is_an_error_not_a_fallback(gtc):
    from graph_tool import _ffi
    src = np.array([0], np.uint32)
    tgt = np.array([1], np.uint32)
    h = C.c_void_p()
    st = _ffi.lib().gtc_graph_create(2, 1, _ffi.ptr(src, _ffi.u32p), _ffi.ptr(tgt, _ffi.u32p),
                                     C.byref(h))
    assert st == _ffi.GTC_ERR_NO_DEVICE
    assert h.value is None
    assert b"no usable CUDA device" in _ffi.lib().gtc_last_error()
    g = gtc.Graph()
    g.add_vertex(2)
    g.add_edge(0, 1)
    with pytest.raises(_ffi.GtcError):
        g.pagerank(g.new_vertex_property("double"))


def test_bad_arguments_are_rejected_before_the_device(gtc):
    from graph_tool import _ffi
    L = _ffi.lib()
    params = _ffi.PowerIteration(1e-6, 0, 3, 1)
    r = np.zeros(3)
    assert L.gtc_pagerank(None, None, None, 0, None, 0, 0.85, C.byref(params),
                          _ffi.ptr(r, _ffi.f64p), 3, 0, None, None) == _ffi.GTC_ERR_ARG
    assert b"graph is NULL" in L.gtc_last_error()
    assert L.gtc_graph_create(2, 1, None, None, None) == _ffi.GTC_ERR_ARG
    assert L.gtc_graph_create(1 << 33, 0, None, None, C.byref(C.c_void_p())) == _ffi.GTC_ERR_ARG

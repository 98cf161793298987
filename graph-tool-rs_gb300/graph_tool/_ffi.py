"""ctypes binding of libgtc.so (the C ABI in include/gtc.h).

The library is built in-tree by ``graph-tool-rs_gb300/build.py``; importing
this module never builds it.  A missing library is an ImportError: there is
no CPU fallback behind these bindings.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgtc.so")

GTC_OK = 0
GTC_ERR_ARG = 1
GTC_ERR_OOM = 2
GTC_ERR_CUDA = 3
GTC_ERR_TIMEOUT = 4
GTC_ERR_INDEX = 5
GTC_ERR_NO_DEVICE = 6

GTC_PREC_F32 = 0
GTC_PREC_F64_EXACT = 1

u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)


class PowerIteration(C.Structure):
    _fields_ = [("epsilon", C.c_double), ("max_iter", C.c_uint64),
                ("plan_len", C.c_uint64), ("plan_chunks", C.c_uint64)]


class View(C.Structure):
    _fields_ = [("reversed", C.c_int32), ("reserved", C.c_int32),
                ("vmask", u8p), ("vmask_len", C.c_uint64),
                ("emask", u8p), ("emask_len", C.c_uint64)]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("schedule", C.c_int32), ("stream", C.c_void_p),
                ("timing", C.c_int32), ("ppr_gather", C.c_int32)]


# gtc_schedule: the FP32 sweep kernels (every one computes the same values)
GTC_SCHED_AUTO = 0
GTC_SCHED_L1 = 1
GTC_SCHED_HOT32K = 2
GTC_SCHED_HOT24K = 3
GTC_SCHED_HOT16K = 4
GTC_SCHED_HOT8K = 5
SCHEDULES = {"auto": GTC_SCHED_AUTO, "l1": GTC_SCHED_L1, "hot32k": GTC_SCHED_HOT32K,
             "hot24k": GTC_SCHED_HOT24K, "hot16k": GTC_SCHED_HOT16K, "hot8k": GTC_SCHED_HOT8K}

# gtc_ppr_gather: the batched PPR gather kernels
GTC_PPR_BULK = 0
GTC_PPR_REGS = 1


class Result(C.Structure):
    _fields_ = [("iterations", C.c_uint64), ("last_delta", C.c_double),
                ("eigenvalue", C.c_double), ("device_ms", C.c_double),
                ("launches", C.c_uint64), ("sweep_ms", C.c_double),
                ("sweep_launches", C.c_uint64)]


GTC_F64 = 0
GTC_F32 = 1


class DVec(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("len", C.c_uint64), ("dtype", C.c_int32),
                ("reserved", C.c_int32)]

    @classmethod
    def of(cls, t):
        """A gtc_dvec over a contiguous CUDA tensor (float32/float64), or
        None for None."""
        if t is None:
            return None
        import torch
        assert t.is_cuda and t.is_contiguous(), "a contiguous CUDA tensor is required"
        dt = {torch.float64: GTC_F64, torch.float32: GTC_F32}[t.dtype]
        return cls(t.data_ptr(), t.numel(), dt, 0)


# every symbol include/gtc.h declares, with its ctypes signature
SIGNATURES = {
    "gtc_version": (C.c_char_p, []),
    "gtc_last_error": (C.c_char_p, []),
    "gtc_graph_create": (C.c_int, [C.c_uint64, C.c_uint64, u32p, u32p, C.POINTER(C.c_void_p)]),
    "gtc_graph_create_device": (C.c_int, [C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.POINTER(C.c_void_p)]),
    "gtc_graph_create_blocks": (C.c_int, [C.c_uint64, C.c_uint64, u64p, u32p, u32p,
                                          C.POINTER(C.c_void_p)]),
    "gtc_graph_destroy": (C.c_int, [C.c_void_p]),
    "gtc_graph_info": (C.c_int, [C.c_void_p, u64p, u64p, u64p]),
    "gtc_graph_export": (C.c_int, [C.c_void_p, u64p, u32p, u32p, u64p, u32p, u32p]),
    "gtc_graph_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gtc_pagerank": (C.c_int, [C.c_void_p, C.POINTER(View), f64p, C.c_uint64, f64p, C.c_uint64,
                               C.c_double, C.POINTER(PowerIteration), f64p, C.c_uint64,
                               C.c_uint64, C.POINTER(Options), C.POINTER(Result)]),
    "gtc_eigenvector": (C.c_int, [C.c_void_p, C.POINTER(View), f64p, C.c_uint64,
                                  C.POINTER(PowerIteration), f64p, C.c_uint64, C.c_uint64,
                                  C.POINTER(Options), C.POINTER(Result)]),
    "gtc_pagerank_device": (C.c_int, [C.c_void_p, C.POINTER(View), C.POINTER(DVec),
                                      C.POINTER(DVec), C.c_double, C.POINTER(PowerIteration),
                                      C.POINTER(DVec), C.c_uint64, C.POINTER(Options),
                                      C.POINTER(Result)]),
    "gtc_eigenvector_device": (C.c_int, [C.c_void_p, C.POINTER(View), C.POINTER(DVec),
                                         C.POINTER(PowerIteration), C.POINTER(DVec), C.c_uint64,
                                         C.POINTER(Options), C.POINTER(Result)]),
    "gtc_ppr_batch": (C.c_int, [C.c_void_p, C.POINTER(View), f64p, C.c_uint64, C.c_uint32, u64p,
                                u32p, f64p, C.c_double, C.POINTER(PowerIteration), f64p, u64p,
                                C.POINTER(Options), C.POINTER(Result)]),
    "gtc_ppr_batch_device": (C.c_int, [C.c_void_p, C.POINTER(View), C.POINTER(DVec), C.c_uint32,
                                       u64p, u32p, f64p, C.c_double, C.POINTER(PowerIteration),
                                       C.POINTER(DVec), u64p, C.POINTER(Options),
                                       C.POINTER(Result)]),
    "gtc_graph_batch_create": (C.c_int, [C.c_uint64, u64p, u64p, u32p, u32p,
                                         C.POINTER(C.c_void_p)]),
    "gtc_graph_batch_destroy": (C.c_int, [C.c_void_p]),
    "gtc_debug_set_batch_sweep_limit": (C.c_int, [C.c_uint64]),
    "gtc_graph_batch_info": (C.c_int, [C.c_void_p, u64p, u64p, u64p]),
    "gtc_pagerank_batch": (C.c_int, [C.c_void_p, f64p, C.c_uint64, C.c_double, C.c_double,
                                     C.c_uint64, f64p, C.c_uint64, u64p, C.POINTER(Options),
                                     C.POINTER(Result)]),
    "gtc_pagerank_batch_device": (C.c_int, [C.c_void_p, C.POINTER(DVec), C.c_double, C.c_double,
                                            C.c_uint64, C.POINTER(DVec), u64p, C.POINTER(Options),
                                            C.POINTER(Result)]),
    "gtc_pagerank_adjoint": (C.c_int, [C.c_void_p, C.POINTER(View), f64p, C.c_uint64, f64p,
                                       C.c_uint64, C.c_double, C.POINTER(PowerIteration), f64p,
                                       f64p, f64p, f64p, C.POINTER(Options), C.POINTER(Result)]),
    "gtc_pagerank_adjoint_device": (C.c_int, [C.c_void_p, C.POINTER(View), C.POINTER(DVec),
                                              C.POINTER(DVec), C.c_double,
                                              C.POINTER(PowerIteration), C.POINTER(DVec),
                                              C.POINTER(DVec), C.POINTER(DVec), C.POINTER(DVec),
                                              C.POINTER(Options), C.POINTER(Result)]),
    "gtc_pagerank_noalloc": (C.c_int, [C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_double, C.c_double, C.c_uint64, C.c_void_p,
                                       C.POINTER(C.c_uint64), C.c_void_p]),
    "gtc_weighted_degree": (C.c_int, [C.c_void_p, C.POINTER(View), C.c_int32, f64p, C.c_uint64,
                                      f64p, C.c_uint64, C.POINTER(Options)]),
    "gtc_betweenness": (C.c_int, [C.c_void_p, C.POINTER(View), C.c_int32, f64p, C.c_uint64, f64p,
                                  C.c_uint64, C.POINTER(Options), C.POINTER(Result)]),
    "gtc_gt_open": (C.c_int, [C.c_char_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "gtc_gt_close": (C.c_int, [C.c_void_p]),
    "gtc_gt_info": (C.c_int, [C.c_void_p, u64p, u64p, C.POINTER(C.c_int32),
                              C.POINTER(C.c_int32), u64p]),
    "gtc_gt_comment": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), u64p]),
    "gtc_gt_property": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p), u64p,
                                  C.POINTER(C.c_int32), C.POINTER(C.c_int32), u64p]),
    "gtc_gt_property_f64": (C.c_int, [C.c_void_p, C.c_uint64, f64p, C.c_uint64]),
    "gtc_gt_property_bytes": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p), u64p]),
    "gtc_gt_graph": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
}

_lib = None


def lib():
    """Load libgtc.so (raises ImportError if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libgtc.so is not built ({LIB_PATH}); run graph-tool-rs_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class GtcError(RuntimeError):
    pass


def check(status: int) -> None:
    """Map a gtc_status to the exception class of the reference's Python
    boundary (crates/gt-py/src/module.rs:78-114)."""
    if status == GTC_OK:
        return
    msg = lib().gtc_last_error().decode(errors="replace")
    if status == GTC_ERR_ARG:
        raise ValueError(msg)
    if status == GTC_ERR_INDEX:
        raise IndexError(msg)
    if status == GTC_ERR_OOM:
        raise MemoryError(msg)
    raise GtcError(f"[gtc status {status}] {msg}")


def ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)

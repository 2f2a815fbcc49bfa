"""Catalog I/O (``baorec_read_ascii``, ``baorec_write_npy``): the reference's
examples read whitespace-delimited catalogs with CSV.jl
(``examples/lightcone.jl:22-23``, ``examples/simulation.jl:13``) and write
the shifted positions with ``npzwrite(path, hcat(x, y, z))``
(``examples/simulation.jl:38-40``)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib

F32 = np.float32


def _ctx_handle(ctx):
    return None if ctx is None else ctx.h


def _call(ctx, name, *args):
    lib = _lib.load()
    _lib.check(_ctx_handle(ctx), getattr(lib, name)(_ctx_handle(ctx), *args))


def read_ascii(path, usecols, skip=0, comment="#", device=False, ctx=None):
    """Columns ``usecols`` (0-based) of a whitespace-delimited ASCII catalog
    as FP32 arrays (NumPy, or CUDA torch tensors with ``device=True``)."""
    cols = np.ascontiguousarray(usecols, np.int32)
    cm = 0 if not comment else ord(comment)
    p = os.fsencode(path)
    n = C.c_int64()
    _call(ctx, "baorec_read_ascii", p, cols.ctypes.data, len(cols), int(skip), cm, None, 0, C.byref(n), _lib.HOST)
    rows = n.value
    if device:
        import torch
        from .recon import _prim_ctx
        c = ctx if ctx is not None else _prim_ctx((2, 2, 2), [1.0] * 3, [0.0] * 3)
        outs = [torch.empty(max(rows, 1), device="cuda", dtype=torch.float32) for _ in cols]
        ptrs = (C.c_void_p * len(cols))(*[o.data_ptr() for o in outs])
        torch.cuda.synchronize()
        _call(c, "baorec_read_ascii", p, cols.ctypes.data, len(cols), int(skip), cm, ptrs, rows, C.byref(n), 0)
        return [o[:rows] for o in outs]
    outs = [np.empty(max(rows, 1), F32) for _ in cols]
    ptrs = (C.c_void_p * len(cols))(*[o.ctypes.data for o in outs])
    _call(ctx, "baorec_read_ascii", p, cols.ctypes.data, len(cols), int(skip), cm, ptrs, rows, C.byref(n), _lib.HOST)
    return [o[:rows] for o in outs]


def write_npy(path, columns, ctx=None):
    """Write equal-length FP32 columns (NumPy arrays or CUDA torch tensors)
    as an (n, ncols) float32 .npy file, the layout ``npzwrite`` gives
    ``hcat(x, y, z)``."""
    cols = list(columns)
    if not cols:
        raise ValueError("write_npy: no columns")
    n = int(len(cols[0]))
    if any(int(len(c)) != n for c in cols):
        raise ValueError("write_npy: columns of different lengths")
    p = os.fsencode(path)
    dev = False
    try:
        import torch
        dev = isinstance(cols[0], torch.Tensor) and cols[0].is_cuda
    except ImportError:
        pass
    if dev:
        from .recon import _prim_ctx
        c = ctx if ctx is not None else _prim_ctx((2, 2, 2), [1.0] * 3, [0.0] * 3)
        keep = [t.contiguous().float() for t in cols]
        ptrs = (C.c_void_p * len(keep))(*[t.data_ptr() for t in keep])
        torch.cuda.synchronize()
        _call(c, "baorec_write_npy", p, ptrs, len(keep), n, 0)
        return
    keep = [np.ascontiguousarray(c, F32) for c in cols]
    ptrs = (C.c_void_p * len(keep))(*[a.ctypes.data for a in keep])
    _call(ctx, "baorec_write_npy", p, ptrs, len(keep), n, _lib.HOST)

"""Ensemble statistics on the device (sgs_ensemble_*, include/geosgs.h).

The reference reduces an Ensemble node by node (src/ensembles.jl:42-52,
76-85): mean, var, cdf, ccdf, quantile.  Here the realizations stay in HBM in
the node-major layout the sweep writes (`Plan.simulate_device`,
`Batch.simulate_device`: a CUDA tensor of N rows of `stride` values, the
first `nreals` of each row used, centred), and the statistics are computed
there; `offset` (the process mean) is added to every value.  Results are
float64 CUDA tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi


def _prec(vals):
    import torch

    if vals.dtype == torch.float32:
        return _abi.SGS_PREC_FP32_REFINE
    if vals.dtype == torch.float64:
        return _abi.SGS_PREC_FP64
    raise ValueError("values must be float32 or float64")


def _shape(vals, nreals, stride):
    n = vals.numel() // stride
    if vals.numel() != n * stride or nreals > stride or not vals.is_cuda or not vals.is_contiguous():
        raise ValueError("values must be a contiguous CUDA tensor of N x stride elements")
    return n


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def mean_var(vals, nreals: int, stride: int | None = None, offset: float = 0.0):
    """Per-node mean and variance (n - 1 divisor) over nreals realizations."""
    import torch

    stride = stride or nreals
    n = _shape(vals, nreals, stride)
    m = torch.empty(n, dtype=torch.float64, device=vals.device)
    v = torch.empty(n, dtype=torch.float64, device=vals.device)
    lib = _abi.load_library()
    _abi.check(lib, lib.sgs_ensemble_stats(C.c_void_p(vals.data_ptr()), _prec(vals), n, nreals, stride,
                                           float(offset), C.c_void_p(m.data_ptr()), C.c_void_p(v.data_ptr()),
                                           _stream(torch)))
    return m, v


def cdf(vals, nreals: int, x, stride: int | None = None, offset: float = 0.0, complement: bool = False):
    """Per-node fraction of realizations <= x[i] (or > x[i]): N x len(x)."""
    import torch

    stride = stride or nreals
    n = _shape(vals, nreals, stride)
    xs = np.ascontiguousarray(np.atleast_1d(np.asarray(x, dtype=np.float64)))
    out = torch.empty((n, xs.size), dtype=torch.float64, device=vals.device)
    lib = _abi.load_library()
    _abi.check(lib, lib.sgs_ensemble_cdf(C.c_void_p(vals.data_ptr()), _prec(vals), n, nreals, stride, float(offset),
                                         xs.ctypes.data_as(C.POINTER(C.c_double)), xs.size, 1 if complement else 0,
                                         C.c_void_p(out.data_ptr()), _stream(torch)))
    return out


def quantile(vals, nreals: int, p, stride: int | None = None, offset: float = 0.0):
    """Per-node quantiles (linear interpolation between order statistics,
    the reference's Statistics.quantile default): N x len(p)."""
    import torch

    stride = stride or nreals
    n = _shape(vals, nreals, stride)
    ps = np.ascontiguousarray(np.atleast_1d(np.asarray(p, dtype=np.float64)))
    out = torch.empty((n, ps.size), dtype=torch.float64, device=vals.device)
    lib = _abi.load_library()
    _abi.check(lib, lib.sgs_ensemble_quantile(C.c_void_p(vals.data_ptr()), _prec(vals), n, nreals, stride,
                                              float(offset), ps.ctypes.data_as(C.POINTER(C.c_double)), ps.size,
                                              C.c_void_p(out.data_ptr()), _stream(torch)))
    return out

"""Translate (process, domain, data, method) into the C struct sgs_problem.

This mirrors what preprocess(rng, process, ::SEQSIM, init, domain, data)
(src/simulation/field/seqsim.jl:50-70) derives from the same objects: the
search neighbourhood (`:range`, a MetricBall or nothing, seqsim.jl:171-177,
221-227), min/max neighbours, the data appended after the grid nodes
(seqsim.jl:211-218, 267-271) and the path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .model import ArgumentError, CartesianGrid, GaussianProcess, GeoTable, IndicatorProcess, MetricBall, path_order

_PREC = {"fp64": _abi.SGS_PREC_FP64, "fp32": _abi.SGS_PREC_FP32_REFINE}


def indicator_levels(process: IndicatorProcess, data: GeoTable | None):
    """(levels, data categories): the categories are the data's distinct
    values in sorted order (the one-hot transform, seqsim.jl:247-249), or
    1..L without data (seqsim.jl:253-261); categories are 0-based indices."""
    L = len(process.prob)
    if data is None or data.nrow() == 0:
        return list(range(1, L + 1)), np.zeros(0, dtype=np.int32)
    col = np.asarray(next(iter(data.values.values())))
    levels, cat = np.unique(col, return_inverse=True)
    if len(levels) != L:
        raise ArgumentError(f"probabilities must have {len(levels)} components, received {L}")
    return list(levels), cat.astype(np.int32)


def multivariate_data(process: GaussianProcess, data: GeoTable | None) -> np.ndarray:
    """The data's values of a multivariate process, D x L (columns in table
    order, one per variable)."""
    L = process.nvariables
    if data is None or data.nrow() == 0:
        return np.zeros((0, L))
    cols = [np.asarray(v, dtype=np.float64) for v in data.values.values()]
    if len(cols) != L:
        raise ArgumentError(f"the data must have {L} variable(s), one per variable of the process")
    return np.ascontiguousarray(np.stack(cols, axis=1))


def build_problem(process, domain: CartesianGrid, data: GeoTable | None, method):
    """Return (sgs_problem, keepalive) — keepalive owns the arrays it points to.
    An IndicatorProcess becomes the problem of its common correlogram, with
    the data's category indices as data values."""
    if not isinstance(process, (GaussianProcess, IndicatorProcess)):
        raise ArgumentError("the GPU SEQSIM path simulates GaussianProcess and IndicatorProcess")
    if not isinstance(domain, CartesianGrid):
        raise ArgumentError("the GPU SEQSIM path simulates on a CartesianGrid")
    # A 1D grid of n cells runs as the n x 1 grid with unit spacing across and
    # the data on the row's centre line (second coordinate 0.5, the cells'
    # centroid): every lag's second component is exactly 0, so distances,
    # neighbour order and covariances are those of the 1D problem.
    dim = domain.dim
    flat = dim == 1
    cdim = 2 if flat else dim
    p = _abi.SgsProblem()
    p.dim = cdim
    for j in range(3):
        p.dims[j] = domain.dims[j] if j < dim else 1
        p.origin[j] = domain.origin[j] if j < dim else 0.0
        p.spacing[j] = domain.spacing[j] if j < dim else 1.0
    keep = []
    if data is not None and data.nrow() > 0:
        if data.coords.shape[1] != dim:
            raise ArgumentError("data coordinates do not match the domain's dimension")
        nv = process.nvariables if isinstance(process, GaussianProcess) else 1
        if len(data.values) != nv:
            raise ArgumentError(f"the data must have {nv} variable(s), one per variable of the process")
        xy = np.ascontiguousarray(data.coords, dtype=np.float64)
        if flat:
            xy = np.ascontiguousarray(np.column_stack([xy[:, 0], np.full(xy.shape[0], 0.5)]))
        if isinstance(process, IndicatorProcess):
            val = np.ascontiguousarray(indicator_levels(process, data)[1], dtype=np.float64)
        else:
            val = np.ascontiguousarray(next(iter(data.values.values())), dtype=np.float64)
        keep += [xy, val]
        p.ndata = xy.shape[0]
        p.data_coords = xy.ctypes.data_as(C.POINTER(C.c_double))
        p.data_values = val.ctypes.data_as(C.POINTER(C.c_double))
    else:
        p.ndata = 0
    func = process.corr if isinstance(process, IndicatorProcess) else process.func
    st = func.structures()
    p.variogram = st[0].to_c(cdim)
    if len(st) > 1:  # further structures of a nested model
        more = (_abi.SgsVariogram * (len(st) - 1))(*[g.to_c(cdim) for g in st[1:]])
        keep.append(more)
        p.nstructures = len(st) - 1
        p.structures = C.cast(more, C.POINTER(_abi.SgsVariogram))
    # a multivariate process keeps its means beside the plan (sgs_plan_set_multivariate)
    p.mean = process.mean if np.ndim(process.mean) == 0 else 0.0
    p.minneighbors = int(method.minneighbors)
    p.maxneighbors = int(method.maxneighbors)
    nb = method.neighborhood
    if isinstance(nb, str) and nb == "range":
        p.search = _abi.SGS_SEARCH_RANGE
    elif nb is None:
        p.search = _abi.SGS_SEARCH_NEAREST
    elif isinstance(nb, MetricBall):
        p.search = _abi.SGS_SEARCH_BALL
        for j, r in enumerate(nb.padded_radii(cdim)):
            p.ball.radii[j] = r
        for i in range(3):
            for j in range(3):
                p.ball.rotation[i + 3 * j] = nb.rotation[i, j]
    else:
        raise ArgumentError("neighborhood must be 'range', a MetricBall or None")
    if getattr(method, "distance", "euclidean") not in ("euclidean", None):
        raise ArgumentError("only the Euclidean distance is supported")
    prec = getattr(method, "precision", "fp32")
    if prec not in _PREC:
        raise ArgumentError("precision must be 'fp32' or 'fp64'")
    p.precision = _PREC[prec]
    p.refine_steps = int(getattr(method, "refine_steps", 2))
    p.warm_start = 1 if getattr(method, "warm_start", False) else 0
    p.device = int(getattr(method, "device", 0))
    p.flags = ((_abi.SGS_FLAG_ONE_LAUNCH_SWEEP if getattr(method, "one_launch_sweep", False) else 0)
               | (_abi.SGS_FLAG_LEVEL_SWEEP if getattr(method, "level_sweep", False) else 0))
    perm = path_order(domain, method.path)
    if perm is not None:
        perm = np.ascontiguousarray(perm, dtype=np.int32)
        keep.append(perm)
        p.path = perm.ctypes.data_as(C.POINTER(C.c_int32))
    keep.append(perm)
    return p, keep


def clamped_neighbors(method, nnodes: int):
    """(nmin, nmax) after the reference's clamps, seqsim.jl:202-208."""
    nmax, nmin = int(method.maxneighbors), int(method.minneighbors)
    if nmax > nnodes or nmax < 1:
        nmax = nnodes
    if nmin > nmax or nmin < 1:
        nmin = 1
    return nmin, nmax

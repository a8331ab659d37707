import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "geostatsprocesses.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, ROOT)  # bench.py (the throughput probes' build)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgeosgs.so")


def golden_cases():
    return sorted(f[len("golden_"):-4] for f in os.listdir(GOLDEN) if f.startswith("golden_") and f.endswith(".npz"))


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, f"golden_{name}.npz")))


def golden_problem(g, precision=0):
    """sgs_problem of a golden fixture; returns (problem, keepalive)."""
    from geosgs import _abi

    p = _abi.SgsProblem()
    dim = int(g["dim"])
    p.dim = dim
    for j in range(3):
        p.dims[j] = int(g["dims"][j]) if j < dim else 1
        p.origin[j] = float(g["origin"][j]) if j < dim else 0.0
        p.spacing[j] = float(g["spacing"][j]) if j < dim else 1.0
    xyz = np.ascontiguousarray(g["data_xyz"], dtype=np.float64)
    val = np.ascontiguousarray(g["data_val"], dtype=np.float64)
    p.ndata = xyz.shape[0]
    p.data_coords = xyz.ctypes.data_as(C.POINTER(C.c_double))
    p.data_values = val.ctypes.data_as(C.POINTER(C.c_double))
    p.variogram.type = int(g["vario_type"])
    p.variogram.sill = float(g["sill"])
    p.variogram.nugget = float(g["nugget"])
    for j in range(3):
        p.variogram.ranges[j] = float(g["ranges"][j])
    for i in range(3):
        for j in range(3):
            p.variogram.rotation[i + 3 * j] = float(g["vario_R"][i, j])
            p.ball.rotation[i + 3 * j] = float(g["search_R"][i, j])
    for j in range(3):
        p.ball.radii[j] = float(g["search_radii"][j])
    kind = str(g["search_kind"])
    p.search = {"iso": _abi.SGS_SEARCH_BALL, "ellipsoid": _abi.SGS_SEARCH_BALL,
                "nearest": _abi.SGS_SEARCH_NEAREST}[kind]
    p.mean = float(g["mean"])
    p.minneighbors = int(g["nmin"])
    p.maxneighbors = int(g["k"])
    path = np.ascontiguousarray(g["path"], dtype=np.int32)
    p.path = path.ctypes.data_as(C.POINTER(C.c_int32))
    p.precision = precision
    p.refine_steps = 2
    return p, (xyz, val, path)


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    oracle.build()
    return oracle


def has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def geosgs_lib():
    """The built CUDA library (build() first); GPU tests only."""
    import geosgs
    from geosgs import _build

    _build.build()
    return geosgs.load_library()

"""Seeded synthetic SGS workloads (grids, data, variograms, paths).

No public dataset is involved: every input is drawn from numpy's PCG64 with
the stated seed.  Coordinates are cell units with origin 0 and unit spacing.

  c1  2D 100x100, spherical (sill 1, range 20), isotropic ball r=40, k=12,
      RandomPath seed 0, unconditional, 4 realizations
  c2  2D 500x500, 1,000 data at distinct random cell centres (seed 1, values
      N(0,1)), gaussian (sill 1, range 30, nugget 0.01), :range ball, k=32,
      RandomPath seed 2, 64 realizations
  c3  3D 200x200x100, 5,000 data uniform in the box (seed 3, values N(0,1)),
      exponential (sill 1, ranges 50/25/5, 30 deg RotZ, nugget 0.05), search
      ellipsoid = the variogram's, k=48, RandomPath seed 4, 256 realizations
  c4  3D 256x256x256 (16.8M nodes), unconditional, spherical (sill 1, ranges
      40/20/8, 30 deg RotZ, nugget 0.1: one draw inside the warm-start
      network's training distribution), search ellipsoid = the variogram's,
      k=32, RandomPath seed 5, 64 realizations (the learned warm start's
      evaluation run)
  c5  a batch of 1,000 independent domains (seed 6): 2D or 3D with equal
      odds, sides uniform in [32, 256] cells (3D depth in [8, 64]), each its
      own variogram (spherical / exponential / gaussian with equal odds,
      isotropic range uniform in [5, 80] cells, nugget uniform in [0, 0.1],
      sill 1), 0-500 data uniform in the box with N(0,1) values, :range
      neighbourhood, maxneighbors drawn from {8, 16, 32, 48}, its own
      RandomPath, 8 realizations
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any

import numpy as np

from .model import (CartesianGrid, ExponentialVariogram, GaussianProcess, GaussianVariogram,
                    MetricBall, RandomPath, RotZ, SphericalVariogram, georef)
from .simulation import GPUSEQSIM


@dataclass
class Workload:
    name: str
    process: GaussianProcess
    domain: CartesianGrid
    data: Any
    method: GPUSEQSIM
    nreals: int


def c1(precision: str = "fp64") -> Workload:
    grid = CartesianGrid((100, 100))
    proc = GaussianProcess(SphericalVariogram(range=20.0, sill=1.0), 0.0)
    m = GPUSEQSIM(path=RandomPath(0), maxneighbors=12, neighborhood=MetricBall(40.0), precision=precision)
    return Workload("c1_2d_100x100_sph_k12", proc, grid, None, m, 4)


def c2(precision: str = "fp32", nreals: int = 64) -> Workload:
    grid = CartesianGrid((500, 500))
    rng = np.random.default_rng(1)
    cells = rng.choice(grid.nelements(), 1000, replace=False)
    xy = grid.centroids()[cells]
    vals = rng.standard_normal(1000)
    data = georef({"Z": vals}, xy)
    proc = GaussianProcess(GaussianVariogram(range=30.0, sill=1.0, nugget=0.01), 0.0)
    m = GPUSEQSIM(path=RandomPath(2), maxneighbors=32, neighborhood="range", precision=precision)
    return Workload("c2_2d_500x500_gau_d1000_k32", proc, grid, data, m, nreals)


def c3(precision: str = "fp32", nreals: int = 256, dims=(200, 200, 100), ndata: int = 5000) -> Workload:
    grid = CartesianGrid(tuple(dims))
    rng = np.random.default_rng(3)
    ext = np.asarray(dims, dtype=np.float64)
    xyz = rng.uniform(0.0, 1.0, (ndata, 3)) * ext
    vals = rng.standard_normal(ndata)
    data = georef({"Z": vals}, xyz)
    ball = MetricBall((50.0, 25.0, 5.0), RotZ(30.0))
    proc = GaussianProcess(ExponentialVariogram(ball, sill=1.0, nugget=0.05), 0.0)
    m = GPUSEQSIM(path=RandomPath(4), maxneighbors=48, neighborhood=ball, precision=precision)
    name = "c3_3d_%dx%dx%d_exp_aniso_d%d_k48" % (*dims, ndata)
    return Workload(name, proc, grid, data, m, nreals)


def c4(precision: str = "fp32", nreals: int = 64, dims=(256, 256, 256)) -> Workload:
    grid = CartesianGrid(tuple(dims))
    ball = MetricBall((40.0, 20.0, 8.0), RotZ(30.0))
    proc = GaussianProcess(SphericalVariogram(ball, sill=1.0, nugget=0.1), 0.0)
    m = GPUSEQSIM(path=RandomPath(5), maxneighbors=32, neighborhood=ball, precision=precision)
    name = "c4_3d_%dx%dx%d_sph_aniso_uncond_k32" % tuple(dims)
    return Workload(name, proc, grid, None, m, nreals)


def small(dim=2, n=24, k=8, ndata=0, vario="sph", seed=0, nugget=0.0, ranges=(6.0, 6.0, 6.0),
          rotation=None, ball=None, precision="fp64", nreals=4, path="random", nz=5) -> Workload:
    """A small case for parity tests (oracle in seconds)."""
    dims = (n, n) if dim == 2 else (n, n, nz)
    grid = CartesianGrid(dims)
    rng = np.random.default_rng(100 + seed)
    data = None
    if ndata:
        xyz = rng.uniform(0.0, 1.0, (ndata, dim)) * np.asarray(dims, dtype=np.float64)
        data = georef({"Z": rng.standard_normal(ndata)}, xyz)
    cls = {"sph": SphericalVariogram, "exp": ExponentialVariogram, "gau": GaussianVariogram}[vario]
    vb = MetricBall(tuple(ranges[:dim]), rotation)
    proc = GaussianProcess(cls(vb, sill=1.0, nugget=nugget), 0.0)
    p = RandomPath(seed) if path == "random" else path
    m = GPUSEQSIM(path=p, maxneighbors=k, neighborhood=ball if ball is not None else "range",
                  precision=precision)
    return Workload(f"small{dim}d_{n}_{vario}_k{k}", proc, grid, data, m, nreals)


@dataclass
class BatchWorkload:
    """Independent domains simulated together (one Workload per domain)."""

    name: str
    items: list = field(default_factory=list)
    nreals: int = 8

    def nodes(self) -> int:
        return int(sum(w.domain.nelements() for w in self.items))


def c5(precision: str = "fp32", nreals: int = 8, ndomains: int = 1000, seed: int = 6, sides=(32, 256),
       depth=(8, 64), ranges=(5.0, 80.0), nugget=(0.0, 0.1), ndata=(0, 500), ks=(8, 16, 32, 48),
       name: str | None = None) -> BatchWorkload:
    """The uneven batch; the keyword ranges shrink it for parity tests."""
    rng = np.random.default_rng(seed)
    classes = (SphericalVariogram, ExponentialVariogram, GaussianVariogram)
    items = []
    for d in range(ndomains):
        dim = 3 if rng.random() < 0.5 else 2
        dims = [int(rng.integers(sides[0], sides[1] + 1)) for _ in range(2)]
        if dim == 3:
            dims.append(int(rng.integers(depth[0], depth[1] + 1)))
        grid = CartesianGrid(tuple(dims))
        cls = classes[int(rng.integers(0, 3))]
        rg = float(rng.uniform(*ranges))
        nug = float(rng.uniform(*nugget))
        nd = int(rng.integers(ndata[0], ndata[1] + 1))
        data = None
        if nd:
            xyz = rng.uniform(0.0, 1.0, (nd, dim)) * np.asarray(dims, dtype=np.float64)
            data = georef({"Z": rng.standard_normal(nd)}, xyz)
        k = int(ks[int(rng.integers(0, len(ks)))])
        proc = GaussianProcess(cls(range=rg, sill=1.0, nugget=nug), 0.0)
        m = GPUSEQSIM(path=RandomPath(seed * 1000003 + d), maxneighbors=k, neighborhood="range",
                      precision=precision)
        items.append(Workload("c5_domain%d" % d, proc, grid, data, m, nreals))
    nm = name or "c5_batch_%d_domains_2d3d_sides%d-%d_depth%d-%d_k8-48" % (ndomains, sides[0], sides[1],
                                                                           depth[0], depth[1])
    return BatchWorkload(nm, items, nreals)


def c5_small(precision: str = "fp32", nreals: int = 8, ndomains: int = 12, seed: int = 60) -> BatchWorkload:
    """A small uneven batch for parity tests (oracle in seconds)."""
    return c5(precision, nreals, ndomains, seed, sides=(8, 40), depth=(3, 9), ranges=(3.0, 12.0),
              nugget=(0.0, 0.1), ndata=(0, 40), ks=(8, 16, 32, 48), name="c5_small_%d_domains" % ndomains)

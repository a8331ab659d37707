"""ctypes wrapper of the FP64 CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product path never imports
it.  Parity status of the oracle itself: partially pinned (see sgs_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

BRUTE = 0
TEMPLATE = 1

_lib = None


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (g++, OpenMP)."""
    subprocess.run(["make", "-C", HERE], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    lib = C.CDLL(LIB)
    P = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int32)
    lib.oracle_create.argtypes = [C.c_void_p, C.POINTER(P)]
    lib.oracle_destroy.argtypes = [P]
    lib.oracle_destroy.restype = None
    lib.oracle_last_error.restype = C.c_char_p
    lib.oracle_search.argtypes = [P, C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_int]
    lib.oracle_solve.argtypes = [P, C.c_int64, C.c_int64, C.c_int64, C.c_int]
    lib.oracle_simulate.argtypes = [P, C.c_int32, dp, C.c_uint64, dp, C.c_int64, C.c_int]
    lib.oracle_krige.argtypes = [P, dp, dp, C.c_int]
    lib.oracle_simulate_indicator.argtypes = [P, C.c_int32, dp, ip, C.c_int32, dp, C.c_uint64, ip, C.c_int]
    lib.oracle_simulate_cokriging.argtypes = [P, C.c_int32, dp, ip, dp, C.c_int32, dp, C.c_uint64, ip, C.c_int]
    lib.oracle_simulate_multivariate.argtypes = [P, C.c_int32, dp, dp, dp, C.c_int32, dp, C.c_uint64, dp, C.c_int]
    lib.oracle_uniforms.argtypes = [C.c_uint64, C.c_int64, C.c_int32, dp]
    lib.oracle_uniforms.restype = None
    lib.oracle_neighbors.argtypes = [P, ip, ip]
    lib.oracle_weights.argtypes = [P, dp, dp, ip]
    lib.oracle_levels.argtypes = [P, ip, ip]
    lib.oracle_template_size.argtypes = [P]
    lib.oracle_normals.argtypes = [C.c_uint64, C.c_int64, C.c_int32, dp]
    lib.oracle_normals.restype = None
    lib.oracle_covariance.argtypes = [C.c_void_p, C.c_int32, dp]
    lib.oracle_covariance.restype = C.c_double
    _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class OraclePlan:
    """One problem on the CPU oracle; arrays are node-indexed like the library's."""

    def __init__(self, problem, keepalive=None):
        self.lib = load()
        self._keep = keepalive
        self.N = int(np.prod([problem.dims[j] for j in range(problem.dim)]))
        self.D = int(problem.ndata)
        h = C.c_void_p()
        rc = self.lib.oracle_create(C.byref(problem), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle_create: {self.lib.oracle_last_error().decode()}")
        self.h = h
        nmax = int(problem.maxneighbors)
        if nmax > self.N or nmax < 1:
            nmax = self.N
        self.k = nmax

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oracle_destroy(self.h)
            self.h = None

    def _rc(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.oracle_last_error().decode())

    def search(self, method=TEMPLATE, t0=0, t1=None, stride=1, nthreads=0):
        self._rc(self.lib.oracle_search(self.h, method, t0, self.N if t1 is None else t1, stride, nthreads))

    def solve(self, t0=0, t1=None, stride=1, nthreads=0):
        self._rc(self.lib.oracle_solve(self.h, t0, self.N if t1 is None else t1, stride, nthreads))

    def prepare(self, method=TEMPLATE, nthreads=0):
        self.search(method, nthreads=nthreads)
        self.solve(nthreads=nthreads)
        return self

    def simulate(self, nreals, z=None, seed=0, t_end=None, nthreads=0):
        out = np.empty((nreals, self.N), dtype=np.float64)
        zp = None
        if z is not None:
            z = np.ascontiguousarray(z, dtype=np.float64).reshape(nreals, self.N)
            zp = _dp(z)
        self._rc(self.lib.oracle_simulate(self.h, nreals, zp, seed, _dp(out),
                                          self.N if t_end is None else t_end, nthreads))
        return out

    def krige(self, nthreads=0):
        """Posterior (mean, var) by simple kriging from the data alone."""
        m = np.empty(self.N, dtype=np.float64)
        v = np.empty(self.N, dtype=np.float64)
        self._rc(self.lib.oracle_krige(self.h, _dp(m), _dp(v), nthreads))
        return m, v

    def simulate_indicator(self, nreals, prob, data_cat=None, u=None, seed=0, nthreads=0):
        """nreals x N categories (sequential indicator simulation)."""
        prob = np.ascontiguousarray(np.asarray(prob, dtype=np.float64))
        dc = np.ascontiguousarray(np.asarray(data_cat if data_cat is not None else np.zeros(1), dtype=np.int32))
        out = np.empty((nreals, self.N), dtype=np.int32)
        up = None
        if u is not None:
            u = np.ascontiguousarray(u, dtype=np.float64).reshape(nreals, self.N)
            up = _dp(u)
        self._rc(self.lib.oracle_simulate_indicator(self.h, len(prob), _dp(prob), _ip(dc), nreals, up, seed,
                                                    _ip(out), nthreads))
        return out

    def simulate_cokriging(self, nreals, prob, coef, data_cat=None, u=None, seed=0, nthreads=0):
        """nreals x N categories by full simple cokriging of the indicators
        (linear model of coregionalization, coef: S x L x L)."""
        prob = np.ascontiguousarray(np.asarray(prob, dtype=np.float64))
        coef = np.ascontiguousarray(np.asarray(coef, dtype=np.float64))
        dc = np.ascontiguousarray(np.asarray(data_cat if data_cat is not None else np.zeros(1), dtype=np.int32))
        out = np.empty((nreals, self.N), dtype=np.int32)
        up = None
        if u is not None:
            u = np.ascontiguousarray(u, dtype=np.float64).reshape(nreals, self.N)
            up = _dp(u)
        self._rc(self.lib.oracle_simulate_cokriging(self.h, len(prob), _dp(prob), _ip(dc), _dp(coef), nreals, up,
                                                    seed, _ip(out), nthreads))
        return out

    def simulate_multivariate(self, nreals, mean, coef, data_values=None, z=None, seed=0, nthreads=0):
        """nreals x L x N values of a multivariate Gaussian process (linear
        model of coregionalization, coef: S x L x L; data_values: D x L)."""
        mean = np.ascontiguousarray(np.asarray(mean, dtype=np.float64).reshape(-1))
        L = mean.size
        coef = np.ascontiguousarray(np.asarray(coef, dtype=np.float64))
        dv = np.ascontiguousarray(np.asarray(data_values if data_values is not None else np.zeros(1),
                                             dtype=np.float64))
        out = np.empty((nreals, L, self.N), dtype=np.float64)
        zp = None
        if z is not None:
            z = np.ascontiguousarray(z, dtype=np.float64).reshape(nreals, L, self.N)
            zp = _dp(z)
        self._rc(self.lib.oracle_simulate_multivariate(self.h, L, _dp(mean), _dp(coef), _dp(dv), nreals, zp, seed,
                                                       _dp(out), nthreads))
        return out

    def neighbors(self):
        idx = np.empty((self.N, self.k), dtype=np.int32)
        cnt = np.empty(self.N, dtype=np.int32)
        self._rc(self.lib.oracle_neighbors(self.h, _ip(idx), _ip(cnt)))
        return idx, cnt

    def weights(self):
        w = np.empty((self.N, self.k), dtype=np.float64)
        s = np.empty(self.N, dtype=np.float64)
        st = np.empty(self.N, dtype=np.int32)
        self._rc(self.lib.oracle_weights(self.h, _dp(w), _dp(s), _ip(st)))
        return w, s, st

    def levels(self):
        lv = np.empty(self.N, dtype=np.int32)
        n = C.c_int32()
        self._rc(self.lib.oracle_levels(self.h, _ip(lv), C.byref(n)))
        return lv, int(n.value)

    def template_size(self):
        return int(self.lib.oracle_template_size(self.h))


def normals(seed: int, nnodes: int, nreals: int) -> np.ndarray:
    z = np.empty((nreals, nnodes), dtype=np.float64)
    load().oracle_normals(seed, nnodes, nreals, _dp(z))
    return z


def uniforms(seed: int, nnodes: int, nreals: int) -> np.ndarray:
    u = np.empty((nreals, nnodes), dtype=np.float64)
    load().oracle_uniforms(seed, nnodes, nreals, _dp(u))
    return u


def covariance(variogram_c, dim, lag) -> float:
    lag = np.ascontiguousarray(np.asarray(lag, dtype=np.float64).reshape(-1))
    if lag.size < 3:
        lag = np.concatenate([lag, np.zeros(3 - lag.size)])
    return float(load().oracle_covariance(C.byref(variogram_c), dim, _dp(lag)))

"""Python handle on a libgeosgs plan (the C-ABI in include/geosgs.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _device_values(vals, nnodes: int, nreals: int, fp64: bool):
    """Pointer of a device value array: an int is taken as is; a tensor (any
    object with data_ptr / element_size / numel) must hold nnodes rows of
    nreals rounded up to 4 values of the sweep's value type."""
    if isinstance(vals, int):
        return vals
    rp = (nreals + 3) // 4 * 4
    es = 8 if fp64 else 4
    if vals.element_size() != es or vals.numel() < nnodes * rp:
        raise ValueError(f"device values must be {nnodes} x {rp} {'float64' if fp64 else 'float32'} elements")
    return vals.data_ptr()


class Plan:
    """Owns one sgs_plan: geometry, neighbour/weight tables and the sweep schedule
    on the GPU.  `prepare()` runs the neighbour search, the level schedule and
    the kriging solves; `simulate()` runs the batched sweep."""

    def __init__(self, problem: _abi.SgsProblem, keepalive=None):
        self.lib = _abi.load_library()
        self._keep = keepalive
        h = C.c_void_p()
        _abi.check(self.lib, self.lib.sgs_plan_create(C.byref(problem), C.byref(h)))
        self.h = h
        self.dim = int(problem.dim)
        self.N = int(np.prod([problem.dims[j] for j in range(self.dim)]))
        info = self.info()
        self.k = int(info.maxneighbors)
        self.prepared = False
        self._sweep = _abi.SgsSweepConfig(2 if problem.flags & _abi.SGS_FLAG_LEVEL_SWEEP else
                                          1 if problem.flags & _abi.SGS_FLAG_ONE_LAUNCH_SWEEP else 0,
                                          1, 0, 1, 0, 0, 0, 0, 0, 0.0).as_dict()

    def close(self):
        if getattr(self, "h", None):
            self.lib.sgs_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        return _abi.check(self.lib, rc, self.h)

    def prepare(self):
        self._check(self.lib.sgs_plan_prepare(self.h))
        self.prepared = True
        return self

    def simulate(self, nreals: int, z=None, seed: int = 0) -> np.ndarray:
        """nreals x N realization-major FP64 array of simulated values."""
        out = np.empty((nreals, self.N), dtype=np.float64)
        zp = None
        if z is not None:
            z = np.ascontiguousarray(np.asarray(z, dtype=np.float64).reshape(nreals, self.N))
            zp = _dp(z)
        self._check(self.lib.sgs_plan_simulate(self.h, nreals, zp, C.c_uint64(seed), _dp(out)))
        return out

    def values_fp64(self) -> bool:
        """Whether the sweep keeps FP64 values (sgs_info.values_fp64): FP64
        precision, or FP32 refinement whose weights amplify FP32 rounding."""
        return bool(self.info().values_fp64)

    def simulate_device(self, nreals: int, z_ptr: int | None, seed: int, vals, stream: int | None = None):
        """Sweep into device memory: `vals` is a device pointer or a CUDA
        tensor of N x (nreals rounded up to 4) values of the sweep's type
        (values_fp64()); tensors are checked."""
        ptr = _device_values(vals, self.N, nreals, self.values_fp64())
        self._check(self.lib.sgs_plan_simulate_device(
            self.h, nreals, C.c_void_p(z_ptr) if z_ptr else None, C.c_uint64(seed),
            C.c_void_p(ptr), C.c_void_p(stream) if stream else None))

    def neighbors(self):
        idx = np.empty((self.N, self.k), dtype=np.int32)
        cnt = np.empty(self.N, dtype=np.int32)
        self._check(self.lib.sgs_plan_neighbors(self.h, _ip(idx), _ip(cnt)))
        return idx, cnt

    def weights(self):
        w = np.empty((self.N, self.k), dtype=np.float64)
        s = np.empty(self.N, dtype=np.float64)
        st = np.empty(self.N, dtype=np.int32)
        self._check(self.lib.sgs_plan_weights(self.h, _dp(w), _dp(s), _ip(st)))
        return w, s, st

    def set_indicator(self, prob, data_cat=None):
        """Sequential indicator simulation: prior probabilities of the
        categories and the data's category indices (0-based); call before
        prepare()."""
        prob = np.ascontiguousarray(np.asarray(prob, dtype=np.float64))
        dc = np.ascontiguousarray(np.asarray(data_cat if data_cat is not None else np.zeros(1), dtype=np.int32))
        self._ind = (prob, dc)
        self._check(self.lib.sgs_plan_set_indicator(self.h, len(prob), _dp(prob), _ip(dc)))
        self.prepared = False
        return self

    def set_indicator_cokriging(self, prob, coef, data_cat=None):
        """Indicator simulation by full simple cokriging: prior probabilities,
        the coregionalization matrices (S x L x L, one per structure of the
        plan's variogram) and the data's category indices; call before
        prepare()."""
        prob = np.ascontiguousarray(np.asarray(prob, dtype=np.float64))
        coef = np.ascontiguousarray(np.asarray(coef, dtype=np.float64))
        dc = np.ascontiguousarray(np.asarray(data_cat if data_cat is not None else np.zeros(1), dtype=np.int32))
        self._ind = (prob, dc, coef)
        self._check(self.lib.sgs_plan_set_indicator_cokriging(self.h, len(prob), _dp(prob), _ip(dc), _dp(coef)))
        self.prepared = False
        return self

    def set_multivariate(self, mean, coef, data_values=None):
        """Multivariate Gaussian simulation: the L variables' means, the
        coregionalization matrices (S x L x L, one per structure of the plan's
        variogram) and the data's values (D x L); call before prepare()."""
        mean = np.ascontiguousarray(np.asarray(mean, dtype=np.float64).reshape(-1))
        coef = np.ascontiguousarray(np.asarray(coef, dtype=np.float64))
        dv = np.ascontiguousarray(np.asarray(data_values if data_values is not None else np.zeros(1),
                                             dtype=np.float64))
        self._mv = (mean, coef, dv)
        self._check(self.lib.sgs_plan_set_multivariate(self.h, mean.size, _dp(mean), _dp(coef), _dp(dv)))
        self.nvars = mean.size
        self.prepared = False
        return self

    def simulate_multivariate(self, nreals: int, z=None, seed: int = 0) -> np.ndarray:
        """nreals x L x N values (realization-major, then variable, then node);
        z in the same layout or None for the seeded normals."""
        out = np.empty((nreals, self.nvars, self.N), dtype=np.float64)
        zp = None
        if z is not None:
            z = np.ascontiguousarray(np.asarray(z, dtype=np.float64).reshape(nreals, self.nvars, self.N))
            zp = _dp(z)
        self._check(self.lib.sgs_plan_simulate_multivariate(self.h, nreals, zp, C.c_uint64(seed), _dp(out)))
        return out

    def simulate_indicator(self, nreals: int, u=None, seed: int = 0) -> np.ndarray:
        """nreals x N realization-major category indices (int32)."""
        out = np.empty((nreals, self.N), dtype=np.int32)
        up = None
        if u is not None:
            u = np.ascontiguousarray(np.asarray(u, dtype=np.float64).reshape(nreals, self.N))
            up = _dp(u)
        self._check(self.lib.sgs_plan_simulate_indicator(self.h, nreals, up, C.c_uint64(seed), _ip(out)))
        return out

    def levels(self):
        lv = np.empty(self.N, dtype=np.int32)
        n = C.c_int32()
        self._check(self.lib.sgs_plan_levels(self.h, _ip(lv), C.byref(n)))
        return lv, int(n.value)

    def set_network(self, params):
        """Warm-start network parameters (SGS_NN_PARAMS floats) or None."""
        if params is None:
            self._check(self.lib.sgs_plan_set_network(self.h, None))
            return self
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float32))
        if p.shape != (_abi.SGS_NN_PARAMS,):
            raise ValueError(f"expected {_abi.SGS_NN_PARAMS} parameters")
        self._check(self.lib.sgs_plan_set_network(self.h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return self

    def set_sweep(self, mode=_abi.SGS_SWEEP_FLOW, chunk=1, blocks_per_sm=0, lanes_g=1, lanes_w=0, level_lo=0,
                  level_hi=0, tight=0, split_nodes=0, **_ignored):
        """How simulate() runs the sweep (SGS_SWEEP_* mode and dataflow
        mapping; see sgs_sweep_config).  Accepts a dict returned by
        tune_sweep() as keyword arguments."""
        c = _abi.SgsSweepConfig(mode, chunk, blocks_per_sm, lanes_g, lanes_w, level_lo, level_hi, tight, split_nodes,
                                0.0)
        self._check(self.lib.sgs_plan_set_sweep(self.h, C.byref(c)))
        self._sweep = c.as_dict()
        return self

    def sweep_config(self) -> dict:
        """The sweep configuration set last (set_sweep / tune_sweep)."""
        return dict(self._sweep)

    def tune_sweep(self, nreals: int):
        """Times the candidate sweep configurations for nreals realizations,
        keeps the fastest; returns (chosen, [all timed]) as dicts."""
        chosen = _abi.SgsSweepConfig()
        tried = (_abi.SgsSweepConfig * 64)()
        n = C.c_int32()
        self._check(self.lib.sgs_plan_tune_sweep(self.h, nreals, C.byref(chosen), tried, 64, C.byref(n)))
        self._sweep = chosen.as_dict()
        return chosen.as_dict(), [tried[i].as_dict() for i in range(min(n.value, 64))]

    def predict_device(self, out_ptr: int, tensor_cores: bool = True, stream: int | None = None):
        """Warm-start predictions [N][k] (float32) into a device buffer."""
        self._check(self.lib.sgs_plan_predict_device(self.h, C.c_void_p(out_ptr), 1 if tensor_cores else 0,
                                                     C.c_void_p(stream) if stream else None))

    def info(self) -> _abi.SgsInfo:
        inf = _abi.SgsInfo()
        self._check(self.lib.sgs_plan_info(self.h, C.byref(inf)))
        return inf


class Batch:
    """Owns one sgs_batch: many independent problems (domains) prepared and
    simulated together, one launch per phase over all domains, CUDA graphs
    for the prepare sequence and the seeded sweep.

    `problems` is a list of (sgs_problem, keepalive) pairs as returned by
    build_problem."""

    def __init__(self, problems):
        self.lib = _abi.load_library()
        n = len(problems)
        arr = (_abi.SgsProblem * n)()
        for i, (p, _) in enumerate(problems):
            arr[i] = p
        self._keep = ([k for _, k in problems], arr)
        h = C.c_void_p()
        _abi.check_batch(self.lib, self.lib.sgs_batch_create(arr, n, C.byref(h)))
        self.h = h
        self.ndomains = n
        self.first = np.empty(n, dtype=np.int64)
        self.sizes = np.empty(n, dtype=np.int64)
        self.k = np.empty(n, dtype=np.int64)
        for d in range(n):
            f, c = C.c_int64(), C.c_int64()
            self._check(self.lib.sgs_batch_domain(self.h, d, C.byref(f), C.byref(c)))
            self.first[d], self.sizes[d] = f.value, c.value
            p = problems[d][0]
            nmax = int(p.maxneighbors)
            self.k[d] = nmax if 1 <= nmax <= c.value else c.value
        self.nnodes = int(self.sizes.sum())
        self.prepared = False

    def close(self):
        if getattr(self, "h", None):
            self.lib.sgs_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        return _abi.check_batch(self.lib, rc, self.h)

    def prepare(self):
        self._check(self.lib.sgs_batch_prepare(self.h))
        self.prepared = True
        return self

    def simulate(self, nreals: int, z=None, seed: int = 0):
        """List of nreals x N_d realization-major FP64 arrays, one per domain.
        z: None (seeded draws), or a list of nreals x N_d arrays, or one flat
        array in the concatenated layout."""
        out = np.empty(nreals * self.nnodes, dtype=np.float64)
        zp = None
        if z is not None:
            if isinstance(z, (list, tuple)):
                z = np.concatenate([np.asarray(a, dtype=np.float64).reshape(-1) for a in z])
            z = np.ascontiguousarray(np.asarray(z, dtype=np.float64).reshape(-1))
            if z.size != nreals * self.nnodes:
                raise ValueError("z does not match nreals x nodes")
            zp = _dp(z)
        self._check(self.lib.sgs_batch_simulate(self.h, nreals, zp, C.c_uint64(seed), _dp(out)))
        return [out[nreals * f: nreals * (f + n)].reshape(nreals, n) for f, n in zip(self.first, self.sizes)]

    def values_fp64(self) -> bool:
        """Whether the sweep keeps FP64 values (sgs_batch_info.values_fp64)."""
        return bool(self.info().values_fp64)

    def domain_values_fp64(self, d: int) -> bool:
        """Whether domain d keeps FP64 values (sgs_batch_domain_values_fp64):
        the precision is chosen per domain from its weights."""
        v = C.c_int32()
        self._check(self.lib.sgs_batch_domain_values_fp64(self.h, d, C.byref(v)))
        return bool(v.value)

    def simulate_device(self, nreals: int, seed: int, vals, stream: int | None = None):
        """Seeded sweep into device memory: a device pointer or a CUDA tensor
        of nnodes x (nreals rounded up to 4) values of the sweep's type
        (values_fp64()); tensors are checked.  With FP64 rows, the domains
        that keep FP32 values (domain_values_fp64) hold their row's floats
        in its first half."""
        ptr = _device_values(vals, self.nnodes, nreals, self.values_fp64())
        self._check(self.lib.sgs_batch_simulate_device(self.h, nreals, C.c_uint64(seed), C.c_void_p(ptr),
                                                       C.c_void_p(stream) if stream else None))

    def neighbors(self, d: int):
        n, k = int(self.sizes[d]), int(self.k[d])
        idx = np.empty((n, k), dtype=np.int32)
        cnt = np.empty(n, dtype=np.int32)
        self._check(self.lib.sgs_batch_neighbors(self.h, d, _ip(idx), _ip(cnt)))
        return idx, cnt

    def weights(self, d: int):
        n, k = int(self.sizes[d]), int(self.k[d])
        w = np.empty((n, k), dtype=np.float64)
        s = np.empty(n, dtype=np.float64)
        st = np.empty(n, dtype=np.int32)
        self._check(self.lib.sgs_batch_weights(self.h, d, _dp(w), _dp(s), _ip(st)))
        return w, s, st

    def set_sweep(self, chunk=1, blocks_per_sm=0, lanes_g=1, lanes_w=0, tight=0, **_ignored):
        c = _abi.SgsSweepConfig(_abi.SGS_SWEEP_FLOW, chunk, blocks_per_sm, lanes_g, lanes_w, 0, 0, tight, 0, 0.0)
        self._check(self.lib.sgs_batch_set_sweep(self.h, C.byref(c)))
        return self

    def tune_sweep(self, nreals: int):
        chosen = _abi.SgsSweepConfig()
        tried = (_abi.SgsSweepConfig * 64)()
        n = C.c_int32()
        self._check(self.lib.sgs_batch_tune_sweep(self.h, nreals, C.byref(chosen), tried, 64, C.byref(n)))
        return chosen.as_dict(), [tried[i].as_dict() for i in range(min(n.value, 64))]

    def info(self) -> _abi.SgsBatchInfo:
        inf = _abi.SgsBatchInfo()
        self._check(self.lib.sgs_batch_info_get(self.h, C.byref(inf)))
        return inf

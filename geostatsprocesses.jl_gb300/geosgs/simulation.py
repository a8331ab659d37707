"""The reference's field-simulation API with the GPU SEQSIM method plugged in.

rand(...)                 src/simulation/field.jl:47-124
FieldSimulationMethod     src/simulation/field.jl:135
defaultsimulation         src/simulation/field.jl:152-180
preprocess / randsingle   src/simulation/field/seqsim.jl:50-156 (SEQSIM's pair)
Ensemble                  src/ensembles.jl:10-52 (container + per-node mean/var)

GPUSEQSIM carries SEQSIM's options (seqsim.jl:42-48: path, minneighbors,
maxneighbors, neighborhood, distance) plus the GPU options (precision,
refine_steps, warm_start, device).  By default the path is drawn once per
`rand` call and shared by all realizations of that call: with it fixed,
neighbour sets and kriging weights are the same for every realization, so
`preprocess` computes them once on the GPU and the first `randsingle`
simulates the whole block of realizations in one batched sweep; later calls
hand out the remaining columns.  With `path_per_realization=True` and a
RandomPath, each realization follows its own permutation, drawn one after
another from the path's generator as the reference's
`traverse(domain, path)` does on every realization (seqsim.jl:98): the
realizations then run as a batch of independent problems (sgs_batch_*), one
per realization, with their own neighbour tables and kriging systems.  An
IndicatorProcess or a multivariate GaussianProcess runs them as one plan per
realization, in turn.  A multivariate GaussianProcess (a linear model of
coregionalization, L means) is simulated by simple cokriging of its variables
(sgs_plan_set_multivariate); each realization is {variable: values}.

mean / expectedvalue / posterior   src/expectation/field.jl:17-42 and
                                   src/expectation/field/gaussian.jl:5-25
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import _abi
from .model import (ArgumentError, CartesianGrid, ExplicitPath, GaussianProcess, GeoTable, IndicatorProcess,
                    LinearCoregionalization,
                    LinearPath, RandomPath, SourcePath, nearest_nodes)
from .plan import Batch, Plan
from .problem import build_problem, indicator_levels, multivariate_data


class FieldSimulationMethod:
    """A method for simulating field processes (src/simulation/field.jl:135)."""


@dataclass
class GPUSEQSIM(FieldSimulationMethod):
    """Sequential Gaussian simulation on one GB300 (drop-in for SEQSIM)."""

    path: Any = field(default_factory=LinearPath)
    minneighbors: int = 1
    maxneighbors: int = 26
    neighborhood: Any = "range"
    distance: str = "euclidean"
    precision: str = "fp32"
    refine_steps: int = 2
    warm_start: bool = False
    device: int = 0
    one_launch_sweep: bool = False  # all dependency levels in one cooperative launch
    level_sweep: bool = False       # one launch per dependency level (default: dataflow)
    path_per_realization: bool = False  # RandomPath: a new permutation per realization


class Ensemble:
    """Realizations of a field process over a domain (src/ensembles.jl:10-16):
    `Ensemble(domain, reals, fetch=identity)`.  Iteration and indexing (an
    int, or a list of ints) give `fetch(real)` as {var: values}.  The
    statistics reduce every variable node by node over the realizations, as
    the reference's ereduce does (ensembles.jl:42-52, 76-85), on the device
    (sgs_ensemble_*: the realizations of one variable are uploaded as N rows
    of nreals FP64 values), and return {var: values}; with `var` given, that
    variable's values alone.  Variables must be numeric (integer category
    labels reduce as numbers; string labels raise ArgumentError)."""

    def __init__(self, domain, reals, fetch=None):
        self.domain = domain
        self.reals = list(reals)
        self.fetch = fetch if fetch is not None else (lambda real: real)

    def __len__(self):
        return len(self.reals)

    def __iter__(self):
        return (self.fetch(r) for r in self.reals)

    def __getitem__(self, i):
        if isinstance(i, (list, tuple, np.ndarray)):
            return [self.fetch(self.reals[j]) for j in i]
        return self.fetch(self.reals[i])

    def variables(self) -> list:
        """The realizations' variable names (evars, ensembles.jl:72-74)."""
        return list(self.fetch(self.reals[0]))

    def _rows(self, var):
        """The realizations of `var` as a CUDA tensor of N rows of nreals FP64
        values (the node-major layout of sgs_ensemble_*)."""
        import torch

        cols = [np.asarray(self.fetch(r)[var]) for r in self.reals]
        if any(c.dtype.kind not in "biuf" for c in cols):
            raise ArgumentError(f"variable {var} is not numeric")
        rows = np.ascontiguousarray(np.stack(cols, axis=1), dtype=np.float64)
        if not torch.cuda.is_available():
            raise _abi.GeoSGSError(_abi.SGS_ERR_NODEVICE, "ensemble statistics run on the GPU: no CUDA device")
        return torch.from_numpy(rows).cuda()

    def _reduce(self, f, var):
        names = [var] if var is not None else self.variables()
        out = {}
        for name in names:
            out[name] = f(self._rows(name)).cpu().numpy()
        return out[var] if var is not None else out

    def mean(self, var=None):
        """Per-node mean over the realizations (ensembles.jl:42)."""
        from . import ensemble

        return self._reduce(lambda V: ensemble.mean_var(V, len(self))[0], var)

    def var(self, var=None):
        """Per-node variance, n - 1 divisor (ensembles.jl:44)."""
        from . import ensemble

        return self._reduce(lambda V: ensemble.mean_var(V, len(self))[1], var)

    def cdf(self, x: float, var=None):
        """Per-node fraction of realizations <= x (ensembles.jl:46)."""
        from . import ensemble

        return self._reduce(lambda V: ensemble.cdf(V, len(self), [x])[:, 0], var)

    def ccdf(self, x: float, var=None):
        """Per-node fraction of realizations > x (ensembles.jl:48)."""
        from . import ensemble

        return self._reduce(lambda V: ensemble.cdf(V, len(self), [x], complement=True)[:, 0], var)

    def quantile(self, p, var=None):
        """Per-node quantile(s) with linear interpolation between order
        statistics (ensembles.jl:50-52): one p, or a list of p giving a list
        of results; at most 1024 realizations."""
        from . import ensemble

        if np.ndim(p) > 0:
            return [self.quantile(float(q), var) for q in p]
        if len(self) > 1024:
            raise ArgumentError("quantiles on the device take at most 1024 realizations")
        return self._reduce(lambda V: ensemble.quantile(V, len(self), [float(p)])[:, 0], var)


@dataclass
class _Preproc:
    plan: Any
    var: str
    seed: int
    z: Any = None
    block: Any = None
    cursor: int = 0
    nreals: int = 1
    batches: Any = None  # per-realization paths: [(Batch, first realization, count)]
    levels: Any = None   # indicator simulation: category labels
    paths: Any = None    # per-realization plans: (process, domain, data, method, perms)
    vars: Any = None     # multivariate Gaussian simulation: variable names

    def close(self):
        if self.plan is not None:
            self.plan.close()
        for b, _, _ in self.batches or []:
            b.close()


def _varname(process, data):
    if data is not None and len(data.values) == 1:
        return next(iter(data.values))
    return "field"


def _varnames(process, data):
    """Names of a multivariate process's variables: the data's columns, or
    field1 .. fieldL (defaultschema, src/processes/field/gaussian.jl:43-48)."""
    if data is not None and len(data.values) == process.nvariables:
        return list(data.values)
    return [f"field{i + 1}" for i in range(process.nvariables)]


def _multivariate(process) -> bool:
    return isinstance(process, GaussianProcess) and process.nvariables > 1


def preprocess(rng, process: GaussianProcess, method: GPUSEQSIM, init, domain: CartesianGrid,
               data: GeoTable | None, *, nreals: int = 1, z=None) -> _Preproc:
    """Realization-independent work: problem upload, neighbour search, level
    schedule and kriging solves (seqsim.jl:50-70 plus the hoisted search!/fit
    of seqsim.jl:107-131).  `init` is ignored like SEQSIM ignores it
    (seqsim.jl:267-271 always uses ExplicitInit with data appended)."""
    seed = int(rng.integers(0, 2**63 - 1)) if rng is not None else 0
    if isinstance(process, IndicatorProcess) or _multivariate(process):
        if method.path_per_realization and isinstance(method.path, RandomPath):
            pre = _Preproc(plan=None, var=_varname(process, data), seed=seed, z=z, nreals=nreals)
            pre.paths = (process, domain, data, method, method.path.permutations(domain.nelements(), nreals))
        else:
            pre = _Preproc(plan=_plan_for(process, domain, data, method), var=_varname(process, data),
                           seed=seed, z=z, nreals=nreals)
        if isinstance(process, IndicatorProcess):
            pre.levels = indicator_levels(process, data)[0]
        else:
            pre.vars = _varnames(process, data)
        return pre
    if method.path_per_realization and isinstance(method.path, RandomPath):
        return _Preproc(plan=None, var=_varname(process, data), seed=seed, z=z, nreals=nreals,
                        batches=_per_realization_batches(process, domain, data, method, nreals))
    problem, keep = build_problem(process, domain, data, method)
    plan = Plan(problem, keep).prepare()
    return _Preproc(plan=plan, var=_varname(process, data), seed=seed, z=z, nreals=nreals)


def _plan_for(process, domain, data, method):
    """A prepared plan of an IndicatorProcess (the separable path, or full
    simple cokriging for a linear model of coregionalization) or of a
    multivariate GaussianProcess (simple cokriging of its variables)."""
    problem, keep = build_problem(process, domain, data, method)
    plan = Plan(problem, keep)
    try:
        if isinstance(process, GaussianProcess):
            plan.set_multivariate(process.mean, process.func.coef, multivariate_data(process, data))
        elif isinstance(process.func, LinearCoregionalization):
            plan.set_indicator_cokriging(process.prob, process.func.coef, indicator_levels(process, data)[1])
        else:
            plan.set_indicator(process.prob, indicator_levels(process, data)[1])
        plan.prepare()
    except BaseException:
        plan.close()
        raise
    return plan


def _simulate_plan(plan, process, nreals, z, seed):
    if isinstance(process, IndicatorProcess):
        return plan.simulate_indicator(nreals, u=z, seed=seed)
    return plan.simulate_multivariate(nreals, z=z, seed=seed)


def _per_realization_plans(pre):
    """Realizations that each follow their own permutation: one plan per
    realization, created, prepared, simulated and destroyed in turn (one
    plan's tables on the device at a time).  Realization r draws with
    seed + r, or takes row r of the given uniforms or normals."""
    process, domain, data, method, perms = pre.paths
    z = None if pre.z is None else np.asarray(pre.z, dtype=np.float64).reshape(pre.nreals, -1)
    rows = []
    for r in range(pre.nreals):
        m = GPUSEQSIM(**{**method.__dict__, "path": ExplicitPath(perms[r]), "path_per_realization": False})
        plan = _plan_for(process, domain, data, m)
        try:
            rows.append(_simulate_plan(plan, process, 1, None if z is None else z[r:r + 1], pre.seed + r)[0])
        finally:
            plan.close()
    return np.stack(rows)


# node budget of one batch of per-realization problems (about 500 bytes of
# device tables per node)
BATCH_NODES = 1 << 27


def _per_realization_batches(process, domain, data, method, nreals):
    """One problem per realization, each with its own permutation of the
    RandomPath's generator, grouped into batches of at most BATCH_NODES."""
    n = domain.nelements()
    perms = method.path.permutations(n, nreals)
    per = max(1, BATCH_NODES // max(1, n))
    out = []
    for r0 in range(0, nreals, per):
        probs = []
        for r in range(r0, min(nreals, r0 + per)):
            m = GPUSEQSIM(**{**method.__dict__, "path": ExplicitPath(perms[r]), "path_per_realization": False})
            probs.append(build_problem(process, domain, data, m))
        out.append((Batch(probs).prepare(), r0, len(probs)))
    return out


def randsingle(rng, process, method: GPUSEQSIM, domain, data, preproc: _Preproc) -> dict:
    """One realization as {var: values} (seqsim.jl:72-156).  The first call
    simulates the whole block of `preproc.nreals` realizations on the GPU."""
    if preproc.block is None:
        if preproc.levels is not None or preproc.vars is not None:
            block = (_per_realization_plans(preproc) if preproc.paths is not None
                     else _simulate_plan(preproc.plan, process, preproc.nreals, preproc.z, preproc.seed))
            if preproc.levels is not None:  # category indices -> the categories' labels
                block = np.asarray(preproc.levels, dtype=object if isinstance(preproc.levels[0], str)
                                   else None)[block]
            preproc.block = block
        elif preproc.batches is not None:
            rows = []
            for b, r0, cnt in preproc.batches:
                z = None
                if preproc.z is not None:
                    zz = np.asarray(preproc.z, dtype=np.float64).reshape(preproc.nreals, -1)
                    z = [zz[r0 + i: r0 + i + 1] for i in range(cnt)]
                rows += [v[0] for v in b.simulate(1, z=z, seed=preproc.seed + r0)]
            preproc.block = np.stack(rows)
        else:
            preproc.block = preproc.plan.simulate(preproc.nreals, z=preproc.z, seed=preproc.seed)
        preproc.cursor = 0
    if preproc.cursor >= preproc.block.shape[0]:
        raise ArgumentError("more realizations requested than the prepared block holds")
    col = preproc.block[preproc.cursor]
    preproc.cursor += 1
    if preproc.vars is not None:
        return {name: col[a] for a, name in enumerate(preproc.vars)}
    return {preproc.var: col}


def defaultsimulation(process, domain, *, data=None) -> GPUSEQSIM:
    """The method `rand` uses when none is given (src/simulation/field.jl:
    152-180).  The reference picks FFTSIM or LUSIM for some Gaussian cases;
    this package provides the SEQSIM method only, so a GaussianProcess gets
    GPUSEQSIM with SEQSIM's defaults.  An IndicatorProcess gets the
    reference's path: linear without data; with data, a SourcePath that starts
    at the grid nodes nearest to the data, each node once, in data order."""
    if isinstance(process, IndicatorProcess) and data is not None:
        nodes = nearest_nodes(domain, data.coords)
        _, first = np.unique(nodes, return_index=True)
        return GPUSEQSIM(path=SourcePath(nodes[np.sort(first)]))
    return GPUSEQSIM()


def _rng_of(x):
    if x is None:
        return np.random.default_rng()
    if isinstance(x, np.random.Generator):
        return x
    return np.random.default_rng(int(x))


def rand(*args, data=None, method=None, init=None, workers=None, async_=False,
         showprogress=False, z=None):
    """rand([rng], process, domain, [nreals]; data, method, init, workers, async)
    (src/simulation/field.jl:47-124).

    Returns a {var: values} dict for a single realization, or an Ensemble.
    `z` (nreals x N standard normals, realization-major) replaces the
    generator's draws, for reproducible comparisons."""
    args = list(args)
    rng = None
    if args and not isinstance(args[0], (GaussianProcess, IndicatorProcess)):
        rng = _rng_of(args.pop(0))
    if len(args) not in (2, 3):
        raise ArgumentError("rand([rng], process, domain, [nreals]; kwargs...)")
    process, domain = args[0], args[1]
    if not isinstance(process, (GaussianProcess, IndicatorProcess)):
        raise ArgumentError("rand(process, ...) takes a GaussianProcess or an IndicatorProcess")
    nreals = args[2] if len(args) == 3 else None
    rng = rng if rng is not None else _rng_of(None)
    smethod = method if method is not None else defaultsimulation(process, domain, data=data)
    if not isinstance(smethod, GPUSEQSIM):
        raise ArgumentError("this package provides the GPUSEQSIM method only")
    if workers not in (None, [0], (0,)):
        # the plan lives on this process's GPU and is not serializable
        raise ArgumentError("GPUSEQSIM runs in the calling process; workers must be the master only")
    if async_:
        raise ArgumentError("the `async` option is not allowed when the master process is in the `workers`")
    n = 1 if nreals is None else int(nreals)
    if n < 1:
        raise ArgumentError("nreals must be >= 1")
    pre = preprocess(rng, process, smethod, init, domain, data, nreals=n, z=z)
    try:
        reals = [randsingle(rng, process, smethod, domain, data, pre) for _ in range(n)]
    finally:
        pre.close()
    if nreals is None:
        return reals[0]
    return Ensemble(domain, reals)


# ----------------------------------------------------------------- expectation
@dataclass
class _KrigingOptions:
    """Neighbourhood of the posterior-mean prediction (GeoStatsModels
    fitpredict's options: k nearest data, optionally inside a ball)."""

    maxneighbors: int = 10
    minneighbors: int = 1
    neighborhood: Any = None
    distance: str = "euclidean"
    precision: str = "fp64"
    refine_steps: int = 2
    device: int = 0
    path: Any = field(default_factory=LinearPath)


def posterior(process: GaussianProcess, domain: CartesianGrid, data: GeoTable, *, maxneighbors: int = 10,
              minneighbors: int = 1, neighborhood=None, precision: str = "fp64", device: int = 0):
    """(mean, variance) of the process at every node conditioned on the data:
    simple kriging (src/expectation/field/gaussian.jl:21-25), computed on the
    GPU by sgs_krige; NaN where fewer than minneighbors data are found or the
    system is singular.  Univariate processes only: a multivariate process's
    posterior needs cokriging from the data, which sgs_krige does not do."""
    if _multivariate(process):
        raise ArgumentError("the posterior mean on the GPU path is for univariate processes")
    opts = _KrigingOptions(maxneighbors=maxneighbors, minneighbors=minneighbors, neighborhood=neighborhood,
                           precision=precision, device=device)
    problem, keep = build_problem(process, domain, data, opts)
    lib = _abi.load_library()
    n = domain.nelements()
    m = np.empty(n, dtype=np.float64)
    v = np.empty(n, dtype=np.float64)
    import ctypes as C

    _abi.check(lib, lib.sgs_krige(C.byref(problem), m.ctypes.data_as(C.POINTER(C.c_double)),
                                  v.ctypes.data_as(C.POINTER(C.c_double))))
    del keep
    return m, v


def mean(process: GaussianProcess, domain: CartesianGrid, *, data: GeoTable | None = None, init=None, **kwargs):
    """mean(process, domain; data, init, kwargs...) (src/expectation/field.jl:
    26-42): the prior mean without data (priormean), simple kriging from the
    data otherwise (posteriormean); {var: values}."""
    if data is None:
        if _multivariate(process):
            return {name: np.full(domain.nelements(), mu) for name, mu in zip(_varnames(process, None), process.mean)}
        return {"field": np.full(domain.nelements(), float(process.mean))}
    m, _ = posterior(process, domain, data, **kwargs)
    return {_varname(process, data): m}


def expectedvalue(process: GaussianProcess, domain: CartesianGrid, **kwargs):
    """expectedvalue(process, domain; kwargs...) (src/expectation/field.jl:
    5-23): the mean of a continuous analytical process."""
    return mean(process, domain, **kwargs)

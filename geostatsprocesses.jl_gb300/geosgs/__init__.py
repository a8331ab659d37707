"""geosgs — GB300-native sequential Gaussian simulation behind the
GeoStatsProcesses.jl SEQSIM method API.

Import with the package folder on sys.path:

    sys.path.insert(0, "<repo>/geostatsprocesses.jl_gb300")
    import geosgs
"""
from ._abi import GeoSGSError, load_library, trim_memory
from .model import (
    ArgumentError,
    CartesianGrid,
    ExplicitPath,
    ExponentialVariogram,
    GaussianProcess,
    GaussianVariogram,
    GeoTable,
    ExponentialTransiogram,
    GaussianTransiogram,
    IndicatorProcess,
    LinearCoregionalization,
    LinearPath,
    MetricBall,
    NestedVariogram,
    RandomPath,
    ShiftedPath,
    SourcePath,
    RotX,
    RotY,
    RotZ,
    SphericalTransiogram,
    SphericalVariogram,
    georef,
    nearest_nodes,
    traverse,
)
from .plan import Batch, Plan
from .problem import build_problem, clamped_neighbors
from .simulation import (GPUSEQSIM, Ensemble, FieldSimulationMethod, defaultsimulation, expectedvalue, mean, posterior,
                         preprocess, rand, randsingle)

__all__ = [
    "ArgumentError", "Batch", "CartesianGrid", "Ensemble", "ExplicitPath", "ExponentialVariogram",
    "FieldSimulationMethod", "GPUSEQSIM", "GaussianProcess", "GaussianVariogram", "GeoSGSError",
    "GeoTable", "ExponentialTransiogram", "GaussianTransiogram", "IndicatorProcess", "SphericalTransiogram",
    "LinearCoregionalization", "LinearPath", "MetricBall", "NestedVariogram", "Plan", "RandomPath", "RotX", "RotY", "RotZ",
    "ShiftedPath", "SourcePath", "SphericalVariogram", "build_problem", "clamped_neighbors", "defaultsimulation",
    "georef", "load_library", "nearest_nodes", "traverse", "trim_memory",
    "expectedvalue", "mean", "posterior", "preprocess", "rand", "randsingle",
]

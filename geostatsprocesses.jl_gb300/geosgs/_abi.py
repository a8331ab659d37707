"""ctypes mirror of include/geosgs.h and the loader of libgeosgs.so.

The structs below are field-for-field copies of the C declarations; the
library is loaded from this package's ``lib/`` folder, where ``build()``
places it.  Loading fails loudly: there is no CPU fallback for the product
path.
"""
from __future__ import annotations

import ctypes as C
import os

SGS_OK = 0
SGS_ERR_ARG = -1
SGS_ERR_CUDA = -2
SGS_ERR_OOM = -3
SGS_ERR_TIMEOUT = -4
SGS_ERR_NUMERIC = -5
SGS_ERR_STATE = -6
SGS_ERR_NODEVICE = -7

SGS_SPHERICAL = 1
SGS_EXPONENTIAL = 2
SGS_GAUSSIAN = 3

SGS_SEARCH_RANGE = 0
SGS_SEARCH_BALL = 1
SGS_SEARCH_NEAREST = 2

SGS_PREC_FP64 = 0
SGS_PREC_FP32_REFINE = 1

SGS_FLAG_ONE_LAUNCH_SWEEP = 1
SGS_FLAG_LEVEL_SWEEP = 2
SGS_FLAG_NN_FP32 = 4
SGS_FLAG_OUTPUT_STAGED = 8

SGS_NN_FEATURES = 8
SGS_NN_PARAMS = 2401
SGS_IND_MAX_CATEGORIES = 8
SGS_MV_MAX_VARIABLES = 8

SGS_NODE_KRIGED = 0
SGS_NODE_PRIOR_NMIN = 1
SGS_NODE_PRIOR_SINGULAR = 2


class SgsVariogram(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("reserved", C.c_int32),
        ("sill", C.c_double),
        ("nugget", C.c_double),
        ("ranges", C.c_double * 3),
        ("rotation", C.c_double * 9),
    ]


class SgsBall(C.Structure):
    _fields_ = [("radii", C.c_double * 3), ("rotation", C.c_double * 9)]


SGS_MAX_STRUCTURES = 4


class SgsProblem(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("dims", C.c_int32 * 3),
        ("origin", C.c_double * 3),
        ("spacing", C.c_double * 3),
        ("ndata", C.c_int64),
        ("data_coords", C.POINTER(C.c_double)),
        ("data_values", C.POINTER(C.c_double)),
        ("variogram", SgsVariogram),
        ("mean", C.c_double),
        ("minneighbors", C.c_int32),
        ("maxneighbors", C.c_int32),
        ("search", C.c_int32),
        ("precision", C.c_int32),
        ("ball", SgsBall),
        ("path", C.POINTER(C.c_int32)),
        ("refine_steps", C.c_int32),
        ("warm_start", C.c_int32),
        ("device", C.c_int32),
        ("flags", C.c_int32),
        ("nstructures", C.c_int32),
        ("reserved2", C.c_int32),
        ("structures", C.POINTER(SgsVariogram)),
    ]


SGS_SWEEP_FLOW = 0
SGS_SWEEP_COOPERATIVE = 1
SGS_SWEEP_LEVELS = 2


class SgsSweepConfig(C.Structure):
    _fields_ = [
        ("mode", C.c_int32),
        ("chunk", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("lanes_g", C.c_int32),
        ("lanes_w", C.c_int32),
        ("level_lo", C.c_int32),
        ("level_hi", C.c_int32),
        ("tight", C.c_int32),
        ("split_nodes", C.c_int32),
        ("ms", C.c_float),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class SgsInfo(C.Structure):
    _fields_ = [
        ("nnodes", C.c_int64),
        ("ndata", C.c_int64),
        ("maxneighbors", C.c_int32),
        ("minneighbors", C.c_int32),
        ("nlevels", C.c_int32),
        ("template_size", C.c_int32),
        ("n_prior", C.c_int64),
        ("n_fp64_fallback", C.c_int64),
        ("n_warm_accepted", C.c_int64),
        ("ms_search", C.c_double),
        ("ms_levels", C.c_double),
        ("ms_solve", C.c_double),
        ("ms_sweep", C.c_double),
        ("launches", C.c_int64),
        ("h2d_bytes", C.c_int64),
        ("d2h_bytes", C.c_int64),
        ("sum_grid_neighbors", C.c_int64),
        ("weight_l1_max", C.c_double),
        ("values_fp64", C.c_int32),
        ("reserved", C.c_int32),
        ("search_grid_candidates", C.c_int64),
        ("search_data_candidates", C.c_int64),
    ]


class SgsBatchInfo(C.Structure):
    _fields_ = [
        ("ndomains", C.c_int32),
        ("nlevels", C.c_int32),
        ("nnodes", C.c_int64),
        ("ndata", C.c_int64),
        ("n_prior", C.c_int64),
        ("n_fp64_fallback", C.c_int64),
        ("sum_grid_neighbors", C.c_int64),
        ("bin_systems", C.c_int64 * 5),
        ("ms_search", C.c_double),
        ("ms_levels", C.c_double),
        ("ms_solve", C.c_double),
        ("ms_prepare", C.c_double),
        ("ms_sweep", C.c_double),
        ("launches", C.c_int64),
        ("graph_launches", C.c_int64),
        ("h2d_bytes", C.c_int64),
        ("d2h_bytes", C.c_int64),
        ("device_bytes", C.c_int64),
        ("weight_l1_max", C.c_double),
        ("values_fp64", C.c_int32),
        ("domains_fp64", C.c_int32),
        ("sum_grid_neighbors_fp64", C.c_int64),
    ]


PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG_DIR, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libgeosgs.so")

# Every entry point declared in include/geosgs.h.
EXPORTS = (
    "sgs_plan_create",
    "sgs_plan_prepare",
    "sgs_plan_simulate",
    "sgs_plan_simulate_device",
    "sgs_plan_neighbors",
    "sgs_plan_weights",
    "sgs_plan_levels",
    "sgs_plan_info",
    "sgs_plan_destroy",
    "sgs_trim_memory",
    "sgs_last_error",
    "sgs_version",
    "sgs_plan_features_device",
    "sgs_plan_set_network",
    "sgs_nn_forward",
    "sgs_nn_backward",
    "sgs_nn_adam",
    "sgs_schedule_noalloc",
    "sgs_plan_set_sweep",
    "sgs_plan_tune_sweep",
    "sgs_plan_predict_device",
    "sgs_batch_create",
    "sgs_batch_prepare",
    "sgs_batch_simulate",
    "sgs_batch_simulate_device",
    "sgs_batch_domain",
    "sgs_batch_domain_values_fp64",
    "sgs_batch_neighbors",
    "sgs_batch_weights",
    "sgs_batch_set_sweep",
    "sgs_batch_tune_sweep",
    "sgs_batch_info_get",
    "sgs_batch_destroy",
    "sgs_batch_last_error",
    "sgs_krige",
    "sgs_plan_set_indicator",
    "sgs_plan_set_indicator_cokriging",
    "sgs_plan_simulate_indicator",
    "sgs_plan_set_multivariate",
    "sgs_plan_simulate_multivariate",
    "sgs_ensemble_stats",
    "sgs_ensemble_cdf",
    "sgs_ensemble_quantile",
)

_lib = None


def trim_memory(device: int = -1) -> None:
    """Return the device memory the library keeps for reuse (freed by
    destroyed plans and batches) to the device; device < 0: every device."""
    rc = load_library().sgs_trim_memory(int(device))
    if rc != 0:
        raise GeoSGSError(rc, "sgs_trim_memory failed")


class GeoSGSError(RuntimeError):
    """A libgeosgs call returned a negative status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"libgeosgs error {code}: {message}")
        self.code = code


def _declare(lib):
    P = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int32)
    lib.sgs_plan_create.argtypes = [C.POINTER(SgsProblem), C.POINTER(P)]
    lib.sgs_plan_create.restype = C.c_int
    lib.sgs_plan_prepare.argtypes = [P]
    lib.sgs_plan_prepare.restype = C.c_int
    lib.sgs_plan_simulate.argtypes = [P, C.c_int32, dp, C.c_uint64, dp]
    lib.sgs_plan_simulate.restype = C.c_int
    lib.sgs_plan_simulate_device.argtypes = [P, C.c_int32, P, C.c_uint64, P, P]
    lib.sgs_plan_simulate_device.restype = C.c_int
    lib.sgs_plan_neighbors.argtypes = [P, ip, ip]
    lib.sgs_plan_neighbors.restype = C.c_int
    lib.sgs_plan_weights.argtypes = [P, dp, dp, ip]
    lib.sgs_plan_weights.restype = C.c_int
    lib.sgs_plan_levels.argtypes = [P, ip, ip]
    lib.sgs_plan_levels.restype = C.c_int
    lib.sgs_plan_info.argtypes = [P, C.POINTER(SgsInfo)]
    lib.sgs_plan_info.restype = C.c_int
    lib.sgs_plan_destroy.argtypes = [P]
    lib.sgs_plan_destroy.restype = None
    lib.sgs_trim_memory.argtypes = [C.c_int32]
    lib.sgs_trim_memory.restype = C.c_int
    lib.sgs_last_error.argtypes = [P]
    lib.sgs_last_error.restype = C.c_char_p
    lib.sgs_version.argtypes = []
    lib.sgs_version.restype = C.c_char_p
    lib.sgs_plan_features_device.argtypes = [P, P, P]
    lib.sgs_plan_features_device.restype = C.c_int
    lib.sgs_plan_set_network.argtypes = [P, C.POINTER(C.c_float)]
    lib.sgs_plan_set_network.restype = C.c_int
    lib.sgs_plan_set_sweep.argtypes = [P, C.POINTER(SgsSweepConfig)]
    lib.sgs_plan_set_sweep.restype = C.c_int
    lib.sgs_plan_tune_sweep.argtypes = [P, C.c_int32, C.POINTER(SgsSweepConfig), C.POINTER(SgsSweepConfig),
                                        C.c_int32, C.POINTER(C.c_int32)]
    lib.sgs_plan_tune_sweep.restype = C.c_int
    lib.sgs_plan_predict_device.argtypes = [P, P, C.c_int32, P]
    lib.sgs_plan_predict_device.restype = C.c_int
    lib.sgs_nn_forward.argtypes = [P, P, P, C.c_int64, C.c_int32, P, P]
    lib.sgs_nn_forward.restype = C.c_int
    lib.sgs_nn_backward.argtypes = [P, P, P, P, C.c_int64, C.c_int32, P, P, P]
    lib.sgs_nn_backward.restype = C.c_int
    lib.sgs_nn_adam.argtypes = [P, P, P, P, C.c_int32, C.c_float, C.c_float, P]
    lib.sgs_nn_adam.restype = C.c_int
    lib.sgs_schedule_noalloc.argtypes = [P, P, P, C.c_int64, C.c_int32, P, P, P, C.c_int32, ip, P]
    lib.sgs_schedule_noalloc.restype = C.c_int
    i64p = C.POINTER(C.c_int64)
    lib.sgs_batch_create.argtypes = [C.POINTER(SgsProblem), C.c_int32, C.POINTER(P)]
    lib.sgs_batch_create.restype = C.c_int
    lib.sgs_batch_prepare.argtypes = [P]
    lib.sgs_batch_prepare.restype = C.c_int
    lib.sgs_batch_simulate.argtypes = [P, C.c_int32, dp, C.c_uint64, dp]
    lib.sgs_batch_simulate.restype = C.c_int
    lib.sgs_batch_simulate_device.argtypes = [P, C.c_int32, C.c_uint64, P, P]
    lib.sgs_batch_simulate_device.restype = C.c_int
    lib.sgs_batch_domain.argtypes = [P, C.c_int32, i64p, i64p]
    lib.sgs_batch_domain_values_fp64.argtypes = [P, C.c_int32, C.POINTER(C.c_int32)]
    lib.sgs_batch_domain_values_fp64.restype = C.c_int
    lib.sgs_batch_domain.restype = C.c_int
    lib.sgs_batch_neighbors.argtypes = [P, C.c_int32, ip, ip]
    lib.sgs_batch_neighbors.restype = C.c_int
    lib.sgs_batch_weights.argtypes = [P, C.c_int32, dp, dp, ip]
    lib.sgs_batch_weights.restype = C.c_int
    lib.sgs_batch_set_sweep.argtypes = [P, C.POINTER(SgsSweepConfig)]
    lib.sgs_batch_set_sweep.restype = C.c_int
    lib.sgs_batch_tune_sweep.argtypes = [P, C.c_int32, C.POINTER(SgsSweepConfig), C.POINTER(SgsSweepConfig),
                                         C.c_int32, C.POINTER(C.c_int32)]
    lib.sgs_batch_tune_sweep.restype = C.c_int
    lib.sgs_batch_info_get.argtypes = [P, C.POINTER(SgsBatchInfo)]
    lib.sgs_batch_info_get.restype = C.c_int
    lib.sgs_batch_destroy.argtypes = [P]
    lib.sgs_batch_destroy.restype = None
    lib.sgs_batch_last_error.argtypes = [P]
    lib.sgs_batch_last_error.restype = C.c_char_p
    lib.sgs_plan_set_indicator.argtypes = [P, C.c_int32, dp, ip]
    lib.sgs_plan_set_indicator.restype = C.c_int
    lib.sgs_plan_set_indicator_cokriging.argtypes = [P, C.c_int32, dp, ip, dp]
    lib.sgs_plan_set_indicator_cokriging.restype = C.c_int
    lib.sgs_plan_simulate_indicator.argtypes = [P, C.c_int32, dp, C.c_uint64, ip]
    lib.sgs_plan_simulate_indicator.restype = C.c_int
    lib.sgs_plan_set_multivariate.argtypes = [P, C.c_int32, dp, dp, dp]
    lib.sgs_plan_set_multivariate.restype = C.c_int
    lib.sgs_plan_simulate_multivariate.argtypes = [P, C.c_int32, dp, C.c_uint64, dp]
    lib.sgs_plan_simulate_multivariate.restype = C.c_int
    lib.sgs_krige.argtypes = [C.POINTER(SgsProblem), dp, dp]
    lib.sgs_krige.restype = C.c_int
    lib.sgs_ensemble_stats.argtypes = [P, C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_double, P, P, P]
    lib.sgs_ensemble_stats.restype = C.c_int
    lib.sgs_ensemble_cdf.argtypes = [P, C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_double, dp, C.c_int32,
                                     C.c_int32, P, P]
    lib.sgs_ensemble_cdf.restype = C.c_int
    lib.sgs_ensemble_quantile.argtypes = [P, C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_double, dp,
                                          C.c_int32, P, P]
    lib.sgs_ensemble_quantile.restype = C.c_int
    return lib


def load_library(path: str | None = None):
    """Load libgeosgs.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"libgeosgs.so not found at {p}: build it first "
            "(python -c 'import __graft_entry__ as g; g.build()')"
        )
    lib = _declare(C.CDLL(p))
    if path is None:
        _lib = lib
    return lib


def check(lib, code: int, plan=None):
    if code != SGS_OK:
        msg = lib.sgs_last_error(plan)
        raise GeoSGSError(code, msg.decode() if msg else "")
    return code


def check_batch(lib, code: int, batch=None):
    if code != SGS_OK:
        msg = lib.sgs_batch_last_error(batch)
        raise GeoSGSError(code, msg.decode() if msg else "")
    return code

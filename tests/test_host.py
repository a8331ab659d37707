"""Host-side logic and the C-ABI library, without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import geosgs
from conftest import ROOT
from geosgs import _abi, workloads


def header_symbols():
    src = open(os.path.join(ROOT, "include", "geosgs.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(sgs_\w+)\s*\(", src, re.M)))


def test_header_declares_the_abi():
    assert header_symbols() == sorted(_abi.EXPORTS)


def test_library_loads_and_exports_every_header_symbol():
    from geosgs import _build

    _build.build()
    lib = C.CDLL(_abi.LIB_PATH)
    for name in header_symbols():
        assert hasattr(lib, name), name
    _abi.load_library()


def test_diagnostic_exports_outside_the_header():
    """The bounded-wait self-tests are exported for the GPU tests but are
    not part of the C ABI the header declares."""
    from geosgs import _build

    _build.build()
    lib = C.CDLL(_abi.LIB_PATH)
    for name in ("sgs_selftest_bounded_wait", "sgs_selftest_levels_wait"):
        assert hasattr(lib, name)
        assert name not in header_symbols()


def test_peak_probe_library_builds_and_exports():
    """The benchmark's throughput probes live in their own library, outside
    the C ABI of include/geosgs.h."""
    import bench

    lib = C.CDLL(bench.build_peaks())
    for name in ("geosgs_peak_fp32", "geosgs_peak_fp64", "geosgs_peak_gj_pattern", "geosgs_peak_host_write",
                 "geosgs_peak_d2h_copy"):
        assert hasattr(lib, name), name
    assert not any(n.startswith("geosgs_peak") for n in header_symbols())


def test_create_without_gpu_fails_cleanly():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from geosgs import _build

    _build.build()
    wl = workloads.small(n=8, k=4)
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    with pytest.raises(geosgs.GeoSGSError) as e:
        geosgs.Plan(p, keep)
    assert e.value.code in (_abi.SGS_ERR_NODEVICE, _abi.SGS_ERR_CUDA)


def test_struct_layout_matches_header():
    # offsets the C compiler gives sgs_problem, checked by compiling a probe
    import subprocess
    import tempfile

    src = r"""
#include <stddef.h>
#include <stdio.h>
#include "geosgs.h"
int main(void){
 printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(sgs_problem), offsetof(sgs_problem, variogram),
   offsetof(sgs_problem, mean), offsetof(sgs_problem, ball), offsetof(sgs_problem, path),
   offsetof(sgs_problem, flags), sizeof(sgs_info), offsetof(sgs_info, ms_sweep),
   sizeof(sgs_sweep_config), offsetof(sgs_sweep_config, ms));
 printf("%zu %zu\n", offsetof(sgs_info, search_data_candidates), offsetof(sgs_batch_info, sum_grid_neighbors_fp64));
 printf("%zu %zu %zu\n", sizeof(sgs_batch_info), offsetof(sgs_batch_info, ms_search),
   offsetof(sgs_batch_info, device_bytes));
 return 0;}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        got = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    P, I, W, B = _abi.SgsProblem, _abi.SgsInfo, _abi.SgsSweepConfig, _abi.SgsBatchInfo
    want = [C.sizeof(P), P.variogram.offset, P.mean.offset, P.ball.offset, P.path.offset, P.flags.offset,
            C.sizeof(I), I.ms_sweep.offset, C.sizeof(W), W.ms.offset, I.search_data_candidates.offset,
            B.sum_grid_neighbors_fp64.offset, C.sizeof(B), B.ms_search.offset, B.device_bytes.offset]
    assert got == want


def test_build_problem_fields():
    wl = workloads.c3(nreals=2)
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    assert p.dim == 3 and list(p.dims) == [200, 200, 100]
    assert p.ndata == 5000 and p.maxneighbors == 48
    assert p.search == _abi.SGS_SEARCH_BALL and p.variogram.type == _abi.SGS_EXPONENTIAL
    R = np.array([[p.ball.rotation[i + 3 * j] for j in range(3)] for i in range(3)])
    np.testing.assert_allclose(R, geosgs.RotZ(30.0))
    assert tuple(p.ball.radii) == (50.0, 25.0, 5.0)


def test_range_neighbourhood_and_grid_forms():
    g = geosgs.CartesianGrid((0.5, 0.5), (100.5, 100.5), dims=(100, 100))
    assert g.origin == (0.5, 0.5) and g.spacing == (1.0, 1.0)
    c = g.centroids()
    assert c.shape == (10000, 2) and tuple(c[0]) == (1.0, 1.0) and tuple(c[1]) == (2.0, 1.0)
    assert g.linear_index(24, 24) == 2424
    v = geosgs.SphericalVariogram(ranges=(10.0, 4.0), sill=2.0)
    assert v.range() == 10.0
    np.testing.assert_allclose(v([0.0, 0.5, 1.0, 2.0]), [0.0, 2 * (0.75 - 0.0625), 2.0, 2.0])


def test_api_argument_errors():
    proc = geosgs.GaussianProcess(geosgs.GaussianVariogram())
    grid = geosgs.CartesianGrid((10, 10))
    with pytest.raises(geosgs.ArgumentError):
        geosgs.rand(proc, grid, 2, async_=True)
    with pytest.raises(geosgs.ArgumentError):
        geosgs.rand(proc, grid, 2, workers=[1, 2])
    with pytest.raises(geosgs.ArgumentError):
        geosgs.GaussianProcess(geosgs.GaussianVariogram(), [0.0, 1.0])
    with pytest.raises(geosgs.ArgumentError):
        geosgs.build_problem(proc, grid, None, geosgs.GPUSEQSIM(precision="fp16"))
    with pytest.raises(geosgs.ArgumentError):
        geosgs.build_problem(proc, grid, None, geosgs.GPUSEQSIM(neighborhood=3.0))


def test_paths():
    assert geosgs.LinearPath().permutation(5) is None
    p = geosgs.RandomPath(4).permutation(1000)
    assert sorted(p) == list(range(1000)) and p.dtype == np.int32
    np.testing.assert_array_equal(p, geosgs.RandomPath(4).permutation(1000))
    with pytest.raises(geosgs.ArgumentError):
        geosgs.ExplicitPath([0, 1]).permutation(3)


def test_reference_arm_line_shares_the_config():
    """bench.py --impl reference times the FP64 oracle on a bounded sample and
    prints the workload's config exactly as the GPU arm builds it (what is
    simulated, not how), marks the value as extrapolated from the sample and
    reports the sample's own wall time per step."""
    import json
    import subprocess
    import sys

    import bench

    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c1",
                        "--steps", "1", "--warmup", "0", "--cpu-nodes", "2000"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    wl = bench.workload("c1", "fp64", None)
    assert line["config"] == bench.config_of(wl, 1)
    assert line["impl"] == "reference" and line["extrapolated"] is True
    assert line["ms_per_step"] == line["sample_wall_ms_per_step"] > 0
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"

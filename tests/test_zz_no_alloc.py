"""sgs_schedule_noalloc: the dependency-level schedule computed without any
allocation by the library, for callers that own all device memory (for
example an application whose memory pool already holds the GPU).  Its
levels must equal those the plan path (sgs_plan_levels) computes, on two
calls in a row that share the library's file-scope working array.

This file is collected last so that a run stopping at the first failure
has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import geosgs
from geosgs import _abi, workloads

pytestmark = pytest.mark.gpu


def _schedule(lib, path_d, nbr_d, cnt_d, N, k, cap, torch):
    level = torch.empty(N, dtype=torch.int32, device="cuda")
    order = torch.empty(N, dtype=torch.int32, device="cuda")
    offsets = torch.empty(cap, dtype=torch.int32, device="cuda")
    nl = C.c_int32(0)
    rc = lib.sgs_schedule_noalloc(path_d.data_ptr(), nbr_d.data_ptr(), cnt_d.data_ptr(), N, k,
                                  level.data_ptr(), order.data_ptr(), offsets.data_ptr(), cap,
                                  C.byref(nl), torch.cuda.current_stream().cuda_stream)
    return rc, level.cpu().numpy(), order.cpu().numpy(), offsets.cpu().numpy(), nl.value


@pytest.mark.parametrize("case", ["c1", "aniso3d"])
def test_noalloc_schedule_matches_plan(case, geosgs_lib):
    torch = pytest.importorskip("torch")
    if case == "c1":
        wl = workloads.c1("fp32")
    else:
        wl = workloads.small(dim=3, n=30, nz=10, k=24, ndata=40, vario="exp", ranges=(9.0, 5.0, 3.0),
                             rotation=geosgs.RotZ(30.0), ball=geosgs.MetricBall((9.0, 5.0, 3.0), geosgs.RotZ(30.0)),
                             precision="fp32")
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    plan = geosgs.Plan(p, keep).prepare()
    ref_level, ref_nl = plan.levels()
    idx, cnt = plan.neighbors()
    N, k = plan.N, plan.k
    path = wl.method.path.permutation(N).astype(np.int32)
    path_d = torch.from_numpy(path).cuda()
    nbr_d = torch.from_numpy(np.ascontiguousarray(idx)).cuda()
    cnt_d = torch.from_numpy(cnt).cuda()
    lib = geosgs_lib
    for call in range(2):  # the second call reuses the working array the first left behind
        rc, level, order, offsets, nl = _schedule(lib, path_d, nbr_d, cnt_d, N, k, ref_nl + 1, torch)
        assert rc == _abi.SGS_OK, lib.sgs_last_error(None)
        assert nl == ref_nl
        np.testing.assert_array_equal(level, ref_level)
        assert offsets[0] == 0 and offsets[nl] == N
        assert np.all(np.diff(offsets[: nl + 1]) > 0)
        assert np.array_equal(np.sort(order), np.arange(N))
        for l in range(nl):
            assert np.all(level[order[offsets[l]:offsets[l + 1]]] == l)
    plan.close()


def test_noalloc_rejects_too_small_offsets(geosgs_lib):
    torch = pytest.importorskip("torch")
    wl = workloads.small(n=20, k=8, precision="fp32")
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    plan = geosgs.Plan(p, keep).prepare()
    _, ref_nl = plan.levels()
    idx, cnt = plan.neighbors()
    path = wl.method.path.permutation(plan.N).astype(np.int32)
    rc, *_ = _schedule(geosgs_lib, torch.from_numpy(path).cuda(), torch.from_numpy(idx).cuda(),
                       torch.from_numpy(cnt).cuda(), plan.N, plan.k, ref_nl, torch)
    assert rc == _abi.SGS_ERR_ARG
    assert b"capacity" in geosgs_lib.sgs_last_error(None)
    plan.close()

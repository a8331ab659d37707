"""sgs_schedule_noalloc: the dependency-level schedule computed without any
allocation by the library, for callers that own all device memory (for
example an application whose memory pool already holds the GPU, so an
allocation inside the library would fail or fragment the pool).  Its levels
must equal those the plan path (sgs_plan_levels) computes, on two calls in a
row that share the library's file-scope working array, and the second call
must leave the device's free memory unchanged.  Invalid tables (a path that
is not a permutation, counts out of range, a neighbour that does not come
earlier in the path) are rejected with SGS_ERR_ARG at once, and a schedule
deeper than SGS_NOALLOC_MAX_LEVELS is rejected too.

This file is collected last so that a run stopping at the first failure
has already run every other test."""
import ctypes as C
import time

import numpy as np
import pytest

import geosgs
from geosgs import _abi, workloads

pytestmark = pytest.mark.gpu

MAX_LEVELS = 262144  # SGS_NOALLOC_MAX_LEVELS in include/geosgs.h


def _outputs(N, cap, torch):
    return (torch.empty(N, dtype=torch.int32, device="cuda"), torch.empty(N, dtype=torch.int32, device="cuda"),
            torch.empty(cap, dtype=torch.int32, device="cuda"))


def _call(lib, path_d, nbr_d, cnt_d, N, k, outs, torch):
    level, order, offsets = outs
    nl = C.c_int32(0)
    rc = lib.sgs_schedule_noalloc(path_d.data_ptr(), nbr_d.data_ptr(), cnt_d.data_ptr(), N, k,
                                  level.data_ptr(), order.data_ptr(), offsets.data_ptr(), offsets.numel(),
                                  C.byref(nl), torch.cuda.current_stream().cuda_stream)
    return rc, nl.value


def _schedule(lib, path_d, nbr_d, cnt_d, N, k, cap, torch):
    outs = _outputs(N, cap, torch)
    rc, nl = _call(lib, path_d, nbr_d, cnt_d, N, k, outs, torch)
    level, order, offsets = outs
    return rc, level.cpu().numpy(), order.cpu().numpy(), offsets.cpu().numpy(), nl


def _device(torch, *arrays):
    return [torch.from_numpy(np.ascontiguousarray(a, dtype=np.int32)).cuda() for a in arrays]


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
    path_d, nbr_d, cnt_d = _device(torch, path, idx, cnt)
    lib = geosgs_lib
    for call in range(2):  # the second call reuses the working array the first left behind
        outs = _outputs(N, ref_nl + 1, torch)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        alloc0 = torch.cuda.memory_allocated()
        rc, nl = _call(lib, path_d, nbr_d, cnt_d, N, k, outs, torch)
        free1, _ = torch.cuda.mem_get_info()
        assert rc == _abi.SGS_OK, lib.sgs_last_error(None)
        if call == 1:
            # the call itself allocates nothing: device free memory (cudaMemGetInfo)
            # and torch's allocator are where they were before it
            assert free1 == free0
            assert torch.cuda.memory_allocated() == alloc0
        level, order, offsets = (t.cpu().numpy() for t in outs)
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
    rc, *_ = _schedule(geosgs_lib, *_device(torch, path, idx, cnt), plan.N, plan.k, ref_nl, torch)
    assert rc == _abi.SGS_ERR_ARG
    assert b"capacity" in geosgs_lib.sgs_last_error(None)
    plan.close()


def _chain(N):
    """A linear path where node g's one neighbour is node g - 1: N levels."""
    path = np.arange(N, dtype=np.int32)
    nbr = (np.arange(N, dtype=np.int32) - 1).reshape(N, 1)
    cnt = np.ones(N, dtype=np.int32)
    cnt[0] = 0
    return path, nbr, cnt


def test_noalloc_level_limit(geosgs_lib):
    """A chain of MAX_LEVELS nodes is the deepest schedule accepted; one more
    node is rejected with SGS_ERR_ARG, and a valid call afterwards works."""
    torch = pytest.importorskip("torch")
    lib = geosgs_lib
    for N, ok in ((MAX_LEVELS, True), (MAX_LEVELS + 1, False)):
        path, nbr, cnt = _chain(N)
        rc, level, _, offsets, nl = _schedule(lib, *_device(torch, path, nbr, cnt), N, 1, N + 1, torch)
        if ok:
            assert rc == _abi.SGS_OK, lib.sgs_last_error(None)
            assert nl == N
            np.testing.assert_array_equal(level, np.arange(N))
            np.testing.assert_array_equal(offsets, np.arange(N + 1))
        else:
            assert rc == _abi.SGS_ERR_ARG
            assert b"levels" in lib.sgs_last_error(None)
    path, nbr, cnt = _chain(100)
    rc, level, *_ = _schedule(lib, *_device(torch, path, nbr, cnt), 100, 1, 101, torch)
    assert rc == _abi.SGS_OK
    np.testing.assert_array_equal(level, np.arange(100))


@pytest.mark.parametrize("fault", ["later_neighbour", "cycle", "repeat", "out_of_range", "count", "negative"])
def test_noalloc_rejects_invalid_tables(fault, geosgs_lib):
    """Inputs are checked on the device before the level kernel reads them:
    each invalid table is rejected with SGS_ERR_ARG promptly (no bounded wait
    runs out), and a valid call on the same working array works after it."""
    torch = pytest.importorskip("torch")
    lib = geosgs_lib
    N, k = 64, 4
    path = np.random.default_rng(5).permutation(N).astype(np.int32)
    rank = np.empty(N, dtype=np.int64)
    rank[path] = np.arange(N)
    nbr = np.full((N, k), -1, dtype=np.int32)
    cnt = np.zeros(N, dtype=np.int32)
    for t in range(1, N):  # each node: up to k earlier nodes of the path
        prev = path[max(0, t - k):t]
        nbr[path[t], :len(prev)] = prev
        cnt[path[t]] = len(prev)
    good = (path.copy(), nbr.copy(), cnt.copy())
    g_last, g_first = path[N - 1], path[0]
    if fault == "later_neighbour":
        nbr[g_first, 0], cnt[g_first] = g_last, 1
        want = b"earlier"
    elif fault == "cycle":  # two nodes each other's neighbour
        nbr[g_first, 0], cnt[g_first] = path[1], 1
        want = b"earlier"
    elif fault == "repeat":
        path[3] = path[4]
        want = b"twice"
    elif fault == "out_of_range":
        path[7] = N
        want = b"outside"
    elif fault == "count":
        cnt[g_last] = k + 1
        want = b"count"
    else:  # a -1 padding entry inside the count
        cnt[g_first] = 1
        want = b"negative"
    t0 = time.perf_counter()
    rc, *_ = _schedule(lib, *_device(torch, path, nbr, cnt), N, k, N + 1, torch)
    assert time.perf_counter() - t0 < 1.0
    assert rc == _abi.SGS_ERR_ARG
    assert want in lib.sgs_last_error(None)
    rc, level, *_ = _schedule(lib, *_device(torch, *good), N, k, N + 1, torch)
    assert rc == _abi.SGS_OK
    expect = np.zeros(N, dtype=np.int64)
    for g in good[0]:  # level = 1 + deepest neighbour level, in path order
        expect[g] = 1 + max((expect[c] for c in good[1][g, :good[2][g]]), default=-1)
    np.testing.assert_array_equal(level, expect)

"""CUDA path (through the C ABI) against the FP64 oracle.

Bars: neighbour indices and counts bit-exact; node status identical; values
within 1e-6 relative, rel = max |v_gpu - v_oracle| / max(|v_oracle|, 1) per
element, for both precisions (FP64 and FP32 + FP64 refinement); weights
within 1e-9 (FP64) and 1e-6 (FP32 refined; stored FP32 in the sweep
tables but exported in FP64)."""
import numpy as np
import pytest

import geosgs
from conftest import golden_cases, golden_problem, load_golden
from geosgs import _abi, workloads

pytestmark = pytest.mark.gpu

VALUE_TOL = 1e-6


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0))) if a.size else 0.0


def gpu_plan(problem, keep):
    return geosgs.Plan(problem, keep).prepare()


def both(wl, oracle_mod, precision, t_end=None, stride=None):
    wl.method.precision = precision
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = gpu_plan(p, keep)
    O = oracle_mod.OraclePlan(p, keep)
    if stride:
        O.search(oracle_mod.TEMPLATE, stride=stride)
        O.solve(stride=stride)
    if t_end:
        O.search(oracle_mod.TEMPLATE, t1=t_end)
        O.solve(t1=t_end)
    if not stride and not t_end:
        O.prepare()
    return G, O


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", golden_cases())
def test_golden_fixtures_on_gpu(name, precision, geosgs_lib):
    g = load_golden(name)
    p, keep = golden_problem(g, precision)
    G = gpu_plan(p, keep)
    idx, cnt = G.neighbors()
    np.testing.assert_array_equal(cnt, g["cnt"])
    np.testing.assert_array_equal(idx, g["nbr"])
    w, s, st = G.weights()
    np.testing.assert_array_equal(st, g["status"])
    np.testing.assert_allclose(w, g["w"], rtol=0, atol=1e-9 if precision == 0 else 1e-6)
    out = G.simulate(g["z"].shape[0], g["z"])
    assert rel_err(out, g["out"]) <= VALUE_TOL


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_c1_full_parity(precision, oracle_mod, geosgs_lib):
    wl = workloads.c1()
    G, O = both(wl, oracle_mod, precision)
    ig, cg = G.neighbors()
    io, co = O.neighbors()
    np.testing.assert_array_equal(cg, co)
    np.testing.assert_array_equal(ig, io)
    wg, sg, stg = G.weights()
    wo, so, sto = O.weights()
    np.testing.assert_array_equal(stg, sto)
    np.testing.assert_allclose(wg, wo, rtol=0, atol=1e-9 if precision == "fp64" else 1e-6)
    z = np.random.default_rng(77).standard_normal((wl.nreals, O.N))
    assert rel_err(G.simulate(wl.nreals, z), O.simulate(wl.nreals, z)) <= VALUE_TOL
    lg, nlg = G.levels()
    lo, nlo = O.levels()
    np.testing.assert_array_equal(lg, lo)
    assert nlg == nlo


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_c2_full_parity(precision, oracle_mod, geosgs_lib):
    """500x500 grid, 1,000 data on cell centres, gaussian variogram with a
    0.01 nugget (duplicate locations -> singular systems), k=32, 64 reals."""
    wl = workloads.c2(nreals=64)
    G, O = both(wl, oracle_mod, precision)
    ig, cg = G.neighbors()
    io, co = O.neighbors()
    np.testing.assert_array_equal(cg, co)
    np.testing.assert_array_equal(ig, io)
    wg, sg, stg = G.weights()
    wo, so, sto = O.weights()
    np.testing.assert_array_equal(stg, sto)
    kriged = sto == 0
    np.testing.assert_allclose(wg[kriged], wo[kriged], rtol=0, atol=1e-10 if precision == "fp64" else 1e-8)
    # at a node on a datum the variance cancels to ~0: compare variances
    np.testing.assert_allclose(sg**2, so**2, rtol=0, atol=1e-10)
    z = np.random.default_rng(5).standard_normal((wl.nreals, O.N))
    err = rel_err(G.simulate(wl.nreals, z), O.simulate(wl.nreals, z))
    print(f"c2 {precision} max rel err {err:.3e}")
    assert err <= VALUE_TOL


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_3d_anisotropic_with_data(precision, oracle_mod, geosgs_lib):
    wl = workloads.small(dim=3, n=40, nz=12, k=24, ndata=150, vario="exp", ranges=(12.0, 6.0, 3.0),
                         rotation=geosgs.RotZ(30.0), nugget=0.05,
                         ball=geosgs.MetricBall((12.0, 6.0, 3.0), geosgs.RotZ(30.0)), nreals=8)
    G, O = both(wl, oracle_mod, precision)
    np.testing.assert_array_equal(G.neighbors()[0], O.neighbors()[0])
    np.testing.assert_array_equal(G.weights()[2], O.weights()[2])
    z = np.random.default_rng(9).standard_normal((wl.nreals, O.N))
    assert rel_err(G.simulate(wl.nreals, z), O.simulate(wl.nreals, z)) <= VALUE_TOL


def test_seeded_draws_match_oracle(oracle_mod, geosgs_lib):
    """On-device Philox draws (float Box-Muller) against the oracle's FP64
    draws of the same counters: equal up to float rounding of the normals."""
    wl = workloads.small(n=30, k=10, ndata=10, nreals=12)
    G, O = both(wl, oracle_mod, "fp64")
    out_g = G.simulate(12, None, seed=99)
    out_o = O.simulate(12, None, seed=99)
    assert rel_err(out_g, out_o) <= 2e-5


def test_c3_sampled_neighbours_and_prefix_values(oracle_mod, geosgs_lib):
    """Full 200x200x100 grid, 5,000 data, rotated ellipsoid, k=48: the oracle
    searches and solves every 997th path rank plus the first 4,000 ranks;
    neighbours of all those nodes are bit-exact and the values of the first
    4,000 path nodes (which depend only on earlier ones) agree within 1e-6."""
    wl = workloads.c3(precision="fp32", nreals=8)
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = gpu_plan(p, keep)
    O = oracle_mod.OraclePlan(p, keep)
    T = 4000
    O.search(oracle_mod.TEMPLATE, stride=997)
    O.search(oracle_mod.TEMPLATE, t1=T)
    O.solve(t1=T)
    path = wl.method.path.permutation(O.N)
    ranks = np.unique(np.concatenate([np.arange(0, O.N, 997), np.arange(T)]))
    nodes = path[ranks]
    ig, cg = G.neighbors()
    io, co = O.neighbors()
    np.testing.assert_array_equal(cg[nodes], co[nodes])
    np.testing.assert_array_equal(ig[nodes], io[nodes])
    z = np.random.default_rng(3).standard_normal((wl.nreals, O.N))
    vg = G.simulate(wl.nreals, z)
    vo = O.simulate(wl.nreals, z, t_end=T)
    first = path[:T]
    assert rel_err(vg[:, first], vo[:, first]) <= VALUE_TOL


def test_c4_sampled_neighbours_and_prefix_values(oracle_mod, geosgs_lib):
    """Full 256^3 grid (16.8 M nodes), unconditional, rotated ellipsoid, k=32,
    both precisions: neighbours of every 4,001st path rank and of the first
    3,000 ranks bit-exact, and the values of the first 3,000 path nodes (which
    depend only on earlier ones) within 1e-6."""
    for precision in ("fp32", "fp64"):
        wl = workloads.c4(precision=precision, nreals=4)
        p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
        G = gpu_plan(p, keep)
        O = oracle_mod.OraclePlan(p, keep)
        T = 3000
        O.search(oracle_mod.TEMPLATE, stride=4001)
        O.search(oracle_mod.TEMPLATE, t1=T)
        O.solve(t1=T)
        path = wl.method.path.permutation(O.N)
        ranks = np.unique(np.concatenate([np.arange(0, O.N, 4001), np.arange(T)]))
        nodes = path[ranks]
        ig, cg = G.neighbors()
        io, co = O.neighbors()
        np.testing.assert_array_equal(cg[nodes], co[nodes])
        np.testing.assert_array_equal(ig[nodes], io[nodes])
        first = path[:T]
        z = np.random.default_rng(6).standard_normal((wl.nreals, O.N))
        vg = G.simulate(wl.nreals, z)
        vo = O.simulate(wl.nreals, z, t_end=T)
        assert rel_err(vg[:, first], vo[:, first]) <= VALUE_TOL, precision
        G.close()


def test_levels_schedule_is_valid(geosgs_lib):
    wl = workloads.small(n=50, k=16, ndata=30, precision="fp32")
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = gpu_plan(p, keep)
    lv, nl = G.levels()
    idx, cnt = G.neighbors()
    N = G.N
    nb = np.where((idx >= 0) & (idx < N), idx, -1)
    prev = np.where(nb >= 0, lv[np.maximum(nb, 0)], -1).max(axis=1)
    np.testing.assert_array_equal(lv, prev + 1)
    assert nl == lv.max() + 1


def test_reference_datum_reproduction_gpu(geosgs_lib):
    """test/field.jl:79-86 through the public rand API on the GPU."""
    grid = geosgs.CartesianGrid((0.5, 0.5), (100.5, 100.5), dims=(100, 100))
    data = geosgs.georef({"Z": [1.0, 0.0, 1.0]}, [(25.0, 25.0), (50.0, 75.0), (75.0, 50.0)])
    proc = geosgs.GaussianProcess(geosgs.SphericalVariogram(range=35.0))
    for prec in ("fp64", "fp32"):
        real = geosgs.rand(np.random.default_rng(2017), proc, grid, data=data,
                           method=geosgs.GPUSEQSIM(maxneighbors=3, precision=prec))
        assert real["Z"].dtype == np.float64
        assert abs(real["Z"][grid.linear_index(24, 24)] - 1.0) <= 1e-4
        ens = geosgs.rand(np.random.default_rng(1), proc, grid, 3, data=data,
                          method=geosgs.GPUSEQSIM(maxneighbors=3, precision=prec))
        assert len(ens) == 3 and ens[2]["Z"].shape == (grid.nelements(),)


@pytest.mark.parametrize("staged", [False, True])
def test_simulate_into_pinned_host_memory(staged, geosgs_lib):
    """A page-locked output buffer is written by the transposing kernel
    directly, or (SGS_FLAG_OUTPUT_STAGED) through device buffers moved by the
    copy engines in chunks; the values equal those returned through pageable
    memory."""
    import ctypes as C

    torch = pytest.importorskip("torch")
    for precision in ("fp32", "fp64"):
        wl = workloads.small(n=40, k=12, ndata=10, vario="exp", nugget=0.05, precision=precision, nreals=12)
        p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
        if staged:
            p.flags |= _abi.SGS_FLAG_OUTPUT_STAGED
        G = gpu_plan(p, keep)
        z = np.random.default_rng(4).standard_normal((12, G.N))
        a = G.simulate(12, z)
        out = torch.empty((12, G.N), dtype=torch.float64, pin_memory=True)
        G._check(G.lib.sgs_plan_simulate(G.h, 12, z.ctypes.data_as(C.POINTER(C.c_double)), 0,
                                         C.cast(out.data_ptr(), C.POINTER(C.c_double))))
        np.testing.assert_array_equal(out.numpy(), a)
        G.close()


def test_bounded_wait_gives_up_and_the_context_survives(oracle_mod, geosgs_lib):
    """The dataflow sweep's dependency wait, run on a flag that nothing sets
    (sgs_selftest_bounded_wait), gives up after its limit and reports it; the
    same process then simulates normally (no fault, no hang)."""
    import ctypes as C

    lib = C.CDLL(_abi.LIB_PATH)
    lib.sgs_selftest_bounded_wait.argtypes = [C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    timed_out, elapsed = C.c_int32(0), C.c_int64(0)
    assert lib.sgs_selftest_bounded_wait(50_000_000, C.byref(timed_out), C.byref(elapsed)) == 0
    assert timed_out.value == 1
    assert 50_000_000 <= elapsed.value < 5_000_000_000
    wl = workloads.small(n=30, k=10, ndata=10, nreals=8, precision="fp32")
    G, O = both(wl, oracle_mod, "fp32")
    z = np.random.default_rng(8).standard_normal((8, O.N))
    assert rel_err(G.simulate(8, z), O.simulate(8, z)) <= VALUE_TOL
    G.close()


def test_level_wait_gives_up_and_the_context_survives(oracle_mod, geosgs_lib):
    """The dependency-level kernel's wait, run on two nodes that are each
    other's neighbour (sgs_selftest_levels_wait: neither level can ever be
    known), gives up after its wall-clock limit and reports it; the same
    process then prepares and simulates normally."""
    import ctypes as C

    lib = C.CDLL(_abi.LIB_PATH)
    lib.sgs_selftest_levels_wait.argtypes = [C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
    timed_out, elapsed = C.c_int32(0), C.c_int64(0)
    assert lib.sgs_selftest_levels_wait(50_000_000, C.byref(timed_out), C.byref(elapsed)) == 0
    assert timed_out.value == 1
    assert 50_000_000 <= elapsed.value < 5_000_000_000
    wl = workloads.small(n=30, k=10, ndata=10, nreals=8, precision="fp32")
    G, O = both(wl, oracle_mod, "fp32")
    z = np.random.default_rng(9).standard_normal((8, O.N))
    assert rel_err(G.simulate(8, z), O.simulate(8, z)) <= VALUE_TOL
    G.close()


def test_search_candidate_counts(geosgs_lib):
    """The search counts the candidates it examines (the byte basis of its
    roofline): at least every neighbour it keeps, grid and data apart, and
    the prior count read back from the device matches the status array."""
    wl = workloads.small(dim=3, n=24, nz=8, k=16, ndata=30, vario="exp", ranges=(8.0, 5.0, 3.0),
                         rotation=geosgs.RotZ(30.0), ball=geosgs.MetricBall((8.0, 5.0, 3.0), geosgs.RotZ(30.0)),
                         precision="fp32")
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = gpu_plan(p, keep)
    info = G.info()
    idx, cnt = G.neighbors()
    _, _, st = G.weights()
    G.close()
    rows = [idx[g, :cnt[g]] for g in range(idx.shape[0])]
    n_grid = sum(int(np.sum(r < G.N)) for r in rows)
    n_data = sum(int(np.sum(r >= G.N)) for r in rows)
    assert n_grid > 0 and n_data > 0
    assert info.search_grid_candidates >= n_grid
    assert info.search_data_candidates >= n_data
    assert info.n_prior == int(np.count_nonzero(st))


def test_device_memory_pool_reuse_and_trim(geosgs_lib):
    """Plans draw device memory from the library's pool: a destroyed plan's
    memory stays with the pool (device free memory does not come back), the
    next plan of the same size reuses it (free memory does not drop again),
    values are unchanged, and sgs_trim_memory returns it to the device."""
    torch = pytest.importorskip("torch")
    wl = workloads.c3("fp32", nreals=16, dims=(80, 80, 40), ndata=400)
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    geosgs.trim_memory(-1)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    outs, frees = [], []
    for _ in range(2):
        G = geosgs.Plan(p, keep).prepare()
        outs.append(G.simulate(16, seed=5))
        G.close()
        torch.cuda.synchronize()
        frees.append(torch.cuda.mem_get_info()[0])
    np.testing.assert_array_equal(outs[0], outs[1])
    MB = 1 << 20
    assert frees[0] < free0 - 64 * MB  # kept by the pool
    assert abs(frees[1] - frees[0]) <= 64 * MB  # reused, not mapped again
    geosgs.trim_memory(0)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0 - 64 * MB


def test_error_codes(geosgs_lib):
    from geosgs import _abi

    wl = workloads.small(n=10, k=4)
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = geosgs.Plan(p, keep)
    with pytest.raises(geosgs.GeoSGSError) as e:
        G.simulate(2)
    assert e.value.code == _abi.SGS_ERR_STATE
    p.maxneighbors = 65
    with pytest.raises(geosgs.GeoSGSError) as e:
        geosgs.Plan(p, keep)
    assert e.value.code == _abi.SGS_ERR_ARG
    p.maxneighbors = 4
    bad = np.zeros(100, dtype=np.int32)
    import ctypes as C

    p.path = bad.ctypes.data_as(C.POINTER(C.c_int32))
    with pytest.raises(geosgs.GeoSGSError) as e:
        geosgs.Plan(p, (keep, bad))
    assert e.value.code == _abi.SGS_ERR_ARG
    # the path ranks are built and checked on the device: a node outside the
    # grid, a repeated node (with one node missing) and a valid reversed path
    for case, expect in (("outside", _abi.SGS_ERR_ARG), ("repeat", _abi.SGS_ERR_ARG), ("reversed", 0)):
        path = np.arange(99, -1, -1, dtype=np.int32)
        if case == "outside":
            path[17] = 100
        elif case == "repeat":
            path[17] = path[18]
        p.path = path.ctypes.data_as(C.POINTER(C.c_int32))
        if expect:
            with pytest.raises(geosgs.GeoSGSError) as e:
                geosgs.Plan(p, (keep, path))
            assert e.value.code == expect, case
            assert "permutation" in str(e.value)
        else:
            G = geosgs.Plan(p, (keep, path)).prepare()
            lv, _ = G.levels()
            G.close()
            assert lv[path[0]] == 0


SWEEP_FORMS = [
    dict(mode=_abi.SGS_SWEEP_FLOW),                                   # default dataflow mapping
    dict(mode=_abi.SGS_SWEEP_FLOW, chunk=2, lanes_w=8),                # rows cut into pieces
    dict(mode=_abi.SGS_SWEEP_FLOW, chunk=4, lanes_g=2, tight=1, blocks_per_sm=1),
    dict(mode=_abi.SGS_SWEEP_FLOW, lanes_w=4, tight=1, level_lo=0, level_hi=3),  # per-level launches first
    dict(mode=_abi.SGS_SWEEP_FLOW, level_lo=5, level_hi=12),           # dataflow, per-level, dataflow
    dict(mode=_abi.SGS_SWEEP_FLOW, level_lo=0, level_hi=10 ** 6),      # every level by per-level launches
    dict(mode=_abi.SGS_SWEEP_LEVELS),
    dict(mode=_abi.SGS_SWEEP_LEVELS, lanes_g=2),                       # two chunks per thread (R > 64)
    dict(mode=_abi.SGS_SWEEP_LEVELS, lanes_g=4),                       # four chunks per thread
    dict(mode=_abi.SGS_SWEEP_LEVELS, lanes_g=2, split_nodes=40),       # small levels: block per node
    dict(mode=_abi.SGS_SWEEP_LEVELS, split_nodes=1 << 30),             # every level: block per node
    dict(mode=_abi.SGS_SWEEP_FLOW, lanes_w=2, lanes_g=2, level_lo=6, level_hi=10 ** 6, split_nodes=30),
    dict(mode=_abi.SGS_SWEEP_COOPERATIVE),
]


@pytest.mark.parametrize("nreals", [4, 8, 12, 64, 200, 256, 520])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_sweep_variants_agree_with_oracle(precision, nreals, oracle_mod, geosgs_lib):
    """Every form of the sweep matches the oracle: the persistent dataflow
    launch (rows cut into independent pieces, 1 or 2 chunks of 4
    realizations per lane, neighbour lists split over lane slices, 1-4 items
    per ticket, register-capped variants, reduced residency, leading levels
    by per-level launches), one launch per level (thread per chunk, or warp
    per node for R <= 64), and one cooperative launch with grid barriers
    between levels."""
    wl = workloads.small(n=48, k=16, ndata=25, vario="gau", nugget=0.02, precision=precision, nreals=nreals)
    z = np.random.default_rng(nreals).standard_normal((nreals, 48 * 48))
    G, O = both(wl, oracle_mod, precision)
    ref = O.simulate(nreals, z)
    for form in SWEEP_FORMS:
        G.set_sweep(**form)
        assert rel_err(G.simulate(nreals, z), ref) <= VALUE_TOL, form
        # seeded draws: the same values whatever the form
        if form is SWEEP_FORMS[0]:
            seeded = G.simulate(nreals, seed=5)
        else:
            assert rel_err(G.simulate(nreals, seed=5), seeded) <= VALUE_TOL, form
    G.close()


def test_sweep_autotuner_keeps_the_fastest_form(oracle_mod, geosgs_lib):
    wl = workloads.small(n=64, k=24, ndata=40, vario="exp", nugget=0.05, precision="fp32", nreals=64)
    z = np.random.default_rng(3).standard_normal((64, 64 * 64))
    G, O = both(wl, oracle_mod, "fp32")
    chosen, tried = G.tune_sweep(64)
    assert len(tried) >= 4 and all(t["ms"] > 0 for t in tried)
    assert chosen["ms"] == min(t["ms"] for t in tried)
    assert rel_err(G.simulate(64, z), O.simulate(64, z)) <= VALUE_TOL
    G.close()


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_nested_variogram_parity(dim, precision, oracle_mod, geosgs_lib):
    """A nested model (spherical + exponential + gaussian structures, each
    with its own ranges, rotation, sill and nugget) with data: neighbours
    bit-exact, status identical, weights and values against the oracle."""
    from test_oracle import _nested_case

    proc, grid, data, method = _nested_case(precision, dim)
    p, keep = geosgs.build_problem(proc, grid, data, method)
    G = gpu_plan(p, keep)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    np.testing.assert_array_equal(G.neighbors()[0], O.neighbors()[0])
    wg, sg, stg = G.weights()
    wo, so, sto = O.weights()
    np.testing.assert_array_equal(stg, sto)
    tol = 1e-9 if precision == "fp64" else 1e-6
    np.testing.assert_allclose(wg, wo, rtol=0, atol=tol)
    np.testing.assert_allclose(sg, so, rtol=0, atol=tol)
    z = np.random.default_rng(12).standard_normal((6, O.N))
    assert rel_err(G.simulate(6, z), O.simulate(6, z)) <= VALUE_TOL
    G.close()

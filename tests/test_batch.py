"""Batches of independent domains (sgs_batch_*, include/geosgs.h) against the
FP64 oracle, domain by domain.

A batch prepares and simulates many problems together (one launch per
phase over all domains, systems solved in size classes, a persistent
dataflow sweep, CUDA graphs for prepare and the seeded sweep); each domain's
results must equal what the oracle gives for that domain alone: neighbour
rows and counts bit-exact, node status identical, weights within 1e-9
(FP64) / 1e-6 (FP32 refined), values within 1e-6 relative
(max |v_gpu - v_oracle| / max(|v_oracle|, 1))."""
import numpy as np
import pytest

import geosgs
from geosgs import _abi, workloads

VALUE_TOL = 1e-6


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0))) if a.size else 0.0


def problems_of(bw, precision):
    out = []
    for w in bw.items:
        w.method.precision = precision
        out.append(geosgs.build_problem(w.process, w.domain, w.data, w.method))
    return out


def test_c5_generator_is_seeded_and_in_range():
    a, b = workloads.c5_small(), workloads.c5_small()
    assert [w.domain.dims for w in a.items] == [w.domain.dims for w in b.items]
    full = workloads.c5()
    assert len(full.items) == 1000 and full.nreals == 8
    dims = [len(w.domain.dims) for w in full.items]
    assert 400 < dims.count(3) < 600
    for w in full.items:
        d = w.domain.dims
        assert all(32 <= s <= 256 for s in d[:2])
        if len(d) == 3:
            assert 8 <= d[2] <= 64
        assert 5.0 <= w.process.func.range() <= 80.0
        assert w.method.maxneighbors in (8, 16, 32, 48)
        assert w.data is None or 1 <= w.data.nrow() <= 500


def test_batch_argument_errors():
    """Argument validation happens before any device work (runs without a
    GPU); the paths are checked on the device (see below)."""
    from geosgs import _build

    _build.build()
    bw = workloads.c5_small(ndomains=3)
    probs = problems_of(bw, "fp32")
    probs[1][0].precision = _abi.SGS_PREC_FP64
    with pytest.raises(geosgs.GeoSGSError) as e:
        geosgs.Batch(probs)
    assert e.value.code == _abi.SGS_ERR_ARG and "domain 1" in str(e.value)
    probs = problems_of(bw, "fp32")
    probs[2][0].maxneighbors = 65
    with pytest.raises(geosgs.GeoSGSError) as e:
        geosgs.Batch(probs)
    assert e.value.code == _abi.SGS_ERR_ARG and "domain 2" in str(e.value)
    probs = problems_of(bw, "fp32")
    probs[0][0].warm_start = 1
    with pytest.raises(geosgs.GeoSGSError) as e:
        geosgs.Batch(probs)
    assert e.value.code == _abi.SGS_ERR_ARG


@pytest.mark.gpu
def test_batch_path_checked_on_the_device(geosgs_lib):
    """The path ranks of a batch are built and checked on the device: a
    domain whose path repeats a node (or leaves the domain) is rejected with
    SGS_ERR_ARG naming the first such domain; a valid batch then works."""
    import ctypes as C

    bw = workloads.c5_small(ndomains=3)
    for case in ("repeat", "outside"):
        probs = problems_of(bw, "fp32")
        p2, keep2 = probs[2]
        n = int(np.prod([p2.dims[j] for j in range(p2.dim)]))
        path = np.arange(n - 1, -1, -1, dtype=np.int32)
        if case == "repeat":
            path[3] = path[4]
        else:
            path[5] = n
        p2.path = path.ctypes.data_as(C.POINTER(C.c_int32))
        probs[2] = (p2, (keep2, path))
        with pytest.raises(geosgs.GeoSGSError) as e:
            geosgs.Batch(probs)
        assert e.value.code == _abi.SGS_ERR_ARG and "domain 2" in str(e.value) and "permutation" in str(e.value)
    B = geosgs.Batch(problems_of(bw, "fp32")).prepare()
    assert B.info().nnodes == bw.nodes()
    B.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_matches_oracle_per_domain(precision, oracle_mod, geosgs_lib):
    bw = workloads.c5_small(precision)
    probs = problems_of(bw, precision)
    B = geosgs.Batch(probs).prepare()
    info = B.info()
    assert info.ndomains == len(probs) and info.nnodes == B.nnodes
    assert info.graph_launches == 1 and sum(info.bin_systems) == B.nnodes
    R = bw.nreals
    zs = [np.random.default_rng(100 + d).standard_normal((R, int(B.sizes[d]))) for d in range(len(probs))]
    vals = B.simulate(R, z=zs)
    priors = 0
    for d, (p, keep) in enumerate(probs):
        O = oracle_mod.OraclePlan(p, keep).prepare()
        ig, cg = B.neighbors(d)
        io, co = O.neighbors()
        np.testing.assert_array_equal(cg, co, err_msg=f"domain {d}")
        np.testing.assert_array_equal(ig, io, err_msg=f"domain {d}")
        wg, sg, stg = B.weights(d)
        wo, so, sto = O.weights()
        np.testing.assert_array_equal(stg, sto, err_msg=f"domain {d}")
        tol = 1e-9 if precision == "fp64" else 1e-6
        np.testing.assert_allclose(wg, wo, rtol=0, atol=tol, err_msg=f"domain {d}")
        np.testing.assert_allclose(sg, so, rtol=0, atol=tol, err_msg=f"domain {d}")
        assert rel_err(vals[d], O.simulate(R, zs[d])) <= VALUE_TOL, d
        priors += int(np.count_nonzero(sto))
    assert B.info().n_prior == priors
    B.close()


@pytest.mark.gpu
def test_batch_promotes_amplifying_weights(oracle_mod, geosgs_lib):
    """A domain whose kriging weights amplify FP32 rounding (a nugget-free
    Gaussian variogram, sum |w| ~ 100) keeps FP64 values, read through the
    packed tables, while the domains whose weights do not keep FP32 values
    (the precision is chosen per domain); every domain stays within 1e-6,
    and the device-resident values follow the documented mixed layout."""
    bw = workloads.c5_small("fp32", ndomains=5, seed=63)
    gau = geosgs.GaussianProcess(geosgs.GaussianVariogram(range=6.0, sill=1.0, nugget=0.0), 0.2)
    grid = geosgs.CartesianGrid((20, 20))
    bw.items.append(workloads.Workload("gau", gau, grid, None,
                                       geosgs.GPUSEQSIM(path=geosgs.LinearPath(), maxneighbors=16, precision="fp32"),
                                       bw.nreals))
    probs = problems_of(bw, "fp32")
    B = geosgs.Batch(probs).prepare()
    info = B.info()
    assert info.values_fp64 == 1 and info.weight_l1_max > 10.0
    fp64 = [B.domain_values_fp64(d) for d in range(len(probs))]
    assert fp64[-1] and not all(fp64) and info.domains_fp64 == sum(fp64)
    # the FP64 domains' share of the sweep's grid neighbours: the rows of
    # every kriged node of those domains, from the neighbour tables
    m64 = 0
    for d in range(len(probs)):
        if fp64[d]:
            idx, cnt = B.neighbors(d)
            _, _, st = B.weights(d)
            n = int(B.sizes[d])
            m64 += sum(int(np.sum(idx[g, :cnt[g]] < n)) for g in range(n) if st[g] == 0)
    assert 0 < info.sum_grid_neighbors_fp64 < info.sum_grid_neighbors
    assert info.sum_grid_neighbors_fp64 == m64
    R = bw.nreals
    zs = [np.random.default_rng(200 + d).standard_normal((R, int(B.sizes[d]))) for d in range(len(probs))]
    vals = B.simulate(R, z=zs)
    seeded = B.simulate(R, seed=3)
    zall = oracle_mod.normals(3, B.nnodes, R)
    for d, (p, keep) in enumerate(probs):
        O = oracle_mod.OraclePlan(p, keep).prepare()
        assert rel_err(vals[d], O.simulate(R, zs[d])) <= VALUE_TOL, d
        f, n = int(B.first[d]), int(B.sizes[d])
        assert rel_err(seeded[d], O.simulate(R, zall[:, f:f + n])) <= VALUE_TOL, d
    # device values: FP64 rows of Rp doubles per node, an FP32 domain's floats
    # in the first half of each of its rows; centred (the mean subtracted)
    torch = pytest.importorskip("torch")
    Rp = (R + 3) // 4 * 4
    V = torch.empty(B.nnodes * Rp, dtype=torch.float64, device="cuda")
    B.simulate_device(R, 3, V)
    torch.cuda.synchronize()
    v64 = V.cpu().numpy().reshape(B.nnodes, Rp)
    v32 = v64.view(np.float32).reshape(B.nnodes, 2 * Rp)
    for d, (p, keep) in enumerate(probs):
        f, n = int(B.first[d]), int(B.sizes[d])
        rows = v64[f:f + n, :R] if fp64[d] else v32[f:f + n, :R].astype(np.float64)
        np.testing.assert_allclose(rows.T + p.mean, seeded[d], rtol=0, atol=1e-12)
    B.close()


@pytest.mark.gpu
def test_batch_of_full_size_c5_domains_sampled(oracle_mod, geosgs_lib):
    """The first 10 domains of the C5 batch at full size (3.4 M nodes; 2D and
    3D, sides up to 243, k 8-48, up to 474 data, :range balls up to 37 cells):
    per domain the oracle searches every ~N/600-th path rank and searches and
    solves the first 500 ranks; neighbours of those nodes are bit-exact and
    the values of the first 500 path nodes are within 1e-6."""
    bw = workloads.c5(ndomains=10)
    probs = problems_of(bw, "fp32")
    B = geosgs.Batch(probs).prepare()
    R = 4
    zs = [np.random.default_rng(300 + d).standard_normal((R, int(B.sizes[d]))) for d in range(len(probs))]
    vals = B.simulate(R, z=zs)
    T = 500
    for d, (p, keep) in enumerate(probs):
        O = oracle_mod.OraclePlan(p, keep)
        N = O.N
        stride = max(1, N // 600)
        O.search(oracle_mod.TEMPLATE, stride=stride)
        O.search(oracle_mod.TEMPLATE, t1=T)
        O.solve(t1=T)
        path = bw.items[d].method.path.permutation(N)
        nodes = path[np.unique(np.concatenate([np.arange(0, N, stride), np.arange(T)]))]
        ig, cg = B.neighbors(d)
        io, co = O.neighbors()
        np.testing.assert_array_equal(cg[nodes], co[nodes], err_msg=f"domain {d}")
        np.testing.assert_array_equal(ig[nodes], io[nodes], err_msg=f"domain {d}")
        first = path[:T]
        vo = O.simulate(R, zs[d], t_end=T)
        assert rel_err(vals[d][:, first], vo[:, first]) <= VALUE_TOL, d
    B.close()


@pytest.mark.gpu
def test_batch_edge_cases(oracle_mod, geosgs_lib):
    """A batch of one domain, and a batch holding a one-node domain, a 1D
    domain (as n x 1) and a domain whose maxneighbors exceeds its node count:
    per domain the same neighbours and values as the oracle."""
    def item(dims, k, nd=0, seed=0):
        grid = geosgs.CartesianGrid(dims)
        rng = np.random.default_rng(seed)
        data = None
        if nd:
            ext = np.asarray(grid.dims, dtype=np.float64)
            data = geosgs.georef({"Z": rng.standard_normal(nd)}, rng.uniform(0.0, 1.0, (nd, len(dims))) * ext)
        proc = geosgs.GaussianProcess(geosgs.ExponentialVariogram(range=5.0, nugget=0.05), 0.3)
        method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(seed), maxneighbors=k, precision="fp32")
        return geosgs.build_problem(proc, grid, data, method)

    for probs in ([item((30, 20), 12, nd=5, seed=1)],
                  [item((1, 1), 8, nd=2, seed=2), item((200,), 6, nd=3, seed=3), item((4, 3), 40, seed=4),
                   item((16, 12, 5), 24, nd=10, seed=5)]):
        B = geosgs.Batch(probs).prepare()
        R = 5
        zs = [np.random.default_rng(400 + d).standard_normal((R, int(B.sizes[d]))) for d in range(len(probs))]
        vals = B.simulate(R, z=zs)
        for d, (p, keep) in enumerate(probs):
            O = oracle_mod.OraclePlan(p, keep).prepare()
            ig, cg = B.neighbors(d)
            io, co = O.neighbors()
            np.testing.assert_array_equal(cg, co, err_msg=f"domain {d}")
            np.testing.assert_array_equal(ig, io, err_msg=f"domain {d}")
            assert rel_err(vals[d], O.simulate(R, zs[d])) <= VALUE_TOL, d
        B.close()


@pytest.mark.gpu
def test_batch_graph_replay_and_seeded_draws(oracle_mod, geosgs_lib):
    """Replayed graphs give identical results; seeded draws are Philox keyed
    by the global node id, so the oracle fed those normals agrees."""
    bw = workloads.c5_small("fp32", ndomains=9, seed=61)
    probs = problems_of(bw, "fp32")
    B = geosgs.Batch(probs).prepare()
    R = 12
    a = B.simulate(R, seed=11)
    B.prepare()
    b = B.simulate(R, seed=11)
    c = B.simulate(R, seed=12)
    for d in range(len(probs)):
        np.testing.assert_array_equal(a[d], b[d])
        assert not np.array_equal(a[d], c[d])
    zall = oracle_mod.normals(11, B.nnodes, R)
    for d, (p, keep) in enumerate(probs):
        O = oracle_mod.OraclePlan(p, keep).prepare()
        f, n = int(B.first[d]), int(B.sizes[d])
        assert rel_err(a[d], O.simulate(R, zall[:, f:f + n])) <= VALUE_TOL, d
    assert B.info().graph_launches >= 4
    B.close()


@pytest.mark.gpu
def test_batch_device_values_and_autotuner(oracle_mod, geosgs_lib):
    torch = pytest.importorskip("torch")
    bw = workloads.c5_small("fp32", ndomains=7, seed=62)
    probs = problems_of(bw, "fp32")
    B = geosgs.Batch(probs).prepare()
    R = 8
    chosen, tried = B.tune_sweep(R)
    assert len(tried) >= 2 and chosen["ms"] == min(t["ms"] for t in tried)
    host = B.simulate(R, seed=5)
    # the same realizations written straight into page-locked host memory
    import ctypes as C

    pinned = torch.empty(R * B.nnodes, dtype=torch.float64, pin_memory=True)
    B._check(B.lib.sgs_batch_simulate(B.h, R, None, C.c_uint64(5), C.cast(pinned.data_ptr(), C.POINTER(C.c_double))))
    np.testing.assert_array_equal(pinned.numpy(), np.concatenate([h.reshape(-1) for h in host]))
    V = torch.empty((B.nnodes, R), dtype=torch.float64 if B.values_fp64() else torch.float32, device="cuda")
    B.simulate_device(R, 5, V)
    info = B.info()
    assert info.ms_sweep > 0
    Vn = V.cpu().numpy()
    for d, w in enumerate(bw.items):
        f, n = int(B.first[d]), int(B.sizes[d])
        if not B.values_fp64():
            rows = Vn[f:f + n].astype(np.float64)
        elif B.domain_values_fp64(d):
            rows = Vn[f:f + n]
        else:  # FP32 values in the first half of the domain's FP64 rows
            rows = Vn.view(np.float32).reshape(B.nnodes, 2 * R)[f:f + n, :R].astype(np.float64)
        dev = rows.T + w.process.mean
        assert rel_err(dev, host[d]) <= 1e-7, d
    B.close()

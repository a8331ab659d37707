"""Two widenings of the path: ensemble statistics on the device
(sgs_ensemble_*, the reference's src/ensembles.jl:42-52) and per-realization
paths (the reference redraws a RandomPath's permutation for every
realization, src/simulation/field/seqsim.jl:98).

Statistics are compared with numpy on the same realizations (mean, var with
ddof=1, cdf, ccdf, numpy's default 'linear' quantile) within 1e-12;
per-realization simulations with the oracle run on each realization's own
permutation, within 1e-6 relative."""
import numpy as np
import pytest

import geosgs
from geosgs import workloads

VALUE_TOL = 1e-6


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0))) if a.size else 0.0


def test_random_path_permutations_are_successive_draws():
    p = geosgs.RandomPath(9)
    perms = p.permutations(50, 3)
    np.testing.assert_array_equal(perms[0], p.permutation(50))
    assert not np.array_equal(perms[0], perms[1]) and not np.array_equal(perms[1], perms[2])
    assert all(np.array_equal(np.sort(q), np.arange(50)) for q in perms)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_device_ensemble_statistics(precision, geosgs_lib):
    torch = pytest.importorskip("torch")
    from geosgs import ensemble

    wl = workloads.small(n=30, k=12, ndata=15, vario="exp", nugget=0.05, precision=precision)
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = geosgs.Plan(p, keep).prepare()
    R, Rp = 37, 40
    dt = torch.float64 if G.values_fp64() else torch.float32
    V = torch.empty((G.N, Rp), dtype=dt, device="cuda")
    # the sweep and the statistics on one stream (a NULL stream handle, as
    # torch's default stream has, would select the plan's own stream)
    st = torch.cuda.Stream()
    mu = 0.75
    xs = [-1.0, 0.0, 0.75, 2.5]
    ps = [0.0, 0.1, 0.5, 0.9, 1.0]
    with torch.cuda.stream(st):
        G.simulate_device(R, None, 3, V, st.cuda_stream)
        m, v = ensemble.mean_var(V, R, Rp, offset=mu)
        c = ensemble.cdf(V, R, xs, Rp, offset=mu)
        cc = ensemble.cdf(V, R, xs, Rp, offset=mu, complement=True)
        q = ensemble.quantile(V, R, ps, Rp, offset=mu)
    torch.cuda.synchronize()
    vals = V.cpu().numpy().astype(np.float64)[:, :R] + mu
    np.testing.assert_allclose(m.cpu().numpy(), vals.mean(axis=1), rtol=0, atol=1e-12)
    np.testing.assert_allclose(v.cpu().numpy(), vals.var(axis=1, ddof=1), rtol=0, atol=1e-12)
    np.testing.assert_array_equal(c.cpu().numpy(), np.stack([(vals <= x).mean(axis=1) for x in xs], axis=1))
    np.testing.assert_array_equal(cc.cpu().numpy(), np.stack([(vals > x).mean(axis=1) for x in xs], axis=1))
    np.testing.assert_allclose(q.cpu().numpy(), np.quantile(vals, ps, axis=1).T, rtol=0, atol=1e-12)
    G.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_per_realization_paths_match_oracle(precision, oracle_mod, geosgs_lib):
    wl = workloads.small(n=28, k=10, ndata=12, vario="sph", nugget=0.0, precision=precision)
    R = 4
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(21), maxneighbors=10, precision=precision,
                              path_per_realization=True)
    z = np.random.default_rng(5).standard_normal((R, wl.domain.nelements()))
    ens = geosgs.rand(np.random.default_rng(1), wl.process, wl.domain, R, data=wl.data, method=method, z=z)
    perms = geosgs.RandomPath(21).permutations(wl.domain.nelements(), R)
    for r in range(R):
        m = geosgs.GPUSEQSIM(path=geosgs.ExplicitPath(perms[r]), maxneighbors=10, precision="fp64")
        p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, m)
        O = oracle_mod.OraclePlan(p, keep).prepare()
        assert rel_err(ens[r]["Z"][None, :], O.simulate(1, z[r:r + 1])) <= VALUE_TOL, r


@pytest.mark.gpu
def test_per_realization_indicator_paths_match_oracle(oracle_mod, geosgs_lib):
    """An IndicatorProcess with per-realization paths: realization r follows
    the r-th permutation of the RandomPath's generator, categories identical
    to the oracle's on that permutation and the same uniforms."""
    from geosgs import problem as gproblem

    wl = workloads.small(n=26, k=10, ndata=14, vario="sph", nugget=0.0, seed=4)
    R = 3
    rng = np.random.default_rng(8)
    labels = rng.integers(0, 3, wl.data.nrow())
    labels[:3] = [0, 1, 2]
    data = geosgs.georef({"C": labels}, wl.data.coords)
    proc = geosgs.IndicatorProcess(geosgs.SphericalTransiogram(range=6.0, proportions=(0.5, 0.3, 0.2)))
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(17), maxneighbors=10, path_per_realization=True)
    u = rng.uniform(0.0, 1.0, (R, wl.domain.nelements()))
    ens = geosgs.rand(np.random.default_rng(1), proc, wl.domain, R, data=data, method=method, z=u)
    perms = geosgs.RandomPath(17).permutations(wl.domain.nelements(), R)
    levels, dcat = gproblem.indicator_levels(proc, data)
    for r in range(R):
        m = geosgs.GPUSEQSIM(path=geosgs.ExplicitPath(perms[r]), maxneighbors=10)
        p, keep = geosgs.build_problem(proc, wl.domain, data, m)
        O = oracle_mod.OraclePlan(p, keep).prepare()
        want = np.asarray(levels)[O.simulate_indicator(1, proc.prob, dcat, u=u[r:r + 1])[0]]
        np.testing.assert_array_equal(ens[r]["C"], want)
    # the shared-path form differs: every realization on the first permutation
    shared = geosgs.rand(np.random.default_rng(1), proc, wl.domain, R, data=data, z=u,
                         method=geosgs.GPUSEQSIM(path=geosgs.RandomPath(17), maxneighbors=10))
    np.testing.assert_array_equal(shared[0]["C"], ens[0]["C"])


def test_ensemble_container_api():
    """Iteration, indexing (an int or a list) and fetch, as src/ensembles.jl:
    10-35 (no device work)."""
    grid = geosgs.CartesianGrid((3, 2))
    reals = [{"a": np.arange(6.0) + r, "b": -np.arange(6.0)} for r in range(4)]
    ens = geosgs.Ensemble(grid, reals)
    assert len(ens) == 4 and ens.variables() == ["a", "b"]
    assert [r["a"][0] for r in ens] == [0.0, 1.0, 2.0, 3.0]
    assert [r["a"][1] for r in ens[[3, 1]]] == [4.0, 2.0]
    doubled = geosgs.Ensemble(grid, reals, fetch=lambda real: {k: 2 * v for k, v in real.items()})
    assert doubled[2]["a"][5] == 14.0
    with pytest.raises(geosgs.ArgumentError):
        geosgs.Ensemble(grid, [{"c": np.array(["x", "y"])}])._rows("c")


@pytest.mark.gpu
def test_ensemble_statistics_through_the_public_api(geosgs_lib):
    """Ensemble.mean/var/cdf/ccdf/quantile of rand's realizations on the
    device against numpy on the same values, for every variable."""
    proc = geosgs.GaussianProcess(geosgs.LinearCoregionalization([
        (np.array([[1.0, 0.3], [0.3, 0.5]]), geosgs.SphericalVariogram(range=5.0))]), [0.5, -1.0])
    grid = geosgs.CartesianGrid((20, 16))
    ens = geosgs.rand(np.random.default_rng(4), proc, grid, 9,
                      method=geosgs.GPUSEQSIM(path=geosgs.RandomPath(2), maxneighbors=12))
    m, v = ens.mean(), ens.var()
    assert sorted(m) == ["field1", "field2"]
    for name in ("field1", "field2"):
        vals = np.stack([r[name] for r in ens])
        np.testing.assert_allclose(m[name], vals.mean(axis=0), rtol=0, atol=1e-12)
        np.testing.assert_allclose(v[name], vals.var(axis=0, ddof=1), rtol=0, atol=1e-12)
        np.testing.assert_array_equal(ens.cdf(0.25, name), (vals <= 0.25).mean(axis=0))
        np.testing.assert_array_equal(ens.ccdf(0.25, name), (vals > 0.25).mean(axis=0))
        q = ens.quantile([0.1, 0.5], name)
        np.testing.assert_allclose(q[0], np.quantile(vals, 0.1, axis=0), rtol=0, atol=1e-12)
        np.testing.assert_allclose(q[1], np.quantile(vals, 0.5, axis=0), rtol=0, atol=1e-12)

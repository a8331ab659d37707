"""Posterior mean by simple kriging from the data (sgs_krige) and the
reference's expectation API (mean / expectedvalue,
src/expectation/field.jl:17-42, src/expectation/field/gaussian.jl:5-25).

The oracle's kriging (oracle_krige) is pinned first, on the CPU: closed
forms (one datum: mean = mu + C(h)/C(0) (d - mu), var = sill - C(h)^2 /
sill), exact interpolation at data on cell centres, the prior without data,
NaN below minneighbors, and an independent numpy restatement (brute-force
neighbours, numpy.linalg.solve).  The GPU is then compared with the oracle:
mean and variance within 1e-10 (FP64) / 1e-6 (FP32 + refinement), NaN at
the same nodes."""
import numpy as np
import pytest

import geosgs
from geosgs import simulation, workloads


def problem_of(wl, precision="fp64", k=10, nmin=1, neighborhood=None):
    opts = simulation._KrigingOptions(maxneighbors=k, minneighbors=nmin, neighborhood=neighborhood,
                                      precision=precision)
    return geosgs.build_problem(wl.process, wl.domain, wl.data, opts)


def case(dim=2, n=20, ndata=30, vario="exp", nugget=0.05, seed=0, ranges=(6.0, 6.0, 6.0), rotation=None):
    return workloads.small(dim=dim, n=n, k=8, ndata=ndata, vario=vario, seed=seed, nugget=nugget, ranges=ranges,
                           rotation=rotation)


def numpy_krige(wl, k, nmin, radius, oracle_mod):
    """Independent restatement: Euclidean distances to every datum, the k
    nearest (ties by index) within `radius` (None: no radius), SK solved
    by numpy."""
    p, keep = problem_of(wl, "fp64", k, nmin)
    grid = wl.domain
    X = grid.centroids()
    D = wl.data.coords
    d = next(iter(wl.data.values.values()))
    mu = wl.process.mean
    sill = p.variogram.sill
    dim = grid.dim
    cov = lambda h: oracle_mod.covariance(p.variogram, dim, h)  # noqa: E731
    mean = np.full(len(X), np.nan)
    var = np.full(len(X), np.nan)
    for g, x in enumerate(X):
        dd = np.sum((D - x) ** 2, axis=1)
        idx = [i for i in np.lexsort((np.arange(len(D)), dd)) if radius is None or dd[i] <= radius * radius][:k]
        if len(idx) < nmin:
            continue
        K = np.array([[cov(D[j] - D[i]) for j in idx] for i in idx])
        c = np.array([cov(x - D[i]) for i in idx])
        w = np.linalg.solve(K, c)
        mean[g] = mu + w @ (d[idx] - mu)
        var[g] = max(sill - w @ c, 0.0)
    return mean, var


def test_oracle_krige_matches_numpy(oracle_mod):
    wl = case(dim=2, n=16, ndata=25, seed=3)
    for k, radius in ((6, None), (4, 5.0)):
        nb = None if radius is None else geosgs.MetricBall(radius)
        p, keep = problem_of(wl, "fp64", k, 1, nb)
        m, v = oracle_mod.OraclePlan(p, keep).krige()
        mn, vn = numpy_krige(wl, k, 1, radius, oracle_mod)
        np.testing.assert_array_equal(np.isnan(m), np.isnan(mn))
        ok = ~np.isnan(mn)
        np.testing.assert_allclose(m[ok], mn[ok], rtol=0, atol=1e-11)
        np.testing.assert_allclose(v[ok], vn[ok], rtol=0, atol=1e-11)


def test_oracle_krige_closed_forms(oracle_mod):
    grid = geosgs.CartesianGrid((12, 9))
    proc = geosgs.GaussianProcess(geosgs.SphericalVariogram(range=7.0, sill=2.0, nugget=0.1), 0.5)
    data = geosgs.georef({"Z": np.array([1.7])}, np.array([[3.3, 4.1]]))
    wl = workloads.Workload("one", proc, grid, data, None, 1)
    p, keep = problem_of(wl, "fp64", k=1)
    m, v = oracle_mod.OraclePlan(p, keep).krige()
    X = grid.centroids()
    for g in range(grid.nelements()):
        h = np.array([3.3, 4.1]) - X[g]
        c = oracle_mod.covariance(p.variogram, 2, h)
        assert abs(m[g] - (0.5 + c / 2.0 * (1.7 - 0.5))) < 1e-13
        assert abs(v[g] - (2.0 - c * c / 2.0)) < 1e-13
    # exact interpolation at data on cell centres, zero variance there
    cells = [5, 40, 77]
    vals = np.array([2.0, -1.0, 0.25])
    data = geosgs.georef({"Z": vals}, X[cells])
    wl = workloads.Workload("cc", proc, grid, data, None, 1)
    p, keep = problem_of(wl, "fp64", k=3)
    m, v = oracle_mod.OraclePlan(p, keep).krige()
    np.testing.assert_allclose(m[cells], vals, rtol=0, atol=1e-12)
    np.testing.assert_allclose(v[cells], 0.0, rtol=0, atol=1e-12)
    # minneighbors above the data count (minneighbors <= maxneighbors, else
    # the clamp of seqsim.jl:202-208 resets it to 1): missing everywhere
    data = geosgs.georef({"Z": vals[:2]}, X[cells[:2]])
    wl = workloads.Workload("two", proc, grid, data, None, 1)
    p, keep = problem_of(wl, "fp64", k=3, nmin=3)
    m, v = oracle_mod.OraclePlan(p, keep).krige()
    assert np.isnan(m).all() and np.isnan(v).all()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gpu_krige_matches_oracle(precision, oracle_mod, geosgs_lib):
    tol = 1e-10 if precision == "fp64" else 1e-6
    cases = [
        (case(dim=2, n=40, ndata=60, vario="exp", seed=1), 10, 1, None),
        (case(dim=2, n=32, ndata=50, vario="gau", nugget=0.02, seed=2), 8, 3, geosgs.MetricBall(7.0)),
        (case(dim=3, n=20, ndata=80, vario="sph", seed=3, ranges=(8.0, 5.0, 3.0), rotation=geosgs.RotZ(30.0)), 12,
         1, geosgs.MetricBall((9.0, 6.0, 3.0), geosgs.RotZ(30.0))),
        (workloads.c2(), 10, 1, None),
    ]
    for wl, k, nmin, nb in cases:
        p, keep = problem_of(wl, precision, k, nmin, nb)
        m, v = geosgs.posterior(wl.process, wl.domain, wl.data, maxneighbors=k, minneighbors=nmin,
                                neighborhood=nb, precision=precision)
        mo, vo = oracle_mod.OraclePlan(p, keep).krige()
        np.testing.assert_array_equal(np.isnan(m), np.isnan(mo))
        ok = ~np.isnan(mo)
        np.testing.assert_allclose(m[ok], mo[ok], rtol=0, atol=tol)
        np.testing.assert_allclose(v[ok], vo[ok], rtol=0, atol=tol)


@pytest.mark.gpu
def test_mean_api(geosgs_lib, oracle_mod):
    wl = case(dim=2, n=24, ndata=20, seed=4)
    prior = geosgs.mean(wl.process, wl.domain)
    assert np.all(prior["field"] == wl.process.mean)
    post = geosgs.expectedvalue(wl.process, wl.domain, data=wl.data)
    m, _ = geosgs.posterior(wl.process, wl.domain, wl.data)
    np.testing.assert_array_equal(post["Z"], m)

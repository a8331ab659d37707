"""Multivariate Gaussian simulation: a GaussianProcess(func, mean) whose
func is a linear model of coregionalization of L variables, simulated with
SEQSIM (src/processes/field/gaussian.jl:22-35; src/simulation/field/
seqsim.jl:277-290 Kriging(func, mean) and the MvNormal(mean, sill(func))
prior, :302-304 predictprob's MvNormal conditional, :335-340 one draw for
all variables of a node; sgs_plan_set_multivariate /
sgs_plan_simulate_multivariate).

The oracle's restatement (oracle_simulate_multivariate) is pinned on the CPU
by reductions to the univariate oracle, which the golden fixtures pin: with
one variable it is univariate SEQSIM on the same structures; with diagonal
coregionalization matrices each variable is an independent univariate
simulation of its own sill.  An independent numpy restatement (the model's
own variogram functions, numpy.linalg.solve and cholesky) checks the
cross-covariance terms on a non-diagonal nested model.  Also checked: a node
on a datum, visited first,
takes the datum's values in every realization, and prior draws have the
model's covariance C(0).  The GPU is then compared with the oracle on the
same normals, within the project's value bar (max |a - b| / max(|b|, 1)
<= 1e-6), and on seeded draws within the FP32 Box-Muller's rounding."""
import numpy as np
import pytest

import geosgs
from geosgs import problem as gproblem
from geosgs import workloads

VALUE_TOL = 1e-6


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0))) if a.size else 0.0


def lmc(L=2, nugget=0.0):
    """A non-separable model: a short isotropic spherical structure and a
    longer anisotropic exponential one with their own coregionalization."""
    A1 = np.array([[1.0, 0.4, -0.2], [0.4, 0.8, 0.1], [-0.2, 0.1, 0.6]])[:L, :L]
    A2 = np.array([[0.5, -0.1, 0.2], [-0.1, 0.3, 0.05], [0.2, 0.05, 0.4]])[:L, :L]
    return geosgs.LinearCoregionalization([
        (A1, geosgs.SphericalVariogram(range=5.0, nugget=nugget)),
        (A2, geosgs.ExponentialVariogram(ranges=(12.0, 6.0, 4.0), rotation=geosgs.RotZ(20.0))),
    ])


def mv_data(rng, ndata, dims, L):
    xyz = rng.uniform(0.0, 1.0, (ndata, len(dims))) * np.asarray(dims, dtype=np.float64)
    return geosgs.georef({f"V{a}": rng.standard_normal(ndata) for a in range(L)}, xyz)


def oracle_mv(oracle_mod, proc, grid, data, method, R, z=None, seed=0):
    p, keep = geosgs.build_problem(proc, grid, data, method)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    return O, O.simulate_multivariate(R, proc.mean, proc.func.coef, gproblem.multivariate_data(proc, data),
                                      z=z, seed=seed)


def test_process_mirror():
    f = lmc(3)
    proc = geosgs.GaussianProcess(f)
    assert proc.nvariables == 3 and proc.mean == (0.0, 0.0, 0.0)
    with pytest.raises(geosgs.ArgumentError):  # gaussian.jl:28-30
        geosgs.GaussianProcess(f, [0.0, 1.0])
    assert geosgs.GaussianProcess(geosgs.SphericalVariogram(range=3.0), [2.0]).mean == 2.0
    with pytest.raises(geosgs.ArgumentError):
        geosgs.GaussianProcess(geosgs.SphericalVariogram(range=3.0), [1.0, 2.0])
    m = geosgs.mean(geosgs.GaussianProcess(f, [1.0, -2.0, 0.5]), geosgs.CartesianGrid((4, 3)))
    assert list(m) == ["field1", "field2", "field3"] and m["field2"][5] == -2.0
    grid = geosgs.CartesianGrid((10, 10))
    with pytest.raises(geosgs.ArgumentError):  # one data column per variable
        geosgs.build_problem(proc, grid, geosgs.georef({"a": [1.0]}, [[2.0, 3.0]]), geosgs.GPUSEQSIM())


@pytest.mark.parametrize("nested", [False, True])
def test_oracle_one_variable_is_univariate_seqsim(oracle_mod, nested):
    wl = workloads.small(n=24, k=12, ndata=20, vario="exp", nugget=0.1, seed=3)
    proc = wl.process
    if nested:
        proc = geosgs.GaussianProcess(geosgs.NestedVariogram([
            geosgs.SphericalVariogram(range=4.0, sill=0.6, nugget=0.05),
            geosgs.GaussianVariogram(range=9.0, sill=0.5)]), 0.3)
    p, keep = geosgs.build_problem(proc, wl.domain, wl.data, wl.method)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    R, N = 5, wl.domain.nelements()
    z = np.random.default_rng(1).standard_normal((R, N))
    uni = O.simulate(R, z)
    S = len(proc.func.structures())
    dv = wl.data.values["Z"].reshape(-1, 1)
    mv = O.simulate_multivariate(R, [proc.mean], np.ones((S, 1, 1)), dv, z=z.reshape(R, 1, N))
    assert rel_err(mv[:, 0, :], uni) <= 1e-10


def test_oracle_diagonal_model_is_independent_univariate_runs(oracle_mod):
    d = np.array([1.5, 0.4, 0.9])
    nug = 0.05
    sph = geosgs.SphericalVariogram(range=7.0, nugget=nug)
    proc = geosgs.GaussianProcess(geosgs.LinearCoregionalization([(np.diag(d), sph)]), [0.5, -1.0, 2.0])
    grid = geosgs.CartesianGrid((22, 20))
    rng = np.random.default_rng(4)
    data = mv_data(rng, 18, grid.dims, 3)
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(6), maxneighbors=12)
    R, N = 4, grid.nelements()
    z = rng.standard_normal((R, 3, N))
    _, mv = oracle_mv(oracle_mod, proc, grid, data, method, R, z=z)
    for a in range(3):
        pa = geosgs.GaussianProcess(geosgs.SphericalVariogram(range=7.0, sill=d[a], nugget=d[a] * nug), proc.mean[a])
        da = geosgs.georef({"Z": data.values[f"V{a}"]}, data.coords)
        p, keep = geosgs.build_problem(pa, grid, da, method)
        O = oracle_mod.OraclePlan(p, keep).prepare()
        assert rel_err(mv[:, a, :], O.simulate(R, z[:, a, :])) <= 1e-10, a


def numpy_multivariate(proc, grid, data, path, nbr, cnt, nmin, z):
    """An independent restatement of the multivariate loop for small cases:
    per node in path order, the (nL x nL) cokriging system from the model's
    own variogram functions, numpy.linalg.solve, the conditional covariance
    C(0) - c' Lambda and numpy's Cholesky factor."""
    dim, L = grid.dim, proc.nvariables
    st, A = proc.func.structures(), proc.func.coef
    X = grid.centroids() if data is None else np.vstack([grid.centroids(), data.coords])
    N = grid.nelements()

    def cov(h):  # lags (m x dim) -> m x L x L
        out = np.zeros((h.shape[0], L, L))
        for s, g in enumerate(st):
            out += (g.sill - g.gamma_at(h, dim))[:, None, None] * A[s][None]
        return out

    mean = np.asarray(proc.mean)
    C0 = cov(np.zeros((1, dim)))[0]
    vals = np.full((X.shape[0], L), np.nan)
    if data is not None:
        vals[N:] = gproblem.multivariate_data(proc, data)
    for g in path:
        n = cnt[g]
        mu, S = mean.copy(), C0.copy()
        if n >= nmin:
            P = X[nbr[g, :n]]
            K = cov((P[:, None, :] - P[None, :, :]).reshape(-1, dim)).reshape(n, n, L, L)
            K = K.transpose(0, 2, 1, 3).reshape(n * L, n * L)
            c = cov(P - X[g]).reshape(n * L, L)
            lam = np.linalg.solve(K, c)
            mu = mean + lam.T @ (vals[nbr[g, :n]].reshape(-1) - np.tile(mean, n))
            S = C0 - c.T @ lam
        vals[g] = mu + np.linalg.cholesky(S) @ z[:, g]
    return vals[:N].T


def test_oracle_matches_an_independent_numpy_restatement(oracle_mod):
    """Cross-covariances, nested structures of different ranges and
    anisotropy, data and prior nodes: the oracle against numpy on the
    oracle's own neighbour sets (the search is pinned elsewhere)."""
    grid = geosgs.CartesianGrid((16, 14))
    rng = np.random.default_rng(21)
    data = mv_data(rng, 10, grid.dims, 2)
    proc = geosgs.GaussianProcess(lmc(2, nugget=0.05), [0.3, -0.6])
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(5), maxneighbors=8, minneighbors=3,
                              neighborhood=geosgs.MetricBall(3.0))
    z = rng.standard_normal((1, 2, grid.nelements()))
    O, out = oracle_mv(oracle_mod, proc, grid, data, method, 1, z=z)
    nbr, cnt = O.neighbors()
    assert np.any(cnt < 3) and np.any(cnt == 8)  # prior nodes and full systems
    path = geosgs.RandomPath(5).permutation(grid.nelements())
    want = numpy_multivariate(proc, grid, data, path, nbr, cnt, 3, z[0])
    assert rel_err(out[0], want) <= 1e-9


def test_oracle_datum_reproduction_and_prior_covariance(oracle_mod):
    grid = geosgs.CartesianGrid((30, 30))
    proc = geosgs.GaussianProcess(lmc(2), [1.0, -1.0])
    cell = grid.linear_index(12, 17)
    xyz = np.vstack([grid.centroids()[cell], [[3.3, 4.4], [25.1, 7.9]]])
    data = geosgs.georef({"a": [2.5, 0.1, -0.3], "b": [-0.7, 0.4, 1.2]}, xyz)
    order = np.concatenate([[cell], np.setdiff1d(np.arange(grid.nelements()), [cell])])
    method = geosgs.GPUSEQSIM(path=geosgs.ExplicitPath(order), maxneighbors=16)
    _, out = oracle_mv(oracle_mod, proc, grid, data, method, 6, seed=3)
    np.testing.assert_allclose(out[:, 0, cell], 2.5, rtol=0, atol=1e-9)
    np.testing.assert_allclose(out[:, 1, cell], -0.7, rtol=0, atol=1e-9)
    # no neighbour inside a tiny ball: every node draws from MvNormal(mean, C(0))
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(2), maxneighbors=16, neighborhood=geosgs.MetricBall(0.1))
    _, out = oracle_mv(oracle_mod, proc, grid, None, method, 20, seed=9)
    x = out.transpose(1, 0, 2).reshape(2, -1)
    C0 = sum(A * g.sill for A, g in zip(proc.func.coef, proc.func.structures()))
    n = x.shape[1]
    np.testing.assert_allclose(x.mean(axis=1), [1.0, -1.0], atol=5 * np.sqrt(np.diag(C0) / n).max())
    np.testing.assert_allclose(np.cov(x), C0, atol=5 * np.sqrt(2.0 / n) * C0.max())


# ------------------------------------------------------------------ the GPU
CASES = [
    (2, 2, 30, 6, 0.0),
    (2, 3, 26, 12, 0.05),
    (3, 2, 14, 0, 0.0),
    (3, 3, 12, 16, 0.02),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(CASES)))
def test_gpu_multivariate_matches_oracle(case, oracle_mod, geosgs_lib):
    dim, L, n, ndata, nug = CASES[case]
    rng = np.random.default_rng(40 + case)
    grid = geosgs.CartesianGrid((n, n) if dim == 2 else (n, n, 6))
    data = mv_data(rng, ndata, grid.dims, L) if ndata else None
    proc = geosgs.GaussianProcess(lmc(L, nug), rng.standard_normal(L))
    k = 64 // L if case == 1 else 10
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(case), maxneighbors=k)
    p, keep = geosgs.build_problem(proc, grid, data, method)
    G = geosgs.Plan(p, keep).set_multivariate(proc.mean, proc.func.coef, gproblem.multivariate_data(proc, data))
    G.prepare()
    R = 6
    z = rng.standard_normal((R, L, G.N))
    got = G.simulate_multivariate(R, z=z)
    O, want = oracle_mv(oracle_mod, proc, grid, data, method, R, z=z)
    np.testing.assert_array_equal(G.weights()[2], O.weights()[2])  # node status
    assert rel_err(got, want) <= VALUE_TOL, rel_err(got, want)
    # seeded normals: Philox counters of pseudo-node a*N + g, FP32 Box-Muller
    got = G.simulate_multivariate(R, seed=17)
    _, want = oracle_mv(oracle_mod, proc, grid, data, method, R, seed=17)
    assert rel_err(got, want) <= 2e-5
    G.close()


@pytest.mark.gpu
def test_gpu_one_variable_equals_the_univariate_plan(geosgs_lib):
    """The cokriging form with one variable against the plan's own FP64
    solve and sweep on the same problem and normals."""
    wl = workloads.small(n=28, k=14, ndata=25, vario="sph", nugget=0.05, seed=8, precision="fp64")
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = geosgs.Plan(p, keep).prepare()
    R = 5
    z = np.random.default_rng(2).standard_normal((R, G.N))
    uni = G.simulate(R, z)
    G.set_multivariate([wl.process.mean], np.ones((1, 1, 1)), wl.data.values["Z"].reshape(-1, 1)).prepare()
    mv = G.simulate_multivariate(R, z=z.reshape(R, 1, G.N))
    assert rel_err(mv[:, 0, :], uni) <= 1e-9
    G.close()


@pytest.mark.gpu
def test_rand_multivariate_api(oracle_mod, geosgs_lib):
    grid = geosgs.CartesianGrid((24, 20))
    rng = np.random.default_rng(12)
    data = geosgs.georef({"cu": rng.standard_normal(10), "au": rng.standard_normal(10)},
                         rng.uniform(0, 1, (10, 2)) * [24, 20])
    proc = geosgs.GaussianProcess(lmc(2), [0.2, -0.4])
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(3), maxneighbors=12)
    z = rng.standard_normal((3, 2, grid.nelements()))
    ens = geosgs.rand(np.random.default_rng(0), proc, grid, 3, data=data, method=method, z=z)
    assert list(ens[0]) == ["cu", "au"]
    _, want = oracle_mv(oracle_mod, proc, grid, data, method, 3, z=z)
    for r in range(3):
        assert rel_err(np.stack([ens[r]["cu"], ens[r]["au"]]), want[r]) <= VALUE_TOL
    real = geosgs.rand(np.random.default_rng(1), proc, grid, method=method)
    assert list(real) == ["field1", "field2"] and real["field1"].shape == (grid.nelements(),)
    # per-realization paths: realization r on the r-th permutation
    pm = geosgs.GPUSEQSIM(path=geosgs.RandomPath(3), maxneighbors=12, path_per_realization=True)
    ens = geosgs.rand(np.random.default_rng(0), proc, grid, 2, data=data, method=pm, z=z[:2])
    perms = geosgs.RandomPath(3).permutations(grid.nelements(), 2)
    for r in range(2):
        m = geosgs.GPUSEQSIM(path=geosgs.ExplicitPath(perms[r]), maxneighbors=12)
        _, want = oracle_mv(oracle_mod, proc, grid, data, m, 1, z=z[r:r + 1])
        assert rel_err(np.stack([ens[r]["cu"], ens[r]["au"]]), want[0]) <= VALUE_TOL

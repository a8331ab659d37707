"""Sequential indicator simulation (IndicatorProcess + SEQSIM,
src/simulation/field/seqsim.jl:247-347; sgs_plan_set_indicator /
sgs_plan_simulate_indicator).

The oracle's restatement is pinned on the CPU by the reference's own test
shapes (test/field.jl:181-204: two categories without data give the set
{1, 2}, data labelled [1, 3, 1] give {1, 3}, three proportions give
{1, 2, 3}, string labels come back as strings), by exact data reproduction
(a node on a datum takes its category in every realization, nugget 0), and
by the prior's proportions where no neighbour is found; its full simple
cokriging form by its reduction to the separable path and by an independent
numpy restatement on a non-separable model.  The GPU is then compared with
the oracle fed the same uniforms: categories identical."""
import numpy as np
import pytest

import geosgs
from geosgs import problem as gproblem
from geosgs import workloads


def oracle_cats(oracle_mod, proc, grid, data, method, nreals, u=None, seed=0):
    p, keep = geosgs.build_problem(proc, grid, data, method)
    levels, dcat = gproblem.indicator_levels(proc, data)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    cats = O.simulate_indicator(nreals, proc.prob, dcat, u=u, seed=seed)
    return np.asarray(levels, dtype=object)[cats], cats


def test_reference_indicator_shapes(oracle_mod):
    grid = geosgs.CartesianGrid((100, 100))
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(123), maxneighbors=26)
    proc = geosgs.IndicatorProcess(geosgs.SphericalTransiogram(range=35.0))
    real, _ = oracle_cats(oracle_mod, proc, grid, None, method, 1)
    assert set(real[0].tolist()) == {1, 2}
    data = geosgs.georef({"C": np.array([1, 3, 1])}, np.array([[25.0, 25.0], [50.0, 75.0], [75.0, 50.0]]))
    real, _ = oracle_cats(oracle_mod, proc, grid, data, method, 1)
    assert set(real[0].tolist()) == {1, 3}
    proc3 = geosgs.IndicatorProcess(geosgs.SphericalTransiogram(range=35.0, proportions=(0.7, 0.2, 0.1)))
    real, _ = oracle_cats(oracle_mod, proc3, grid, None, method, 1)
    assert set(real[0].tolist()) == {1, 2, 3}
    data = geosgs.georef({"C": np.array(["a", "b", "c"])}, np.array([[25.0, 25.0], [50.0, 75.0], [75.0, 50.0]]))
    real, _ = oracle_cats(oracle_mod, proc3, grid, data, method, 1)
    assert set(real[0].tolist()) == {"a", "b", "c"}


def test_oracle_indicator_data_reproduction_and_prior(oracle_mod):
    grid = geosgs.CartesianGrid((30, 30))
    X = grid.centroids()
    cells = [31, 250, 777]
    data = geosgs.georef({"C": np.array([2, 0, 1])}, X[cells])
    proc = geosgs.IndicatorProcess(geosgs.SphericalVariogram(range=8.0), prob=(0.5, 0.3, 0.2))
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(3), maxneighbors=12)
    _, cats = oracle_cats(oracle_mod, proc, grid, data, method, 16, seed=5)
    np.testing.assert_array_equal(cats[:, cells], np.tile([2, 0, 1], (16, 1)))
    # no neighbour inside a tiny ball: every node draws from the prior
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(3), maxneighbors=12, neighborhood=geosgs.MetricBall(0.1))
    _, cats = oracle_cats(oracle_mod, proc, grid, None, method, 40, seed=6)
    frac = np.bincount(cats.ravel(), minlength=3) / cats.size
    n = cats.size
    for f, p in zip(frac, (0.5, 0.3, 0.2)):
        assert abs(f - p) < 5 * np.sqrt(p * (1 - p) / n)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_gpu_indicator_matches_oracle(precision, oracle_mod, geosgs_lib):
    cases = [
        (workloads.small(dim=2, n=40, k=16, ndata=30, vario="sph", seed=1), (0.5, 0.3, 0.2)),
        (workloads.small(dim=3, n=20, k=24, ndata=40, vario="exp", nugget=0.05, seed=2, ranges=(8.0, 5.0, 3.0),
                         rotation=geosgs.RotZ(30.0)), (0.4, 0.6)),
        (workloads.small(dim=2, n=32, k=8, ndata=0, vario="gau", seed=3), (0.25, 0.25, 0.25, 0.125, 0.125)),
    ]
    R = 12
    for wl, prob in cases:
        rng = np.random.default_rng(7)
        data = None
        if wl.data is not None:
            labels = rng.integers(0, len(prob), wl.data.nrow())
            labels[: len(prob)] = np.arange(len(prob))  # every category present in the data
            data = geosgs.georef({"C": labels}, wl.data.coords)
        proc = geosgs.IndicatorProcess(wl.process.func, prob=prob)
        method = geosgs.GPUSEQSIM(path=wl.method.path, maxneighbors=wl.method.maxneighbors, precision=precision)
        p, keep = geosgs.build_problem(proc, wl.domain, data, method)
        levels, dcat = gproblem.indicator_levels(proc, data)
        G = geosgs.Plan(p, keep).set_indicator(proc.prob, dcat).prepare()
        u = rng.uniform(0.0, 1.0, (R, G.N))
        got = G.simulate_indicator(R, u=u)
        O = oracle_mod.OraclePlan(p, keep).prepare()
        np.testing.assert_array_equal(got, O.simulate_indicator(R, proc.prob, dcat, u=u))
        # seeded uniforms: the oracle's Philox restatement gives the same draws
        got = G.simulate_indicator(R, seed=99)
        np.testing.assert_array_equal(got, O.simulate_indicator(R, proc.prob, dcat, seed=99))
        G.close()


@pytest.mark.gpu
def test_rand_indicator_api(geosgs_lib):
    grid = geosgs.CartesianGrid((100, 100))
    rng = np.random.default_rng(123)
    proc = geosgs.IndicatorProcess(geosgs.SphericalTransiogram(range=35.0))
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(1), maxneighbors=26)
    real = geosgs.rand(rng, proc, grid, method=method)
    assert set(real["field"].tolist()) == {1, 2}
    data = geosgs.georef({"C": np.array(["a", "b", "c"])}, np.array([[25.0, 25.0], [50.0, 75.0], [75.0, 50.0]]))
    proc3 = geosgs.IndicatorProcess(geosgs.SphericalTransiogram(range=35.0, proportions=(0.7, 0.2, 0.1)))
    ens = geosgs.rand(rng, proc3, grid, 3, data=data, method=method)
    assert len(ens) == 3 and set(ens[0]["C"].tolist()) == {"a", "b", "c"}


@pytest.mark.gpu
def test_default_method_with_data_grows_from_the_data(oracle_mod, geosgs_lib):
    """With data and no method, `rand` simulates an IndicatorProcess along the
    reference's SourcePath (src/simulation/field.jl:168-180): the GPU follows
    that path with categories identical to the oracle's on the same uniforms.
    The path's first node sits on the first datum and has only data as
    neighbours, so it takes that datum's category in every realization
    (nugget 0).  Later data nodes need not: a system holding a datum and the
    simulated node on the same centre is singular, and the node draws from
    the prior as the reference's failed fit does."""
    grid = geosgs.CartesianGrid((48, 40))
    rng = np.random.default_rng(11)
    cells = rng.choice(grid.nelements(), size=25, replace=False)
    xyz = grid.centroids()[cells]
    labels = rng.integers(0, 3, cells.size)
    labels[:3] = [0, 1, 2]
    data = geosgs.georef({"C": labels}, xyz)
    proc = geosgs.IndicatorProcess(geosgs.SphericalTransiogram(range=9.0, proportions=(0.5, 0.3, 0.2)))
    method = geosgs.defaultsimulation(proc, grid, data=data)
    np.testing.assert_array_equal(method.path.sources, cells)
    p, keep = geosgs.build_problem(proc, grid, data, method)
    levels, dcat = gproblem.indicator_levels(proc, data)
    G = geosgs.Plan(p, keep).set_indicator(proc.prob, dcat).prepare()
    u = rng.uniform(0.0, 1.0, (8, G.N))
    got = G.simulate_indicator(8, u=u)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    np.testing.assert_array_equal(got, O.simulate_indicator(8, proc.prob, dcat, u=u))
    np.testing.assert_array_equal(got[:, cells[0]], np.full(8, dcat[0]))
    G.close()
    ens = geosgs.rand(np.random.default_rng(2), proc, grid, 2, data=data)
    assert set(ens[0]["C"].tolist()) <= {0, 1, 2}
    assert ens[0]["C"][cells[0]] == labels[0] and ens[1]["C"][cells[0]] == labels[0]


# ---- full simple cokriging: linear models of coregionalization ----
def lmc_model(L=3):
    """A non-separable indicator covariance: a short spherical structure and a
    longer anisotropic exponential one with different coregionalization
    matrices (symmetric positive definite)."""
    A1 = np.array([[0.20, -0.08, -0.05], [-0.08, 0.15, -0.03], [-0.05, -0.03, 0.10]])[:L, :L]
    A2 = np.array([[0.05, -0.02, 0.01], [-0.02, 0.06, -0.01], [0.01, -0.01, 0.04]])[:L, :L]
    return geosgs.LinearCoregionalization([
        (A1, geosgs.SphericalVariogram(range=6.0)),
        (A2, geosgs.ExponentialVariogram(ranges=(14.0, 7.0, 4.0), rotation=geosgs.RotZ(25.0))),
    ])


def test_oracle_cokriging_reduces_to_the_separable_path(oracle_mod):
    """With one structure, C_ab(h) = A_ab C(h) with A nonsingular, simple
    cokriging gives every category the simple kriging weights of C: the
    cokriging restatement draws the same categories as the separable one
    from the same uniforms."""
    grid = geosgs.CartesianGrid((24, 20))
    A = np.array([[1.0, 0.4, 0.1], [0.4, 0.8, 0.2], [0.1, 0.2, 0.6]])
    g = geosgs.ExponentialVariogram(range=7.0)
    prob = (0.5, 0.3, 0.2)
    rng = np.random.default_rng(4)
    data = geosgs.georef({"C": np.array([0, 2, 1, 1])}, rng.uniform(0.0, 1.0, (4, 2)) * [24.0, 20.0])
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(8), maxneighbors=10)
    sep = geosgs.IndicatorProcess(g, prob=prob)
    cok = geosgs.IndicatorProcess(geosgs.LinearCoregionalization([(A, g)]), prob=prob)
    p, keep = geosgs.build_problem(cok, grid, data, method)
    _, dcat = gproblem.indicator_levels(cok, data)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    u = rng.uniform(0.0, 1.0, (6, O.N))
    np.testing.assert_array_equal(O.simulate_cokriging(6, prob, cok.func.coef, dcat, u=u),
                                  O.simulate_indicator(6, sep.prob, dcat, u=u))


def test_oracle_cokriging_matches_an_independent_numpy_restatement(oracle_mod):
    """A non-separable model (two structures, different ranges and
    anisotropy) with data of every category: the oracle's categories against
    numpy on the oracle's neighbour sets — the (nL x nL) system from the
    model's own variogram functions, numpy.linalg.solve,
    p = prob + Lambda' (I - prob) clamped and normalized, the inverse cdf at
    the same uniforms."""
    L, prob = 3, np.array([0.5, 0.3, 0.2])
    grid = geosgs.CartesianGrid((18, 15))
    rng = np.random.default_rng(31)
    labels = rng.integers(0, L, 12)
    labels[:L] = np.arange(L)
    data = geosgs.georef({"C": labels}, rng.uniform(0.0, 1.0, (12, 2)) * [18.0, 15.0])
    proc = geosgs.IndicatorProcess(lmc_model(L), prob=prob)
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(9), maxneighbors=8, minneighbors=2,
                              neighborhood=geosgs.MetricBall(3.0))
    p, keep = geosgs.build_problem(proc, grid, data, method)
    _, dcat = gproblem.indicator_levels(proc, data)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    N = O.N
    u = rng.uniform(0.0, 1.0, (1, N))
    got = O.simulate_cokriging(1, prob, proc.func.coef, dcat, u=u)[0]
    nbr, cnt = O.neighbors()
    assert np.any(cnt < 2) and np.any(cnt == 8)  # prior nodes and full systems
    st, A = proc.func.structures(), proc.func.coef
    X = np.vstack([grid.centroids(), data.coords])

    def cov(h):
        out = np.zeros((h.shape[0], L, L))
        for s, g in enumerate(st):
            out += (g.sill - g.gamma_at(h, 2))[:, None, None] * A[s][None]
        return out

    cat = np.concatenate([np.full(N, -1), dcat])
    for g in geosgs.RandomPath(9).permutation(N):
        n = cnt[g]
        q = prob.copy()
        if n >= 2:
            P = X[nbr[g, :n]]
            K = cov((P[:, None, :] - P[None, :, :]).reshape(-1, 2)).reshape(n, n, L, L)
            lam = np.linalg.solve(K.transpose(0, 2, 1, 3).reshape(n * L, n * L), cov(P - X[g]).reshape(n * L, L))
            onehot = (cat[nbr[g, :n]][:, None] == np.arange(L)[None, :]).astype(float)
            q = prob + lam.T @ (onehot - prob).reshape(-1)
        q = np.clip(q, 0.0, 1.0)
        q = q / q.sum() if q.sum() > 0 else prob
        cat[g] = min(int(np.searchsorted(np.cumsum(q)[:-1], u[0, g], side="right")), L - 1)
    np.testing.assert_array_equal(got, cat[:N])


def test_oracle_cokriging_proportions(oracle_mod):
    """An unconditional simulation with a non-separable model reproduces the
    prior proportions on average over realizations."""
    grid = geosgs.CartesianGrid((40, 40))
    prob = (0.5, 0.3, 0.2)
    proc = geosgs.IndicatorProcess(lmc_model(3), prob=prob)
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(2), maxneighbors=12)
    p, keep = geosgs.build_problem(proc, grid, None, method)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    cats = O.simulate_cokriging(60, prob, proc.func.coef, seed=3)
    frac = np.bincount(cats.ravel(), minlength=3) / cats.size
    assert np.abs(frac - np.array(prob)).max() < 0.04, frac


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_cokriging_matches_oracle(dim, oracle_mod, geosgs_lib):
    """Full simple cokriging with a non-separable model (two structures of
    different ranges and anisotropy, each with its own coregionalization
    matrix), with data of every category: node status identical and the
    categories equal to the oracle's, for given and for seeded uniforms.  A
    one-structure model run through the cokriging path also equals the
    separable path."""
    L = 3
    prob = (0.5, 0.3, 0.2)
    if dim == 2:
        grid = geosgs.CartesianGrid((36, 30))
        k = 12
    else:
        grid = geosgs.CartesianGrid((18, 16, 8))
        k = 16
    rng = np.random.default_rng(20 + dim)
    npts = 40
    xy = rng.uniform(0.0, 1.0, (npts, dim)) * np.asarray(grid.dims, dtype=float)
    labels = rng.integers(0, L, npts)
    labels[:L] = np.arange(L)
    data = geosgs.georef({"C": labels}, xy)
    proc = geosgs.IndicatorProcess(lmc_model(L), prob=prob)
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(4), maxneighbors=k, precision="fp64")
    p, keep = geosgs.build_problem(proc, grid, data, method)
    _, dcat = gproblem.indicator_levels(proc, data)
    G = geosgs.Plan(p, keep).set_indicator_cokriging(proc.prob, proc.func.coef, dcat).prepare()
    O = oracle_mod.OraclePlan(p, keep).prepare()
    R = 8
    u = rng.uniform(0.0, 1.0, (R, G.N))
    got = G.simulate_indicator(R, u=u)
    want = O.simulate_cokriging(R, proc.prob, proc.func.coef, dcat, u=u)
    np.testing.assert_array_equal(G.weights()[2], O.weights()[2])  # cokriging status of every node
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(G.simulate_indicator(R, seed=5),
                                  O.simulate_cokriging(R, proc.prob, proc.func.coef, dcat, seed=5))
    G.close()
    # one structure: the cokriging path equals the separable path
    A = np.array([[1.0, 0.4, 0.1], [0.4, 0.8, 0.2], [0.1, 0.2, 0.6]])
    g1 = geosgs.ExponentialVariogram(range=7.0)
    cok1 = geosgs.IndicatorProcess(geosgs.LinearCoregionalization([(A, g1)]), prob=prob)
    p, keep = geosgs.build_problem(cok1, grid, data, method)
    Gc = geosgs.Plan(p, keep).set_indicator_cokriging(prob, cok1.func.coef, dcat).prepare()
    Gs = geosgs.Plan(p, keep).set_indicator(prob, dcat).prepare()
    np.testing.assert_array_equal(Gc.simulate_indicator(R, u=u), Gs.simulate_indicator(R, u=u))
    Gc.close()
    Gs.close()


@pytest.mark.gpu
def test_rand_cokriging_api(geosgs_lib):
    """rand with an IndicatorProcess on a linear model of coregionalization
    runs the cokriging path and returns the data's labels."""
    grid = geosgs.CartesianGrid((40, 40))
    data = geosgs.georef({"C": np.array(["a", "b", "c"])}, np.array([[5.5, 5.5], [20.5, 30.5], [30.5, 10.5]]))
    proc = geosgs.IndicatorProcess(lmc_model(3), prob=(0.5, 0.3, 0.2))
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(2), maxneighbors=12)
    ens = geosgs.rand(np.random.default_rng(1), proc, grid, 2, data=data, method=method)
    assert len(ens) == 2 and set(ens[0]["C"].tolist()) <= {"a", "b", "c"}

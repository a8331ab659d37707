"""Sequential indicator simulation (IndicatorProcess + SEQSIM,
src/simulation/field/seqsim.jl:247-347; sgs_plan_set_indicator /
sgs_plan_simulate_indicator).

The oracle's restatement is pinned on the CPU by the reference's own test
shapes (test/field.jl:181-204: two categories without data give the set
{1, 2}, data labelled [1, 3, 1] give {1, 3}, three proportions give
{1, 2, 3}, string labels come back as strings), by exact data reproduction
(a node on a datum takes its category in every realization, nugget 0), and
by the prior's proportions where no neighbour is found.  The GPU is then
compared with the oracle fed the same uniforms: categories identical."""
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

"""The FP64 CPU oracle against the reference's known answers, closed-form
kriging systems and the golden fixtures of an independent numpy
restatement (tests/golden/make_golden.py)."""
import math

import numpy as np
import pytest

import geosgs
from conftest import golden_cases, golden_problem, load_golden
from geosgs import workloads


def oracle_of(wl, oracle_mod, method=1):
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    O = oracle_mod.OraclePlan(p, keep)
    O.search(method)
    O.solve()
    return O


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_golden(name, oracle_mod):
    g = load_golden(name)
    p, keep = golden_problem(g)
    for method in (oracle_mod.BRUTE, oracle_mod.TEMPLATE):
        O = oracle_mod.OraclePlan(p, keep)
        O.search(method)
        O.solve()
        idx, cnt = O.neighbors()
        np.testing.assert_array_equal(cnt, g["cnt"])
        np.testing.assert_array_equal(idx, g["nbr"])
        w, s, st = O.weights()
        np.testing.assert_array_equal(st, g["status"])
        np.testing.assert_allclose(w, g["w"], rtol=0, atol=1e-10)
        # sigma^2 = sill - w'c cancels to ~1e-16 at data locations, so the
        # standard deviations are compared through the variance
        np.testing.assert_allclose(s**2, g["sigma"] ** 2, rtol=0, atol=1e-12)
        out = O.simulate(g["z"].shape[0], g["z"])
        np.testing.assert_allclose(out, g["out"], rtol=0, atol=1e-7)


def test_reference_datum_reproduction(oracle_mod):
    """test/field.jl:79-86: a conditional SEQSIM realization reproduces the
    datum at cell (25,25) within 1e-4 (maxneighbors=3, spherical range 35,
    grid (0.5,0.5)-(100.5,100.5), default LinearPath and :range ball)."""
    grid = geosgs.CartesianGrid((0.5, 0.5), (100.5, 100.5), dims=(100, 100))
    data = geosgs.georef({"Z": [1.0, 0.0, 1.0]}, [(25.0, 25.0), (50.0, 75.0), (75.0, 50.0)])
    proc = geosgs.GaussianProcess(geosgs.SphericalVariogram(range=35.0))
    method = geosgs.GPUSEQSIM(maxneighbors=3)
    p, keep = geosgs.build_problem(proc, grid, data, method)
    O = oracle_mod.OraclePlan(p, keep)
    O.prepare()
    z = np.random.default_rng(2017).standard_normal((1, grid.nelements()))
    out = O.simulate(1, z)
    # inds = LinearIndices(size(grid)); inds[25, 25] (1-based) -> node 24 + 100*24
    g = grid.linear_index(24, 24)
    assert abs(out[0, g] - 1.0) <= 1e-4
    # all three data reproduced
    assert abs(out[0, grid.linear_index(49, 74)] - 0.0) <= 1e-4
    assert abs(out[0, grid.linear_index(74, 49)] - 1.0) <= 1e-4


def test_explicit_init_layout(oracle_mod):
    """Data are appended after the grid nodes (seqsim.jl:211-218, 267-271;
    test/initialization.jl:31-59 pins ExplicitInit's destination indices):
    datum i is augmented point N+i, and it is the nearest neighbour of the
    grid node it sits on."""
    grid = geosgs.CartesianGrid((6, 5))
    xy = np.array([[0.5, 0.5], [5.5, 4.5], [2.5, 1.5]])
    data = geosgs.georef({"Z": [3.0, -1.0, 0.5]}, xy)
    proc = geosgs.GaussianProcess(geosgs.ExponentialVariogram(range=3.0))
    method = geosgs.GPUSEQSIM(maxneighbors=4, path=geosgs.RandomPath(5))
    p, keep = geosgs.build_problem(proc, grid, data, method)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    idx, cnt = O.neighbors()
    N = grid.nelements()
    for i, (x, y) in enumerate(xy):
        g = grid.linear_index(int(x), int(y))
        assert idx[g, 0] == N + i
    w, s, st = O.weights()
    z = np.random.default_rng(0).standard_normal((2, N))
    out = O.simulate(2, z)
    for i, (x, y) in enumerate(xy):
        g = grid.linear_index(int(x), int(y))
        assert st[g] == 0 and s[g] < 1e-7
        np.testing.assert_allclose(out[:, g], data.values["Z"][i], atol=1e-7)


def _single_system(oracle_mod, vario, data_xy, data_val, node_xy, k):
    """Oracle weights of the first path node (only data as neighbours)."""
    grid = geosgs.CartesianGrid((20, 20))
    data = geosgs.georef({"Z": data_val}, np.asarray(data_xy, dtype=float))
    proc = geosgs.GaussianProcess(vario, 0.0)
    g = grid.linear_index(*node_xy)
    perm = np.arange(grid.nelements())
    perm[[0, g]] = perm[[g, 0]]
    method = geosgs.GPUSEQSIM(maxneighbors=k, path=geosgs.ExplicitPath(perm), neighborhood=geosgs.MetricBall(50.0))
    p, keep = geosgs.build_problem(proc, grid, data, method)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    idx, cnt = O.neighbors()
    w, s, st = O.weights()
    return g, idx[g, : cnt[g]], w[g, : cnt[g]], s[g], st[g]


def test_one_neighbour_closed_form(oracle_mod):
    # node (10,10) centre (10.5,10.5); datum at distance 3 along x
    v = geosgs.SphericalVariogram(range=10.0, sill=2.0, nugget=0.2)
    g, idx, w, s, st = _single_system(oracle_mod, v, [[13.5, 10.5]], [1.0], (10, 10), 1)
    h = 0.3
    C0 = 2.0
    Ch = 2.0 - (0.2 + 1.8 * (1.5 * h - 0.5 * h**3))
    assert st == 0
    np.testing.assert_allclose(w, [Ch / C0], rtol=1e-14)
    np.testing.assert_allclose(s, math.sqrt(C0 - Ch * Ch / C0), rtol=1e-13)


def test_two_neighbour_closed_form(oracle_mod):
    v = geosgs.ExponentialVariogram(range=8.0, sill=1.0, nugget=0.0)
    xy = [[12.5, 10.5], [10.5, 14.5]]  # distances 2 and 4 from (10.5,10.5)
    g, idx, w, s, st = _single_system(oracle_mod, v, xy, [0.3, -0.7], (10, 10), 2)
    c = lambda h: math.exp(-3.0 * h / 8.0)
    d12 = math.hypot(2.0, 4.0)
    K = np.array([[1.0, c(d12)], [c(d12), 1.0]])
    rhs = np.array([c(2.0), c(4.0)])
    w_ref = np.linalg.solve(K, rhs)
    assert list(idx) == [400, 401]
    np.testing.assert_allclose(w, w_ref, rtol=1e-13)
    np.testing.assert_allclose(s, math.sqrt(1.0 - w_ref @ rhs), rtol=1e-12)


def test_duplicate_location_is_singular(oracle_mod):
    """Two neighbours at one location give identical LHS rows: the
    factorization fails and the node takes the prior (seqsim.jl:127-131)."""
    v = geosgs.GaussianVariogram(range=10.0, nugget=0.01)
    g, idx, w, s, st = _single_system(oracle_mod, v, [[12.5, 10.5], [12.5, 10.5]], [1.0, 1.0], (10, 10), 2)
    assert st == 2 and s == 1.0 and np.all(w == 0)


def test_first_node_prior_draw(oracle_mod):
    """Unconditional: the first node has no neighbours -> prior N(mu, sill)."""
    wl = workloads.small(n=12, k=6)
    wl.process.mean = 1.5
    wl.process.func.sill = 4.0
    O = oracle_of(wl, oracle_mod)
    w, s, st = O.weights()
    first = wl.method.path.permutation(wl.domain.nelements())[0]
    assert st[first] == 1 and s[first] == 2.0
    z = np.random.default_rng(1).standard_normal((2, O.N))
    out = O.simulate(2, z)
    np.testing.assert_allclose(out[:, first], 1.5 + 2.0 * z[:, first], rtol=1e-15)


def test_neighbour_clamps(oracle_mod):
    """seqsim.jl:202-208: nmax > N or < 1 -> N; nmin > nmax or < 1 -> 1."""
    assert geosgs.clamped_neighbors(geosgs.GPUSEQSIM(maxneighbors=500, minneighbors=3), 100) == (3, 100)
    assert geosgs.clamped_neighbors(geosgs.GPUSEQSIM(maxneighbors=0, minneighbors=0), 100) == (1, 100)
    assert geosgs.clamped_neighbors(geosgs.GPUSEQSIM(maxneighbors=5, minneighbors=9), 100) == (1, 5)


@pytest.mark.parametrize("case", ["2d_data", "3d_aniso", "nearest", "spacing"])
def test_template_search_equals_brute_force(case, oracle_mod):
    if case == "2d_data":
        wl = workloads.small(n=40, k=16, ndata=60, vario="gau", ranges=(9.0, 9.0))
    elif case == "3d_aniso":
        wl = workloads.small(dim=3, n=20, nz=8, k=20, ndata=30, vario="exp", ranges=(9.0, 5.0, 3.0),
                             rotation=geosgs.RotZ(30.0),
                             ball=geosgs.MetricBall((9.0, 5.0, 3.0), geosgs.RotZ(30.0)))
    elif case == "nearest":
        wl = workloads.small(n=15, k=7, ndata=5)
        wl.method.neighborhood = None
    else:
        wl = workloads.small(n=18, k=9, ndata=12)
        wl.domain.spacing = (0.7, 1.3)
        wl.domain.origin = (-3.0, 2.0)
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    A = oracle_mod.OraclePlan(p, keep)
    A.search(oracle_mod.BRUTE)
    B = oracle_mod.OraclePlan(p, keep)
    B.search(oracle_mod.TEMPLATE)
    ia, ca = A.neighbors()
    ib, cb = B.neighbors()
    np.testing.assert_array_equal(ca, cb)
    np.testing.assert_array_equal(ia, ib)


def test_levels_are_a_valid_schedule(oracle_mod):
    O = oracle_of(workloads.small(n=30, k=10, ndata=20), oracle_mod)
    lv, nl = O.levels()
    idx, cnt = O.neighbors()
    N = O.N
    for g in range(N):
        nb = idx[g, : cnt[g]]
        nb = nb[nb < N]
        if len(nb):
            assert lv[g] == lv[nb].max() + 1
        else:
            assert lv[g] == 0
    assert nl == lv.max() + 1


def test_unconditional_statistics(oracle_mod):
    """Many realizations reproduce the prior mean and variance (sill)."""
    wl = workloads.small(n=24, k=12, ranges=(4.0, 4.0))
    O = oracle_of(wl, oracle_mod)
    out = O.simulate(400, seed=11)
    assert abs(out.mean()) < 0.06
    assert abs(out.var() - 1.0) < 0.08


def test_seeded_normals_are_standard(oracle_mod):
    z = oracle_mod.normals(123, 5000, 8)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1.0) < 0.02
    z2 = oracle_mod.normals(123, 5000, 8)
    np.testing.assert_array_equal(z, z2)


def _nested_case(precision="fp64", dim=2):
    """A nested model (three structures with their own ranges, rotations,
    sills and nuggets) on a small grid with data."""
    if dim == 2:
        grid = geosgs.CartesianGrid((14, 12))
        rng = np.random.default_rng(41)
        xy = rng.uniform(0.0, 1.0, (12, 2)) * np.array([14.0, 12.0])
    else:
        grid = geosgs.CartesianGrid((10, 9, 6))
        rng = np.random.default_rng(42)
        xy = rng.uniform(0.0, 1.0, (15, 3)) * np.array([10.0, 9.0, 6.0])
    func = (geosgs.SphericalVariogram(ranges=(7.0, 3.0, 2.0), rotation=geosgs.RotZ(35.0), sill=0.5, nugget=0.03)
            + geosgs.ExponentialVariogram(range=9.0, sill=0.3)
            + geosgs.GaussianVariogram(ranges=(4.0, 6.0, 3.0), rotation=geosgs.RotZ(-20.0), sill=0.2, nugget=0.01))
    data = geosgs.georef({"Z": rng.standard_normal(len(xy))}, xy)
    proc = geosgs.GaussianProcess(func, 0.25)
    method = geosgs.GPUSEQSIM(path=geosgs.RandomPath(3), maxneighbors=10, precision=precision)
    return proc, grid, data, method


@pytest.mark.parametrize("dim", [2, 3])
def test_nested_variogram_weights_against_numpy(dim, oracle_mod):
    """The oracle's kriging weights and variances for a nested model equal a
    numpy solve whose covariances are the structures' summed, C(h) = sill -
    sum_s gamma_s(h) (model.NestedVariogram.gamma_at), on the oracle's own
    neighbours."""
    proc, grid, data, method = _nested_case("fp64", dim)
    func = proc.func
    assert len(func.structures()) == 3 and abs(func.sill - 1.0) < 1e-15 and abs(func.nugget - 0.04) < 1e-15
    p, keep = geosgs.build_problem(proc, grid, data, method)
    O = oracle_mod.OraclePlan(p, keep).prepare()
    idx, cnt = O.neighbors()
    w, s, st = O.weights()
    pts = np.concatenate([grid.centroids(), data.coords])
    checked = 0
    for g in range(O.N):
        n = cnt[g]
        if st[g] != 0 or n < 2:
            continue
        x = pts[idx[g, :n]]
        lag = (x[:, None, :] - x[None, :, :]).reshape(-1, dim)
        K = func.sill - func.gamma_at(lag, dim).reshape(n, n)
        K[np.all(lag.reshape(n, n, dim) == 0, axis=2)] = func.sill
        c = func.sill - func.gamma_at(x - pts[g], dim)
        wn = np.linalg.solve(K, c)
        np.testing.assert_allclose(w[g, :n], wn, rtol=0, atol=1e-10)
        assert abs(s[g] - np.sqrt(max(func.sill - wn @ c, 0.0))) < 1e-10
        checked += 1
    assert checked > O.N // 2


def test_nested_range_sets_the_search_radius(oracle_mod):
    """`:range` takes the largest range of any structure (GeoStatsFunctions'
    range of a nested model): the template is that of the longer structure."""
    grid = geosgs.CartesianGrid((40, 40))
    short = geosgs.SphericalVariogram(range=4.0, sill=0.5)
    long = geosgs.ExponentialVariogram(range=11.0, sill=0.5)
    m = geosgs.GPUSEQSIM(path=geosgs.RandomPath(1), maxneighbors=8)
    sizes = []
    for f in (short + long, long, short):
        p, keep = geosgs.build_problem(geosgs.GaussianProcess(f), grid, None, m)
        sizes.append(oracle_mod.OraclePlan(p, keep).template_size())
    assert sizes[0] == sizes[1] > sizes[2]

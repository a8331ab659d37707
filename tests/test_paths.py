"""Visiting orders (Meshes' paths, traversed at seqsim.jl:98) and the
method `rand` picks when none is given (src/simulation/field.jl:152-180).

The reference builds `SEQSIM(; path=SourcePath(unique(inds)))` for an
IndicatorProcess with data, `inds` being the grid node nearest to each datum
(field.jl:168-180).  SourcePath's order is restated from Meshes 0.57, which
the reference does not vendor: sources first, then the other nodes by their
sorted distances to all the sources, compared lexicographically, with node id
settling what stays tied.  The lazy restatement in geosgs is checked here
against a brute-force evaluation of that rule, including lattices whose
symmetry leaves ties beyond the first columns it computes."""
import numpy as np
import pytest

import geosgs
from geosgs import _abi


def brute_source_order(grid, sources):
    """The rule evaluated directly: every other node's full sorted vector of
    distances to all sources, one lexicographic sort, node id last."""
    xyz = grid.centroids()
    n = grid.nelements()
    src = np.asarray(sources, dtype=np.int64)
    others = np.setdiff1d(np.arange(n), src)
    diff = xyz[others][:, None, :] - xyz[src][None, :, :]
    s = diff[..., 0] * diff[..., 0]
    for a in range(1, xyz.shape[1]):
        s = s + diff[..., a] * diff[..., a]
    d = np.sort(np.sqrt(s), axis=1)
    keys = [others] + [d[:, j] for j in reversed(range(d.shape[1]))]
    return np.concatenate([src, others[np.lexsort(tuple(keys))]])


def test_source_path_hand_cases():
    g = geosgs.CartesianGrid((10,))
    # nodes 3 and 6 are one cell from a source and four from the other:
    # tied vectors (1, 4), node id decides; then (1, 6), (2, 3), (2, 7)
    np.testing.assert_array_equal(geosgs.traverse(g, geosgs.SourcePath([2, 7])), [2, 7, 3, 6, 1, 8, 4, 5, 0, 9])
    np.testing.assert_array_equal(geosgs.traverse(geosgs.CartesianGrid((7,)), geosgs.SourcePath([3])),
                                  [3, 2, 4, 1, 5, 0, 6])
    # sources keep their given order; a path of only sources is the sources
    np.testing.assert_array_equal(geosgs.traverse(geosgs.CartesianGrid((3,)), geosgs.SourcePath([2, 0, 1])), [2, 0, 1])


@pytest.mark.parametrize("case", range(8))
def test_source_path_matches_the_brute_force_rule(case):
    rng = np.random.default_rng(100 + case)
    if case < 3:
        g = geosgs.CartesianGrid((int(rng.integers(5, 30)), int(rng.integers(5, 30))),
                                 origin=(-3.0, 1.5), spacing=(1.0, 2.5) if case == 1 else (1.0, 1.0))
    else:
        g = geosgs.CartesianGrid((int(rng.integers(4, 12)),) * 3, spacing=(1.0, 1.0, 0.5 if case == 4 else 1.0))
    n = g.nelements()
    k = int(rng.integers(1, min(60, n)))
    src = rng.choice(n, size=k, replace=False)
    got = geosgs.traverse(g, geosgs.SourcePath(src))
    assert got.dtype == np.int32 and sorted(got.tolist()) == list(range(n))
    np.testing.assert_array_equal(got, brute_source_order(g, src))


def test_source_path_symmetric_sources_need_every_column():
    """Sources on a symmetric pattern: mirror-image nodes tie on their whole
    distance vectors, others only break ties after several columns, so the
    lazy refinement has to widen past its first columns to reach the rule's
    order."""
    g = geosgs.CartesianGrid((15, 15))
    src = [g.linear_index(i, j) for i, j in [(3, 3), (11, 3), (3, 11), (11, 11), (7, 7), (7, 3), (3, 7),
                                              (11, 7), (7, 11), (0, 0), (14, 14)]]
    np.testing.assert_array_equal(geosgs.traverse(g, geosgs.SourcePath(src)), brute_source_order(g, src))
    g3 = geosgs.CartesianGrid((9, 9, 9))
    src3 = [g3.linear_index(*c) for c in [(2, 2, 2), (6, 2, 2), (2, 6, 2), (2, 2, 6), (6, 6, 6), (4, 4, 4)]]
    np.testing.assert_array_equal(geosgs.traverse(g3, geosgs.SourcePath(src3)), brute_source_order(g3, src3))


def test_source_path_errors():
    g = geosgs.CartesianGrid((4, 4))
    for bad in ([], [16], [-1], [3, 3]):
        with pytest.raises(geosgs.ArgumentError):
            geosgs.traverse(g, geosgs.SourcePath(bad))


def test_source_path_at_scale():
    """A 400 x 400 grid with 2,000 sources: the k-d tree and the lazy columns
    keep it to seconds (the brute-force rule would hold 320 M distances)."""
    g = geosgs.CartesianGrid((400, 400))
    rng = np.random.default_rng(5)
    src = rng.choice(g.nelements(), size=2000, replace=False)
    p = geosgs.traverse(g, geosgs.SourcePath(src))
    assert np.array_equal(np.sort(p), np.arange(g.nelements()))
    np.testing.assert_array_equal(p[:2000], src)
    # distance to the nearest source never decreases along the path
    xyz = g.centroids()
    from scipy.spatial import cKDTree

    d, _ = cKDTree(xyz[src]).query(xyz[p[2000:]])
    assert np.all(np.diff(d) >= -1e-12)


def test_shifted_path():
    g = geosgs.CartesianGrid((6, 5))
    base = geosgs.RandomPath(3)
    p = geosgs.traverse(g, base)
    np.testing.assert_array_equal(geosgs.traverse(g, geosgs.ShiftedPath(base, 7)), np.concatenate([p[7:], p[:7]]))
    np.testing.assert_array_equal(geosgs.traverse(g, geosgs.ShiftedPath(base, -4)), np.concatenate([p[-4:], p[:-4]]))
    np.testing.assert_array_equal(geosgs.traverse(g, geosgs.ShiftedPath(geosgs.LinearPath(), 0)), np.arange(30))
    src = geosgs.SourcePath([4, 20])
    np.testing.assert_array_equal(geosgs.traverse(g, geosgs.ShiftedPath(src, 2)), np.roll(geosgs.traverse(g, src), -2))


def test_nearest_nodes():
    g = geosgs.CartesianGrid((4, 3), origin=(1.0, -2.0), spacing=(2.0, 1.0))
    pts = np.array([
        [2.0, -1.5],    # centre of cell (0, 0)
        [7.9, 0.9],     # inside cell (3, 2)
        [100.0, -50.0],  # outside: the nearest edge cell (3, 0)
        [3.0, -1.0],    # on the face between cells (0, 0)/(1, 0) and (0, 1)/(0, 0): the lower cells
        [4.1, -0.49],   # cell (1, 1)
    ])
    want = [g.linear_index(0, 0), g.linear_index(3, 2), g.linear_index(3, 0), g.linear_index(0, 0),
            g.linear_index(1, 1)]
    np.testing.assert_array_equal(geosgs.nearest_nodes(g, pts), want)
    with pytest.raises(geosgs.ArgumentError):
        geosgs.nearest_nodes(g, np.zeros((2, 3)))


def test_defaultsimulation_follows_the_reference():
    grid = geosgs.CartesianGrid((20, 20))
    gp = geosgs.GaussianProcess(geosgs.SphericalVariogram(range=5.0))
    ip = geosgs.IndicatorProcess(geosgs.SphericalTransiogram(range=5.0))
    assert isinstance(geosgs.defaultsimulation(gp, grid).path, geosgs.LinearPath)
    assert isinstance(geosgs.defaultsimulation(ip, grid).path, geosgs.LinearPath)
    # data: the nearest nodes, each once, in data order
    coords = np.array([[10.2, 3.7], [0.1, 0.1], [10.4, 3.9], [19.5, 19.5], [0.6, 0.4]])
    data = geosgs.georef({"C": np.array([1, 2, 1, 2, 1])}, coords)
    m = geosgs.defaultsimulation(ip, grid, data=data)
    assert isinstance(m.path, geosgs.SourcePath)
    np.testing.assert_array_equal(m.path.sources, [grid.linear_index(10, 3), 0, grid.linear_index(19, 19)])
    assert (m.minneighbors, m.maxneighbors, m.neighborhood) == (1, 26, "range")
    # a Gaussian process keeps the linear path with data too
    gdata = geosgs.georef({"Z": np.array([0.1, 0.2])}, coords[:2])
    assert isinstance(geosgs.defaultsimulation(gp, grid, data=gdata).path, geosgs.LinearPath)


def test_source_path_reaches_the_problem():
    grid = geosgs.CartesianGrid((12, 9))
    ip = geosgs.IndicatorProcess(geosgs.SphericalTransiogram(range=4.0))
    data = geosgs.georef({"C": np.array([1, 2, 2])}, np.array([[3.5, 4.5], [8.2, 1.1], [3.4, 4.4]]))
    m = geosgs.defaultsimulation(ip, grid, data=data)
    p, keep = geosgs.build_problem(ip, grid, data, m)
    got = np.ctypeslib.as_array(p.path, shape=(grid.nelements(),))
    np.testing.assert_array_equal(got, geosgs.traverse(grid, m.path))
    assert got[0] == grid.linear_index(3, 4) and got[1] == grid.linear_index(8, 1)
    assert isinstance(p, _abi.SgsProblem)


def test_paths_on_1d_and_3d_grids():
    g1 = geosgs.CartesianGrid((9,), origin=(2.0,), spacing=(0.5,))
    np.testing.assert_array_equal(geosgs.nearest_nodes(g1, [[2.1], [6.4], [-3.0]]), [0, 8, 0])
    np.testing.assert_array_equal(geosgs.traverse(g1, geosgs.SourcePath([4])), [4, 3, 5, 2, 6, 1, 7, 0, 8])
    g3 = geosgs.CartesianGrid((5, 4, 3), spacing=(1.0, 2.0, 0.5))
    pts = np.array([[0.2, 0.1, 0.1], [4.9, 7.9, 1.4], [2.5, 3.0, 0.74]])
    want = [g3.linear_index(0, 0, 0), g3.linear_index(4, 3, 2), g3.linear_index(2, 1, 1)]
    np.testing.assert_array_equal(geosgs.nearest_nodes(g3, pts), want)
    ip = geosgs.IndicatorProcess(geosgs.SphericalTransiogram(range=2.0))
    m = geosgs.defaultsimulation(ip, g3, data=geosgs.georef({"C": [1, 2, 1]}, pts))
    np.testing.assert_array_equal(m.path.sources, want)
    p = geosgs.traverse(g3, m.path)
    np.testing.assert_array_equal(p, brute_source_order(g3, want))

"""Edge cases of the plan path against the FP64 oracle: the largest and
smallest neighbour counts, maxneighbors clamped to the grid size, a one-node
grid, degenerate axes, a 1D grid (run as n x 1), duplicate data locations (colliding data make the
kriging system singular where both are neighbours), data outside the grid,
minneighbors equal to maxneighbors, a single realization, non-unit and
unequal spacings with an offset origin.  Bars as in the parity suite:
neighbour rows and counts bit-exact, node status identical, values within
1e-6 relative."""
import numpy as np
import pytest

import geosgs

pytestmark = pytest.mark.gpu

VALUE_TOL = 1e-6


def rel_err(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0))) if a.size else 0.0


def case(dims, k, ndata=0, nmin=1, seed=0, vario=geosgs.ExponentialVariogram, rng_=6.0, nugget=0.02,
         origin=None, spacing=None, ball=None, data_xyz=None, data_val=None, path="random"):
    grid = geosgs.CartesianGrid(tuple(dims), origin=origin, spacing=spacing)
    rng = np.random.default_rng(seed)
    data = None
    if data_xyz is not None:
        data = geosgs.georef({"Z": np.asarray(data_val, dtype=np.float64)}, np.asarray(data_xyz, dtype=np.float64))
    elif ndata:
        lo = np.asarray(grid.origin, dtype=np.float64)
        ext = np.asarray(grid.dims, dtype=np.float64) * np.asarray(grid.spacing, dtype=np.float64)
        xyz = lo + rng.uniform(0.0, 1.0, (ndata, len(dims))) * ext
        data = geosgs.georef({"Z": rng.standard_normal(ndata)}, xyz)
    proc = geosgs.GaussianProcess(vario(range=rng_, sill=1.3, nugget=nugget), 0.4)
    p = geosgs.RandomPath(seed) if path == "random" else geosgs.LinearPath()
    return proc, grid, data, p, k, nmin, ball


CASES = {
    "k64_max": case((20, 20), 64, ndata=30, seed=1, rng_=9.0),
    "k1": case((24, 24), 1, ndata=10, seed=2),
    "k_above_n": case((5, 5), 40, ndata=3, seed=3),
    "one_node": case((1, 1), 8, ndata=2, seed=4),
    "line_1x50": case((1, 50), 6, ndata=5, seed=5),
    "flat_3d": case((16, 12, 1), 10, ndata=8, seed=6),
    "duplicate_data": case((12, 12), 8, data_xyz=[[3.5, 4.5], [3.5, 4.5], [8.2, 2.1], [8.2, 2.1], [6.0, 9.0]],
                           data_val=[1.0, -1.0, 0.5, 0.5, 2.0], seed=7),
    "data_outside": case((15, 15), 10, data_xyz=[[-3.0, 4.0], [20.0, 7.5], [7.0, -2.0], [7.5, 7.5]],
                         data_val=[1.0, 2.0, -1.0, 0.0], seed=8, ball=geosgs.MetricBall(10.0)),
    "nmin_equals_k": case((20, 20), 8, ndata=12, nmin=8, seed=9),
    "spacing_origin": case((18, 14, 6), 12, ndata=20, seed=10, origin=(100.0, -50.0, 3.0), spacing=(2.5, 1.0, 0.5),
                           rng_=12.0, vario=geosgs.SphericalVariogram),
    "gaussian_linear_path": case((20, 20), 16, ndata=15, seed=11, vario=geosgs.GaussianVariogram, nugget=0.0,
                                 path="linear"),
    "line_1d": case((300,), 8, ndata=6, seed=12, rng_=12.0),
}


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_edge_case_matches_oracle(name, precision, oracle_mod, geosgs_lib):
    proc, grid, data, path, k, nmin, ball = CASES[name]
    method = geosgs.GPUSEQSIM(path=path, maxneighbors=k, minneighbors=nmin, precision=precision,
                              neighborhood=ball if ball is not None else "range")
    p, keep = geosgs.build_problem(proc, grid, data, method)
    G = geosgs.Plan(p, keep).prepare()
    O = oracle_mod.OraclePlan(p, keep).prepare()
    info = G.info()
    if precision == "fp64":
        assert info.values_fp64 == 1
    else:
        # FP32 values while the weights keep FP32 rounding small; the nugget-free
        # Gaussian model's weights (sum |w| ~ 100) make the sweep keep FP64 values
        assert info.values_fp64 == (1 if info.weight_l1_max > 4.0 else 0)
        if name == "gaussian_linear_path":
            assert info.values_fp64 == 1 and info.weight_l1_max > 10.0
    ig, cg = G.neighbors()
    io, co = O.neighbors()
    np.testing.assert_array_equal(cg, co)
    np.testing.assert_array_equal(ig, io)
    _, _, stg = G.weights()
    _, _, sto = O.weights()
    np.testing.assert_array_equal(stg, sto)
    for R in (1, 5):
        z = np.random.default_rng(R).standard_normal((R, G.N))
        assert rel_err(G.simulate(R, z), O.simulate(R, z)) <= VALUE_TOL, R
    G.close()

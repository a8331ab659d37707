"""Neighbour order and ball membership under the reference's `_scale`
(src/simulation/field/seqsim.jl:162-189).

The reference scales the domain, the data, the variogram and the ball by
alpha = 1 / max(largest absolute bounding-box coordinate of the domain, of
the data, range(f)) and searches in scaled FP64 coordinates.  This build
searches unscaled grid lags (integer offsets x spacing) in one canonical FP64
arithmetic (host_d2 / metric_d2: the ellipsoid metric with reciprocal radii
rounded once).  In exact arithmetic the two agree: scaling is a similarity
transform.  For every grid offset of each benchmark configuration's search
template these tests check where rounding could make them disagree:

  * offsets fall into classes of equal squared distance (up to 1e-15
    relative: exact ties such as h and -h, and ties of the true rotation that
    the FP64 cosines and sines split by ~1e-17), with relative gaps between
    classes far above FP64 rounding, so neither arithmetic can reorder two
    classes; the canonical FP64 values order the classes exactly as the
    exact values do, and so do the scaled FP64 values at sample query nodes.
    Within a class both arithmetics break ties by rounding noise and then by
    their own rule (canonical: point index; reference: tree traversal), the
    one order no build can reproduce without the reference's code;
  * the canonical in/out decision equals the exact one for every offset;
  * the scaled FP64 decision can differ from the exact one only for offsets
    lying exactly on the ball's boundary.  Those exist in the isotropic 2D
    cases with integer radii (12 offsets each, d = 40 at 100x100 and d = 30
    at 500x500) and in the ellipsoids rotated 30 degrees about z, whose
    metric is rational on the lattice's x and z axes (d^2 = 7x^2/(4 r_x^2) +
    ... + z^2/r_z^2 at y = 0): (0, 0, +-5) for radii 50/25/5, and (0, 0, +-8),
    (+-30, 0, +-1), (+-20, 0, +-6) for radii 40/20/8.  The canonical
    arithmetic decides them as the exact values do (checked above), while the
    reference's scaled rounding keeps or drops them depending on the node's
    position.  The counts are printed.

Exact values are taken in extended precision (numpy longdouble, 64-bit
significand), far below the 1e-12 relative gaps asserted."""
import numpy as np
import pytest

import geosgs
from geosgs import _abi, workloads

TIE = 1e-15      # relative: one class (exact ties, and ties of the true rotation
                 # that the FP64 cosines and sines split by ~1e-17)
MIN_GAP = 1e-12  # relative gap required between distinct classes


def _rmax(p):
    dim = p.dim
    r = max(p.variogram.ranges[j] for j in range(dim))
    for s in range(p.nstructures):
        r = max(r, max(p.structures[s].ranges[j] for j in range(dim)))
    return r


def _metric(p):
    """(kind, radii, rotation) as the library chooses them (api.cu)."""
    dim = p.dim
    if p.search == _abi.SGS_SEARCH_RANGE:
        r = _rmax(p)
        return "iso", np.array([r, r, r]), np.eye(3).reshape(-1)
    radii = np.array(p.ball.radii[:])
    R = np.array(p.ball.rotation[:])
    iso = np.array_equal(R.reshape(3, 3)[:dim, :dim], np.eye(dim)) and all(radii[j] == radii[0] for j in range(dim))
    return ("iso" if iso else "ellipsoid"), radii, R


def _offsets(p, kind, radii, R):
    dim = p.dim
    if kind == "iso":
        ext = np.full(3, radii[0])
    else:
        ext = np.array([np.sqrt(sum((R[i + 3 * j] * radii[j]) ** 2 for j in range(dim))) for i in range(3)])
    e = [int(np.ceil(ext[j] / p.spacing[j])) + 1 if j < dim else 0 for j in range(3)]
    g = np.meshgrid(*[np.arange(-e[j], e[j] + 1) for j in range(3)], indexing="ij")
    return np.stack([x.reshape(-1) for x in g], axis=1)


def _d2(h, kind, radii, R, dim, dtype, inv=None):
    """Squared metric distance of lags h (M x 3) in the canonical operation
    order, in `dtype`.  `inv`: reciprocal radii (the canonical form rounds
    1/r once in FP64; the exact form divides)."""
    h = h.astype(dtype)
    if kind == "iso":
        s = h[:, 0] * h[:, 0]
        s = s + h[:, 1] * h[:, 1]
        if dim == 3:
            s = s + h[:, 2] * h[:, 2]
        return s
    s = None
    for j in range(dim):
        u = dtype(R[0 + 3 * j]) * h[:, 0]
        u = u + dtype(R[1 + 3 * j]) * h[:, 1]
        if dim == 3:
            u = u + dtype(R[2 + 3 * j]) * h[:, 2]
        q = u * inv[j] if inv is not None else u / dtype(radii[j])
        s = q * q if s is None else s + q * q
    return s


def _classes(exact):
    """Sort order, and the start of each class of equal exact values."""
    o = np.argsort(exact, kind="stable")
    v = exact[o]
    rel = np.diff(v) / np.maximum(np.abs(v[1:]), np.finfo(np.float64).tiny)
    starts = np.concatenate([[0], np.nonzero(rel > TIE)[0] + 1])
    gaps = rel[rel > TIE]
    return o, starts, (float(gaps.min()) if gaps.size else np.inf)


def _order_kept(values, o, starts):
    """True when every class's values lie strictly below the next class's."""
    v = values[o]
    hi = np.maximum.reduceat(v, starts)
    lo = np.minimum.reduceat(v, starts)
    return bool(np.all(hi[:-1] < lo[1:]))


def _alpha(p, data):
    dim = p.dim
    hi = [abs(p.origin[j] + p.dims[j] * p.spacing[j]) for j in range(dim)]
    lo = [abs(p.origin[j]) for j in range(dim)]
    a = max(hi + lo)
    if data is not None and p.ndata:
        xyz = np.ctypeslib.as_array(p.data_coords, shape=(p.ndata * dim,)).reshape(p.ndata, dim)
        a = max(a, float(np.abs(xyz.min(axis=0)).max()), float(np.abs(xyz.max(axis=0)).max()))
    return 1.0 / max(a, _rmax(p))


def _check(name, wl, expect_boundary):
    if np.finfo(np.longdouble).eps > 1e-18:
        pytest.skip("needs an extended-precision longdouble")
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    dim = p.dim
    kind, radii, R = _metric(p)
    L = _offsets(p, kind, radii, R)
    sp = np.array(p.spacing[:])
    h64 = L * sp  # FP64 grid lags, exact (integers x spacing)
    exact = _d2(h64, kind, radii, R, dim, np.longdouble)
    bound_x = np.longdouble(radii[0]) ** 2 if kind == "iso" else np.longdouble(1.0)
    near = np.abs(exact - bound_x) / bound_x
    keep_sel = exact <= bound_x * (1 + 1e-6)  # the template and a thin shell outside it
    L, h64, exact, near = L[keep_sel], h64[keep_sel], exact[keep_sel], near[keep_sel]
    o, starts, gap = _classes(exact)
    assert gap > MIN_GAP, (name, gap)
    # canonical FP64 (unscaled): the exact order and the exact decision
    inv = np.array([1.0 / radii[j] for j in range(3)])
    ours = _d2(h64, kind, radii, R, dim, np.float64, inv)
    assert _order_kept(ours, o, starts), name
    bound64 = radii[0] * radii[0] if kind == "iso" else 1.0
    np.testing.assert_array_equal(ours <= bound64, exact <= bound_x)
    on_boundary = near <= TIE
    assert int(on_boundary.sum()) == expect_boundary, (name, int(on_boundary.sum()))
    assert float(near[~on_boundary].min()) > MIN_GAP, name
    # the reference's arithmetic: coordinates scaled after the centroid, lag
    # of scaled coordinates, scaled radii, at sample query nodes
    alpha = _alpha(p, wl.data)
    rs = alpha * radii
    inv_s = np.array([1.0 / rs[j] for j in range(3)])
    bound_s = rs[0] * rs[0] if kind == "iso" else 1.0
    rng = np.random.default_rng(0)
    dims = np.array([p.dims[j] if j < dim else 1 for j in range(3)])
    queries = [np.zeros(3, int), dims - 1, dims // 2] + [rng.integers(0, dims) for _ in range(13)]
    flips = 0
    for qi in queries:
        xp = np.array([p.origin[j] + (qi[j] + 0.5) * p.spacing[j] for j in range(3)])
        xq = np.array([p.origin[j] + (qi[j] + L[:, j] + 0.5) * p.spacing[j] for j in range(3)]).T
        hs = alpha * xq - alpha * xp
        if dim == 2:
            hs[:, 2] = 0.0
        scaled = _d2(hs, kind, rs, R, dim, np.float64, inv_s)
        assert _order_kept(scaled, o, starts), (name, qi)
        differ = (scaled <= bound_s) != (exact <= bound_x)
        assert not np.any(differ & ~on_boundary), (name, qi)
        flips += int(differ.sum())
    v = ours[o]
    split = int(np.sum(np.maximum.reduceat(v, starts) != np.minimum.reduceat(v, starts)))
    print(f"{name}: {len(L)} offsets, {len(starts)} distance classes ({split} split by FP64 rounding), "
          f"min relative gap {gap:.2e}, "
          f"{int(on_boundary.sum())} on the boundary; scaled-arithmetic decisions differing there: "
          f"{flips} of {int(on_boundary.sum()) * len(queries)} (alpha = {alpha:g})")


@pytest.mark.parametrize("config", ["c1", "c2", "c3", "c4"])
def test_template_order_and_boundary_under_scaling(config):
    wl, expect = {"c1": (workloads.c1("fp64"), 12), "c2": (workloads.c2("fp32"), 12),
                  "c3": (workloads.c3("fp32"), 2), "c4": (workloads.c4("fp32"), 10)}[config]
    _check(config, wl, expect)


def test_c5_domain_templates_under_scaling():
    """The first 40 domains of the uneven batch (isotropic :range balls of
    real-valued radii: no offset on a boundary)."""
    for d, wl in enumerate(workloads.c5("fp32", ndomains=40).items):
        _check(f"c5 domain {d}", wl, 0)

"""Host-side mirror of the reference's objects on the SEQSIM path.

GaussianProcess            src/processes/field/gaussian.jl:22-35
variograms / MetricBall    GeoStatsFunctions 0.15 / Meshes 0.57 (the reference's
                           dependencies): practical-range spherical, exponential
                           and gaussian variograms with nugget, anisotropy by a
                           rotated ellipsoid
CartesianGrid, paths       Meshes 0.57 CartesianGrid, LinearPath, RandomPath,
                           ShiftedPath, SourcePath, traverse
georef / GeoTable          GeoTables: values + point coordinates

Only what the GPU SEQSIM path consumes is mirrored.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _abi


class ArgumentError(ValueError):
    """Invalid argument (the reference raises Julia's ArgumentError)."""


# ---------------------------------------------------------------- rotations
def RotZ(deg: float) -> np.ndarray:
    """Counter-clockwise rotation by `deg` degrees about +z (Rotations.jl RotZ)."""
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


def RotY(deg: float) -> np.ndarray:
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0.0, s], [0.0, 1.0, 0.0], [-s, 0.0, c]])


def RotX(deg: float) -> np.ndarray:
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    return np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])


def _rot3(rotation) -> np.ndarray:
    if rotation is None:
        return np.eye(3)
    R = np.asarray(rotation, dtype=np.float64)
    if R.shape == (2, 2):
        R3 = np.eye(3)
        R3[:2, :2] = R
        return R3
    if R.shape != (3, 3):
        raise ArgumentError("rotation must be a 2x2 or 3x3 matrix")
    return R


# -------------------------------------------------------------- neighbourhoods
@dataclass
class MetricBall:
    """Ellipsoid |diag(1/radii) R^T h| <= 1 (isotropic ball when one radius)."""

    radii: Sequence[float] | float
    rotation: np.ndarray | None = None

    def __post_init__(self):
        r = np.atleast_1d(np.asarray(self.radii, dtype=np.float64))
        self.radii = tuple(float(x) for x in r)
        self.rotation = _rot3(self.rotation)

    def radius(self) -> float:
        return self.radii[0]

    def padded_radii(self, dim: int) -> tuple:
        r = list(self.radii)
        if len(r) == 1:
            r = r * dim
        if len(r) < dim:
            raise ArgumentError("MetricBall has fewer radii than the domain's dimension")
        return tuple(r[:dim]) + (1.0,) * (3 - dim)


# ----------------------------------------------------------------- variograms
@dataclass
class _Variogram:
    ball: MetricBall = field(default_factory=lambda: MetricBall(1.0))
    sill: float = 1.0
    nugget: float = 0.0
    TYPE = 0

    def __init__(self, ball=None, *, range=None, ranges=None, rotation=None, sill=1.0, nugget=0.0):
        if ball is None:
            if ranges is not None:
                ball = MetricBall(ranges, rotation)
            else:
                ball = MetricBall(1.0 if range is None else range, rotation)
        self.ball = ball
        self.sill = float(sill)
        self.nugget = float(nugget)

    def range(self) -> float:
        """Largest radius of the variogram's ellipsoid (GeoStatsFunctions `range`)."""
        return max(self.ball.radii)

    def _f(self, h):
        raise NotImplementedError

    def __call__(self, h):
        """gamma(h) for a normalized lag h (h = 1 at the range)."""
        h = np.asarray(h, dtype=np.float64)
        return np.where(h > 0, self.nugget + (self.sill - self.nugget) * self._f(h), 0.0)

    def gamma_at(self, lag, dim: int):
        """gamma of lag vectors (rows of `lag`, dim components): the lag is
        normalized by the structure's ellipsoid, |diag(1/ranges) R^T lag|."""
        lag = np.atleast_2d(np.asarray(lag, dtype=np.float64))[:, :dim]
        R = self.ball.rotation[:dim, :dim]
        r = np.asarray(self.ball.padded_radii(dim)[:dim])
        return self(np.sqrt((((lag @ R) / r) ** 2).sum(axis=1)))

    def structures(self) -> list:
        """The model's structures (one for a single variogram)."""
        return [self]

    def __add__(self, other):
        """gamma_1 + gamma_2: a nested model (GeoStatsFunctions NestedVariogram)."""
        if not isinstance(other, _Variogram):
            return NotImplemented
        return NestedVariogram(self.structures() + other.structures())

    def to_c(self, dim: int) -> _abi.SgsVariogram:
        v = _abi.SgsVariogram()
        v.type = self.TYPE
        v.sill = self.sill
        v.nugget = self.nugget
        for j, r in enumerate(self.ball.padded_radii(dim)):
            v.ranges[j] = r
        R = self.ball.rotation
        for i in range(3):
            for j in range(3):
                v.rotation[i + 3 * j] = R[i, j]
        return v


class SphericalVariogram(_Variogram):
    TYPE = _abi.SGS_SPHERICAL

    def _f(self, h):
        return np.where(h < 1, 1.5 * h - 0.5 * h**3, 1.0)


class ExponentialVariogram(_Variogram):
    TYPE = _abi.SGS_EXPONENTIAL

    def _f(self, h):
        return 1.0 - np.exp(-3.0 * h)


class GaussianVariogram(_Variogram):
    TYPE = _abi.SGS_GAUSSIAN

    def _f(self, h):
        return 1.0 - np.exp(-3.0 * h * h)


class NestedVariogram(_Variogram):
    """A sum of variogram structures, gamma(h) = gamma_1(h) + ... + gamma_m(h)
    (GeoStatsFunctions' NestedVariogram, written `g1 + g2` there and here):
    every structure keeps its own sill, nugget, ranges and rotation; the
    model's sill and nugget are their sums and its range the largest
    (`range` of a nested model).  Up to SGS_MAX_STRUCTURES structures."""

    def __init__(self, structures):
        st = []
        for g in structures:
            if not isinstance(g, _Variogram):
                raise ArgumentError("a nested variogram sums variograms")
            st += g.structures()
        if not 1 <= len(st) <= _abi.SGS_MAX_STRUCTURES:
            raise ArgumentError("a nested variogram takes 1 to %d structures on the GPU" % _abi.SGS_MAX_STRUCTURES)
        self._st = st
        self.ball = st[0].ball
        self.sill = float(sum(g.sill for g in st))
        self.nugget = float(sum(g.nugget for g in st))

    def structures(self) -> list:
        return list(self._st)

    def range(self) -> float:
        return max(g.range() for g in self._st)

    def __call__(self, h):
        raise ArgumentError("a nested model has one normalized lag per structure; evaluate gamma_at(lag)")

    def gamma_at(self, lag, dim: int):
        """gamma of a lag vector (rows of `lag`), summed over the structures."""
        return sum(g.gamma_at(lag, dim) for g in self._st)

    def to_c(self, dim: int) -> _abi.SgsVariogram:
        return self._st[0].to_c(dim)


# ------------------------------------------------------------------- process
class GaussianProcess:
    """GaussianProcess(func, mean=0) — src/processes/field/gaussian.jl:22-35.

    A variogram with a scalar mean, or a multivariate function (a linear
    model of coregionalization of L variables) with L means (zeros by
    default, as gaussian.jl:35 gives)."""

    def __init__(self, func, mean=None):
        if isinstance(func, LinearCoregionalization):
            L = func.nvariables
            m = np.zeros(L) if mean is None else np.asarray(mean, dtype=np.float64).reshape(-1)
            if m.size != L:  # gaussian.jl:28-30
                raise ArgumentError(f"mean must have {L} components, received {m.size}")
            if not np.all(np.isfinite(m)):
                raise ArgumentError("mean must be finite")
            self.func = func
            self.mean = tuple(float(x) for x in m)
            return
        if not isinstance(func, _Variogram):
            raise ArgumentError("GaussianProcess on the GPU path takes a variogram or a linear model of "
                                "coregionalization")
        if mean is None:
            mean = 0.0
        if np.ndim(mean) != 0 and np.size(mean) != 1:
            raise ArgumentError(f"mean must have 1 components, received {np.size(mean)}")
        self.func = func
        self.mean = float(np.asarray(mean).reshape(-1)[0])

    @property
    def nvariables(self) -> int:
        return self.func.nvariables if isinstance(self.func, LinearCoregionalization) else 1


class _Transiogram:
    """A proportional transiogram: t_ab(h) = p_b + (delta_ab - p_b) (1 - g(h))
    with g a unit-sill variogram shape (GeoStatsFunctions' Spherical /
    Exponential / Gaussian transiograms with `range` and `proportions`).  Its
    indicator covariances p_a (t_ab(h) - p_b) = (diag(p) - p p')_ab (1 - g(h))
    are separable: every category shares the correlogram 1 - g."""

    SHAPE = None

    def __init__(self, ball=None, *, range=None, ranges=None, rotation=None, proportions=(0.5, 0.5)):
        self.shape = self.SHAPE(ball, range=range, ranges=ranges, rotation=rotation, sill=1.0, nugget=0.0)
        p = np.asarray(proportions, dtype=np.float64)
        if p.ndim != 1 or len(p) < 2 or np.any(p < 0) or not p.sum() > 0:
            raise ArgumentError("proportions must be at least two non-negative numbers")
        self.proportions = tuple(float(x) for x in p / p.sum())


class SphericalTransiogram(_Transiogram):
    SHAPE = SphericalVariogram


class ExponentialTransiogram(_Transiogram):
    SHAPE = ExponentialVariogram


class GaussianTransiogram(_Transiogram):
    SHAPE = GaussianVariogram


class LinearCoregionalization:
    """A multivariate covariance C_ab(h) = sum_s A_s[a][b] C_s(h) (a linear model
    of coregionalization): symmetric positive semi-definite L x L matrices A_s
    times the covariances C_s = sill_s - gamma_s of variogram structures
    (GeoStatsFunctions writes it `A1 * Covariance1 + A2 * Covariance2`).  As an
    IndicatorProcess function it gives the categories' indicator
    cross-covariances; with structures of different ranges it is not
    separable, and the GPU path solves full simple cokriging systems."""

    def __init__(self, terms):
        terms = list(terms)
        if not 1 <= len(terms) <= _abi.SGS_MAX_STRUCTURES:
            raise ArgumentError("1 to %d structures" % _abi.SGS_MAX_STRUCTURES)
        mats, sts = [], []
        for A, g in terms:
            A = np.asarray(A, dtype=np.float64)
            if not isinstance(g, _Variogram) or isinstance(g, NestedVariogram):
                raise ArgumentError("each term is a matrix times one variogram structure")
            if A.ndim != 2 or A.shape[0] != A.shape[1] or A.shape[0] < 2 or not np.allclose(A, A.T):
                raise ArgumentError("coefficients must be symmetric L x L matrices, L >= 2")
            mats.append(A)
            sts.append(g)
        L = mats[0].shape[0]
        if any(A.shape[0] != L for A in mats):
            raise ArgumentError("all coefficient matrices must have the same size")
        if L > _abi.SGS_IND_MAX_CATEGORIES:
            raise ArgumentError("at most %d categories on the GPU" % _abi.SGS_IND_MAX_CATEGORIES)
        self.coef = np.ascontiguousarray(np.stack(mats))
        self.nested = NestedVariogram(sts) if len(sts) > 1 else sts[0]
        self.nvariables = L

    def structures(self) -> list:
        return self.nested.structures()

    def range(self) -> float:
        return self.nested.range()


class IndicatorProcess:
    """IndicatorProcess(func, prob) — src/processes/field/indicator.jl:5-45.

    On the GPU path `func` is a separable indicator model: a transiogram
    above (prob defaults to its proportions) or a variogram taken as the
    categories' common correlogram with explicit `prob`; prob is normalized
    to sum to one (indicator.jl:40-43)."""

    def __init__(self, func, prob=None):
        if isinstance(func, _Transiogram):
            corr = func.shape
            prob = func.proportions if prob is None else prob
        elif isinstance(func, LinearCoregionalization):
            corr = func.nested
            if prob is None:
                raise ArgumentError("an indicator process on a coregionalization model needs its probabilities")
            if len(prob) != func.nvariables:
                raise ArgumentError(f"probabilities must have {func.nvariables} components, received {len(prob)}")
        elif isinstance(func, _Variogram):
            corr = func
            if prob is None:
                raise ArgumentError("an indicator process on a variogram needs its probabilities")
        else:
            raise ArgumentError("IndicatorProcess on the GPU path takes a transiogram, a variogram or a "
                                "linear model of coregionalization")
        p = np.asarray(prob, dtype=np.float64)
        if p.ndim != 1 or len(p) < 2 or np.any(p < 0) or np.any(p > 1) or not p.sum() > 0:
            raise ArgumentError("probabilities must be in [0, 1], at least two of them")
        if len(p) > _abi.SGS_IND_MAX_CATEGORIES:
            raise ArgumentError("at most %d categories on the GPU" % _abi.SGS_IND_MAX_CATEGORIES)
        self.func = func
        self.corr = corr
        self.prob = tuple(float(x) for x in p / p.sum())
        self.mean = 0.0


# -------------------------------------------------------------------- domain
class CartesianGrid:
    """Regular grid: CartesianGrid(dims) or CartesianGrid(start, finish, dims=...)
    or CartesianGrid(dims, origin=..., spacing=...)."""

    def __init__(self, *args, dims=None, origin=None, spacing=None):
        if len(args) == 1:
            d = args[0]
            dims = (d,) if np.ndim(d) == 0 else tuple(d)
            origin = origin if origin is not None else (0.0,) * len(dims)
            spacing = spacing if spacing is not None else (1.0,) * len(dims)
        elif len(args) == 2:
            start, finish = (np.asarray(a, dtype=np.float64) for a in args)
            if dims is None:
                raise ArgumentError("dims is required with start/finish")
            dims = tuple(dims)
            origin = tuple(start)
            spacing = tuple((finish - start) / np.asarray(dims, dtype=np.float64))
        elif dims is not None:
            dims = tuple(dims)
            origin = origin if origin is not None else (0.0,) * len(dims)
            spacing = spacing if spacing is not None else (1.0,) * len(dims)
        else:
            raise ArgumentError("invalid CartesianGrid arguments")
        self.dims = tuple(int(x) for x in dims)
        self.origin = tuple(float(x) for x in origin)
        self.spacing = tuple(float(x) for x in spacing)
        if len(self.dims) not in (1, 2, 3) or len(self.origin) != len(self.dims) or len(self.spacing) != len(self.dims):
            raise ArgumentError("the GPU path supports 1D, 2D and 3D grids")

    @property
    def dim(self) -> int:
        return len(self.dims)

    def nelements(self) -> int:
        return int(np.prod(self.dims))

    def centroids(self) -> np.ndarray:
        """Cell centres, node-major (first axis fastest)."""
        axes = [self.origin[j] + (np.arange(self.dims[j]) + 0.5) * self.spacing[j] for j in range(self.dim)]
        mesh = np.meshgrid(*axes, indexing="ij")
        return np.stack([m.reshape(-1, order="F") for m in mesh], axis=1)

    def linear_index(self, *ijk) -> int:
        """0-based node id of (0-based) cell indices."""
        g, mult = 0, 1
        for j, i in enumerate(ijk):
            g += int(i) * mult
            mult *= self.dims[j]
        return g


class GeoTable:
    """Point data: one variable per column and D x dim coordinates."""

    def __init__(self, values: dict, coords):
        # numeric columns as FP64, categorical ones (integer or string
        # labels of an indicator process) as given
        self.values = {k: (np.asarray(v, dtype=np.float64) if np.asarray(v).dtype.kind == "f" else np.asarray(v))
                       for k, v in values.items()}
        c = np.asarray(coords, dtype=np.float64)
        if c.ndim == 1:
            c = c[:, None]
        self.coords = np.ascontiguousarray(c)
        for k, v in self.values.items():
            if v.shape != (self.coords.shape[0],):
                raise ArgumentError(f"column {k} does not match the number of points")

    def nrow(self) -> int:
        return self.coords.shape[0]


def georef(values: dict, coords) -> GeoTable:
    return GeoTable(values, coords)


# --------------------------------------------------------------------- paths
class LinearPath:
    """Visit nodes in linear index order (SEQSIM's default path)."""

    def permutation(self, n: int):
        return None


class RandomPath:
    """A random visiting order from a seeded generator (numpy PCG64).

    The permutation is drawn once per plan and shared by all realizations
    of that plan; Julia's randperm stream is not reproduced."""

    def __init__(self, seed: int = 0):
        self.seed = int(seed)

    def permutation(self, n: int):
        return np.random.Generator(np.random.PCG64(self.seed)).permutation(n).astype(np.int32)

    def permutations(self, n: int, count: int):
        """The first `count` permutations the path's generator draws, one
        after another: what `traverse(domain, path)` yields on successive
        realizations of the reference's randsingle (seqsim.jl:98)."""
        gen = np.random.Generator(np.random.PCG64(self.seed))
        return [gen.permutation(n).astype(np.int32) for _ in range(count)]


class ExplicitPath:
    """A caller-given permutation of the grid nodes (0-based)."""

    def __init__(self, perm):
        self.perm = np.ascontiguousarray(np.asarray(perm, dtype=np.int32))

    def permutation(self, n: int):
        if self.perm.shape != (n,):
            raise ArgumentError("path length does not match the domain")
        return self.perm


class ShiftedPath:
    """Meshes' ShiftedPath(path, offset): the order of `path` rotated so that
    it starts at its entry `offset` (0-based; a negative offset counts from
    the end) and wraps around to the entries before it."""

    def __init__(self, path, offset: int):
        self.path = path
        self.offset = int(offset)

    def order(self, domain):
        p = traverse(domain, self.path)
        return np.roll(p, -self.offset) if p.size else p


# rows of one k-d tree query (bounds the query's index and distance arrays)
_QUERY_ROWS = 1 << 20


def _sorted_source_distances(tree, src_xyz, xyz, k):
    """For each row of `xyz`, its Euclidean distances to its k nearest sources
    in ascending order: neighbours from the k-d tree, distances recomputed
    from the centroids in one FP64 order (squared coordinate differences
    summed in axis order, then the square root)."""
    out = np.empty((xyz.shape[0], k), dtype=np.float64)
    for r0 in range(0, xyz.shape[0], _QUERY_ROWS):
        x = xyz[r0: r0 + _QUERY_ROWS]
        _, nb = tree.query(x, k=k)
        nb = np.asarray(nb).reshape(x.shape[0], k)
        diff = x[:, None, :] - src_xyz[nb]
        s = diff[..., 0] * diff[..., 0]
        for a in range(1, x.shape[1]):
            s = s + diff[..., a] * diff[..., a]
        out[r0: r0 + _QUERY_ROWS] = np.sort(np.sqrt(s), axis=1)
    return out


def _lexsort_rows(keys, ids, group=None):
    """Indices ordering the rows of `keys` lexicographically (first column
    first), then by `ids`; within `group` first when given."""
    cols = [ids] + [keys[:, j] for j in reversed(range(keys.shape[1]))]
    if group is not None:
        cols.append(group)
    return np.lexsort(tuple(cols))


class SourcePath:
    """Meshes' SourcePath(sources): the sources first, in the given order,
    then the other nodes growing outwards from them.

    Meshes 0.57 (a dependency the reference does not vendor) fits a k-d tree
    to the sources' centroids, queries every other element for its distances
    to all the sources, sorted ascending, and orders the elements by these
    distance vectors compared lexicographically (the nearest source decides,
    then the second nearest, and so on) in a stable sort over element order.
    This restatement computes the same keys in FP64 and lets node id settle
    what the vectors leave tied.  It refines lazily: the order is first taken
    on each node's few nearest distances, and only runs of nodes still tied
    get further columns, doubling until the ties break or every source is
    used.  Sources are 0-based node ids.  The reference builds this path for
    IndicatorProcess with data (src/simulation/field.jl:168-180)."""

    def __init__(self, sources):
        self.sources = np.asarray(sources, dtype=np.int64).reshape(-1)

    def order(self, domain):
        from scipy.spatial import cKDTree

        n = domain.nelements()
        src = self.sources
        if src.size == 0:
            raise ArgumentError("SourcePath needs at least one source")
        if np.any(src < 0) or np.any(src >= n):
            raise ArgumentError("sources must be valid locations")
        if np.unique(src).size != src.size:
            raise ArgumentError("non-unique sources")
        others = np.setdiff1d(np.arange(n, dtype=np.int64), src)
        if others.size == 0:
            return src.astype(np.int32)
        xyz = domain.centroids()
        src_xyz = np.ascontiguousarray(xyz[src])
        tree = cKDTree(src_xyz)
        K = src.size
        k = min(K, 4)
        keys = _sorted_source_distances(tree, src_xyz, xyz[others], k)
        order = _lexsort_rows(keys, others)
        pos, run = _tied_runs(keys[order], np.zeros(others.size, dtype=np.int64))
        while pos.size and k < K:
            k = min(K, 2 * k)
            mem = others[order[pos]]
            keys = _sorted_source_distances(tree, src_xyz, xyz[mem], k)
            o = _lexsort_rows(keys, mem, run)
            order[pos] = order[pos][o]
            sub, run = _tied_runs(keys[o], run[o])
            pos = pos[sub]
        return np.concatenate([src, others[order]]).astype(np.int32)


def _tied_runs(keys, group):
    """Rows (of sorted `keys`) that equal a neighbour row of the same group,
    and a run id for each of them."""
    same = np.all(keys[1:] == keys[:-1], axis=1) & (group[1:] == group[:-1])
    tied = np.zeros(keys.shape[0], dtype=bool)
    tied[1:] |= same
    tied[:-1] |= same
    starts = np.ones(keys.shape[0], dtype=bool)
    starts[1:] = ~same
    rid = np.cumsum(starts) - 1
    sel = np.nonzero(tied)[0]
    return sel, rid[sel]


def traverse(domain, path) -> np.ndarray:
    """The nodes of `domain` in the order `path` visits them, 0-based (Meshes'
    traverse(domain, path), called once per realization at seqsim.jl:98)."""
    perm = path_order(domain, path)
    return np.arange(domain.nelements(), dtype=np.int32) if perm is None else np.asarray(perm, dtype=np.int32)


def path_order(domain, path):
    """What the library takes as the path: None for the linear order,
    otherwise the permutation."""
    if hasattr(path, "order"):
        return path.order(domain)
    return path.permutation(domain.nelements())


def nearest_nodes(domain, coords) -> np.ndarray:
    """The grid node whose centroid is nearest to each point (Meshes'
    KNearestSearch(domain, 1), src/simulation/field.jl:173-177).  On a
    regular grid the nearest centroid minimises each axis apart; equal
    distances go to the lower cell on that axis, so to the lowest node id."""
    c = np.asarray(coords, dtype=np.float64)
    if c.ndim == 1:
        c = c[:, None]
    if c.shape[1] != domain.dim:
        raise ArgumentError("point and grid dimensions differ")
    node = np.zeros(c.shape[0], dtype=np.int64)
    mult = 1
    for j in range(domain.dim):
        o, s, d = domain.origin[j], domain.spacing[j], domain.dims[j]
        i0 = np.clip(np.floor((c[:, j] - o) / s).astype(np.int64), 0, d - 1)
        cand = np.clip(i0[:, None] + np.array([-1, 0, 1]), 0, d - 1)
        dist = np.abs(c[:, j][:, None] - (o + (cand + 0.5) * s))
        node += cand[np.arange(c.shape[0]), np.argmin(dist, axis=1)] * mult
        mult *= d
    return node

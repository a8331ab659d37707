"""Generate the golden SGS fixtures in this folder from an independent numpy
restatement of the method (no code shared with the C++ oracle or the CUDA
library).

Restated from GeoStatsProcesses.jl v0.13.0 src/simulation/field/seqsim.jl:
the path loop (:98-138), neighbour search among data + earlier-visited
nodes (:107), simple kriging with the covariance sill - gamma (:124,
src/utils.jl:50-62), the prior fallback (:109-111, :127-131) and the draw
(:335-340); with the canonical neighbour order (FP64 distance, then
augmented index) and singular-pivot rule (pivot <= 1e-10 * sill) this
project defines for the parts the reference leaves to tree traversal order
and rounding.  Brute force everywhere: every earlier node and datum is a
candidate, sorted with numpy's lexsort; Cholesky by numpy's own loop.

    python tests/golden/make_golden.py      # rewrites golden_*.npz
"""
from __future__ import annotations

import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TAU = 1e-10


def rotz(deg):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


def cell(g, n):
    return np.array([g % n[0], (g // n[0]) % n[1], g // (n[0] * n[1])])


def centroid(i, origin, spacing, dim):
    return np.array([origin[j] + (float(i[j]) + 0.5) * spacing[j] for j in range(dim)] + [0.0] * (3 - dim))


def d2_metric(h, kind, radii, R, dim):
    h = [float(x) for x in h]
    if kind != "ellipsoid":
        s = h[0] * h[0]
        s = s + h[1] * h[1]
        if dim == 3:
            s = s + h[2] * h[2]
        return s
    s = 0.0
    for j in range(dim):
        u = R[0, j] * h[0]
        u = u + R[1, j] * h[1]
        if dim == 3:
            u = u + R[2, j] * h[2]
        q = u * (1.0 / radii[j])
        s = q * q if j == 0 else s + q * q
    return s


def cov(h, v, dim):
    h = np.asarray(h, dtype=np.float64)[:dim]
    if np.all(h == 0.0):
        return v["sill"]
    u = v["R"][:dim, :dim].T @ h
    hn = math.sqrt(float(np.sum((u / np.asarray(v["ranges"][:dim])) ** 2)))
    if v["type"] == 1:
        f = 1.5 * hn - 0.5 * hn**3 if hn < 1 else 1.0
    elif v["type"] == 2:
        f = 1.0 - math.exp(-3.0 * hn)
    else:
        f = 1.0 - math.exp(-3.0 * hn * hn)
    return v["sill"] - (v["nugget"] + (v["sill"] - v["nugget"]) * f)


def simulate(case):
    dim, n = case["dim"], case["dims"]
    origin, spacing = case["origin"], case["spacing"]
    N = int(np.prod(n[:dim]))
    nn = list(n[:dim]) + [1] * (3 - dim)
    X = case["data_xyz"]
    D = X.shape[0]
    path = case["path"]
    rank = np.empty(N, dtype=np.int64)
    rank[path] = np.arange(N)
    k = case["k"]
    kind, radii, R = case["search_kind"], case["search_radii"], case["search_R"]
    v = case["vario"]
    pts = np.zeros((N + D, 3))
    for g in range(N):
        pts[g] = centroid(cell(g, nn), origin, spacing, dim)
    pts[N:, :dim] = X

    def lag(a, b):
        if a < N and b < N:
            ia, ib = cell(a, nn), cell(b, nn)
            return np.array([float(ib[j] - ia[j]) * spacing[j] for j in range(dim)] + [0.0] * (3 - dim))
        return pts[b] - pts[a]

    nbr = -np.ones((N, k), dtype=np.int32)
    cnt = np.zeros(N, dtype=np.int32)
    W = np.zeros((N, k))
    sig = np.zeros(N)
    st = np.zeros(N, dtype=np.int32)
    rr = radii[0] * radii[0]
    for t in range(N):
        g = path[t]
        cands = [c for c in range(N) if rank[c] < t] + list(range(N, N + D))
        ds = np.array([d2_metric(lag(g, c), kind, radii, R, dim) for c in cands]) if cands else np.zeros(0)
        ids = np.array(cands, dtype=np.int64)
        if kind == "iso":
            keep = ds <= rr
        elif kind == "ellipsoid":
            keep = ds <= 1.0
        else:
            keep = np.ones_like(ds, dtype=bool)
        ds, ids = ds[keep], ids[keep]
        order = np.lexsort((ids, ds))[:k]
        sel = ids[order]
        cnt[g] = len(sel)
        nbr[g, : len(sel)] = sel
        m = len(sel)
        if m < case["nmin"]:
            st[g] = 1
            sig[g] = math.sqrt(v["sill"])
            continue
        K = np.array([[cov(lag(sel[a], sel[b]), v, dim) for b in range(m)] for a in range(m)])
        c = np.array([cov(lag(sel[a], g), v, dim) for a in range(m)])
        L = np.zeros_like(K)
        ok = True
        for j in range(m):
            s = K[j, j] - np.dot(L[j, :j], L[j, :j])
            if not s > TAU * v["sill"]:
                ok = False
                break
            L[j, j] = math.sqrt(s)
            for i in range(j + 1, m):
                L[i, j] = (K[i, j] - np.dot(L[i, :j], L[j, :j])) / L[j, j]
        if not ok:
            st[g] = 2
            sig[g] = math.sqrt(v["sill"])
            continue
        y = np.zeros(m)
        for i in range(m):
            y[i] = (c[i] - np.dot(L[i, :i], y[:i])) / L[i, i]
        w = np.zeros(m)
        for i in range(m - 1, -1, -1):
            w[i] = (y[i] - np.dot(L[i + 1:, i], w[i + 1:])) / L[i, i]
        W[g, :m] = w
        sig[g] = math.sqrt(max(v["sill"] - float(np.dot(w, c)), 0.0))
    # draws
    z = case["z"]
    R_ = z.shape[0]
    out = np.zeros((R_, N))
    mu = case["mean"]
    for r in range(R_):
        vals = np.full(N + D, np.nan)
        vals[N:] = case["data_val"]
        for t in range(N):
            g = path[t]
            if st[g] != 0:
                vals[g] = mu + math.sqrt(v["sill"]) * z[r, g]
            else:
                vals[g] = mu + float(np.dot(W[g, : cnt[g]], vals[nbr[g, : cnt[g]]] - mu)) + sig[g] * z[r, g]
        out[r] = vals[:N]
    return dict(nbr=nbr, cnt=cnt, w=W, sigma=sig, status=st, out=out)


def cases():
    rng = np.random.default_rng(2024)
    I = np.eye(3)
    cs = []
    # 2D isotropic spherical, unconditional, ball radius 4
    n = (10, 9, 1)
    N = 90
    cs.append(dict(name="sph2d", dim=2, dims=n, origin=(0.0, 0.0), spacing=(1.0, 1.0),
                   data_xyz=np.zeros((0, 2)), data_val=np.zeros(0), path=rng.permutation(N), k=6, nmin=1,
                   search_kind="iso", search_radii=(4.0, 4.0, 4.0), search_R=I,
                   vario=dict(type=1, sill=1.0, nugget=0.0, ranges=(5.0, 5.0, 5.0), R=I), mean=0.0,
                   z=rng.standard_normal((3, N))))
    # 2D gaussian with nugget, data (two on cell centres), :range ball, mean 2
    n = (11, 8, 1)
    N = 88
    xy = np.array([[2.5, 3.5], [7.5, 1.5], [4.2, 6.1], [9.9, 7.7], [0.3, 0.1]])
    cs.append(dict(name="gau2d_data", dim=2, dims=n, origin=(0.0, 0.0), spacing=(1.0, 1.0),
                   data_xyz=xy, data_val=rng.standard_normal(5), path=rng.permutation(N), k=8, nmin=2,
                   search_kind="iso", search_radii=(6.0, 6.0, 6.0), search_R=I,
                   vario=dict(type=3, sill=2.0, nugget=0.1, ranges=(6.0, 6.0, 6.0), R=I), mean=2.0,
                   z=rng.standard_normal((2, N))))
    # 3D anisotropic exponential, rotated search ellipsoid, data, non-unit spacing
    n = (7, 6, 4)
    N = 168
    R = rotz(30.0)
    xyz = rng.uniform(0, 1, (6, 3)) * np.array([7 * 2.0, 6 * 1.5, 4 * 1.0]) + np.array([10.0, -5.0, 0.5])
    cs.append(dict(name="exp3d_aniso", dim=3, dims=n, origin=(10.0, -5.0, 0.5), spacing=(2.0, 1.5, 1.0),
                   data_xyz=xyz, data_val=rng.standard_normal(6), path=rng.permutation(N), k=10, nmin=1,
                   search_kind="ellipsoid", search_radii=(8.0, 5.0, 2.5), search_R=R,
                   vario=dict(type=2, sill=1.0, nugget=0.05, ranges=(8.0, 5.0, 2.5), R=R), mean=-1.0,
                   z=rng.standard_normal((2, N))))
    # 2D nearest (no ball), linear path
    n = (8, 7, 1)
    N = 56
    cs.append(dict(name="knn2d_linear", dim=2, dims=n, origin=(0.0, 0.0), spacing=(1.0, 1.0),
                   data_xyz=np.array([[3.5, 3.5]]), data_val=np.array([1.5]), path=np.arange(N), k=5, nmin=1,
                   search_kind="nearest", search_radii=(1.0, 1.0, 1.0), search_R=I,
                   vario=dict(type=1, sill=1.0, nugget=0.0, ranges=(4.0, 4.0, 4.0), R=I), mean=0.0,
                   z=rng.standard_normal((2, N))))
    return cs


def main():
    for case in cases():
        res = simulate(case)
        v = case["vario"]
        np.savez_compressed(
            os.path.join(HERE, f"golden_{case['name']}.npz"),
            dim=case["dim"], dims=np.array(case["dims"]), origin=np.array(case["origin"]),
            spacing=np.array(case["spacing"]), data_xyz=case["data_xyz"], data_val=case["data_val"],
            path=np.asarray(case["path"], dtype=np.int32), k=case["k"], nmin=case["nmin"],
            search_kind=case["search_kind"], search_radii=np.array(case["search_radii"]),
            search_R=case["search_R"], vario_type=v["type"], sill=v["sill"], nugget=v["nugget"],
            ranges=np.array(v["ranges"]), vario_R=v["R"], mean=case["mean"], z=case["z"], **res)
        print(case["name"], "status", np.bincount(res["status"], minlength=3), "mean cnt", res["cnt"].mean())


if __name__ == "__main__":
    main()

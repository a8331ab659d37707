"""Learned warm start: the CUDA forward/backward kernels against the numpy
restatement (oracle/nn_oracle.py), training on systems the method
generates, and the warm-started solve against the oracle."""
import numpy as np
import pytest

import geosgs
import nn_oracle
from geosgs import learned, workloads

pytestmark = pytest.mark.gpu


def _random_batch(rng, S=24, k=32):
    feat = rng.standard_normal((S, k, nn_oracle.F)).astype(np.float32)
    count = rng.integers(1, k + 1, S).astype(np.int32)
    target = rng.standard_normal((S, k)).astype(np.float32) * 0.2
    for s in range(S):
        feat[s, count[s]:] = 0
        target[s, count[s]:] = 0
    return feat, count, target


def test_forward_and_gradients_match_cpu_oracle(geosgs_lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    params = learned.init_params(3) + rng.standard_normal(nn_oracle.NPARAMS).astype(np.float32) * 0.05
    feat, count, target = _random_batch(rng)
    p_d, f_d = torch.from_numpy(params).cuda(), torch.from_numpy(feat).cuda()
    c_d, t_d = torch.from_numpy(count).cuda(), torch.from_numpy(target).cuda()
    pred = learned.predict(p_d, f_d, c_d, torch).cpu().numpy()
    for s in range(len(count)):
        np.testing.assert_allclose(pred[s, :count[s]], nn_oracle.forward(params, feat[s], count[s]),
                                   rtol=1e-4, atol=1e-5)
    loss, grad = learned.loss_and_grad(p_d, f_d, c_d, t_d, torch)
    loss_ref, grad_ref = nn_oracle.loss_and_grad(params, feat, count, target)
    assert abs(loss - loss_ref) <= 1e-4 * max(1.0, abs(loss_ref))
    g = grad.cpu().numpy()
    scale = np.abs(grad_ref).max()
    np.testing.assert_allclose(g, grad_ref, rtol=0, atol=2e-4 * scale)


def test_training_and_warm_started_solve(oracle_mod, geosgs_lib):
    torch = pytest.importorskip("torch")
    feat, count, target = learned.generate(150000, seed=1, torch=torch, dims=(40, 40, 24))
    loss0, _ = learned.loss_and_grad(torch.from_numpy(learned.init_params(0)).cuda(), feat, count, target, torch)
    params, hist = learned.train(feat, count, target, torch, epochs=20, batch=8192, lr=3e-3)
    mean0 = loss0 / feat.shape[0]
    print(f"training loss {mean0:.3e} -> {hist[-1]:.3e} (mean squared weight {float((target ** 2).mean()):.3e})")
    assert hist[-1] < mean0 / 3
    # warm start on a held-out workload: every value still matches the oracle
    wl = workloads.small(dim=3, n=36, nz=16, k=32, vario="exp", ranges=(14.0, 7.0, 4.0),
                         rotation=geosgs.RotZ(20.0), nugget=0.08,
                         ball=geosgs.MetricBall((14.0, 7.0, 4.0), geosgs.RotZ(20.0)), precision="fp32", nreals=8)
    wl.method.warm_start = True
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = geosgs.Plan(p, keep).set_network(params).prepare()
    O = oracle_mod.OraclePlan(p, keep).prepare()
    inf = G.info()
    kriged = int((O.weights()[2] == 0).sum())
    print(f"warm start accepted {inf.n_warm_accepted} of {kriged} kriged systems, fallback {inf.n_fp64_fallback}")
    assert inf.n_warm_accepted > 0
    z = np.random.default_rng(4).standard_normal((8, O.N))
    vg, vo = G.simulate(8, z), O.simulate(8, z)
    assert float(np.max(np.abs(vg - vo) / np.maximum(np.abs(vo), 1.0))) <= 1e-6


@pytest.mark.parametrize("k", [32, 48])
def test_tensor_core_inference_matches_fp32(k, geosgs_lib):
    """BF16 tensor-core inference (tcgen05, FP32 accumulation) agrees with
    the FP32 CUDA-core forward pass of the same network on a plan's systems
    within BF16 rounding, and writes zeros past each node's neighbour count."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    params = learned.init_params(5) + rng.standard_normal(nn_oracle.NPARAMS).astype(np.float32) * 0.05
    wl = workloads.small(dim=3, n=40, nz=12, k=k, ndata=30, vario="exp", ranges=(12.0, 6.0, 4.0),
                         rotation=geosgs.RotZ(25.0), nugget=0.05,
                         ball=geosgs.MetricBall((12.0, 6.0, 4.0), geosgs.RotZ(25.0)), precision="fp32", nreals=4)
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = geosgs.Plan(p, keep).set_network(params).prepare()
    N = G.N
    tc = torch.full((N, G.k), 7.0, dtype=torch.float32, device="cuda")
    f32 = torch.full((N, G.k), 7.0, dtype=torch.float32, device="cuda")
    G.predict_device(tc.data_ptr(), tensor_cores=True)
    G.predict_device(f32.data_ptr(), tensor_cores=False)
    a, b = tc.cpu().numpy(), f32.cpu().numpy()
    _, cnt = G.neighbors()
    pad = np.arange(G.k)[None, :] >= cnt[:, None]
    assert np.all(a[pad] == 0.0) and np.all(b[pad] == 0.0)
    scale = float(np.abs(b).max())
    err = np.abs(a - b)
    print(f"k={k}: max |tc - fp32| {err.max():.3e}, mean {err.mean():.3e}, scale {scale:.3e}")
    assert err.max() <= 0.05 * scale
    assert err.mean() <= 0.01 * float(np.abs(b).mean()) + 1e-4
    # the FP32 path itself is the numpy restatement's forward
    feat = torch.empty((N, G.k, nn_oracle.F), dtype=torch.float32, device="cuda")
    G._check(G.lib.sgs_plan_features_device(G.h, __import__("ctypes").c_void_p(feat.data_ptr()), None))
    fh = feat.cpu().numpy()
    for g in rng.choice(N, 20, replace=False):
        n = int(cnt[g])
        if n:
            np.testing.assert_allclose(b[g, :n], nn_oracle.forward(params, fh[g], n), rtol=1e-4, atol=1e-5)
    G.close()


def _cg_iterations(K, c, x0, tol=1e-6, maxit=400):
    """Conjugate-gradient iterations (FP32 arithmetic) from x0 until the
    residual is below tol x |c|_inf."""
    K = K.astype(np.float32)
    c = c.astype(np.float32)
    x = x0.astype(np.float32).copy()
    r = c - K @ x
    p = r.copy()
    rr = float(r @ r)
    cn = float(np.abs(c).max())
    it = 0
    while float(np.abs(r).max()) > tol * cn and it < maxit:
        Ap = K @ p
        a = rr / float(p @ Ap)
        x += a * p
        r -= a * Ap
        rr2 = float(r @ r)
        p = r + (rr2 / rr) * p
        rr = rr2
        it += 1
    return it


def test_warm_start_gain_and_crossover(oracle_mod, geosgs_lib):
    """What the trained network gains over the method without it, on
    held-out systems: its predictions start closer to the exact weights than
    a zero start or an untrained network (relative L2 error of the start),
    and the conjugate-gradient iterations to 1e-6 from each start, beside
    those from starts of controlled accuracy (1e-1 .. 1e-4).  The curve is
    the crossover: an iterative solve from a prediction beats the FP32
    inverse (whose Gauss-Jordan cost is about 35 such iterations at k = 32..48)
    only for starts better than about 1e-2."""
    torch = pytest.importorskip("torch")
    feat, count, target = learned.generate(150000, seed=1, torch=torch, dims=(40, 40, 24))
    trained, _ = learned.train(feat, count, target, torch, epochs=20, batch=8192, lr=3e-3)
    untrained = learned.init_params(0)
    wl = workloads.small(dim=3, n=36, nz=16, k=32, vario="exp", ranges=(14.0, 7.0, 4.0),
                         rotation=geosgs.RotZ(20.0), nugget=0.08,
                         ball=geosgs.MetricBall((14.0, 7.0, 4.0), geosgs.RotZ(20.0)), precision="fp64", nreals=4)
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = geosgs.Plan(p, keep).prepare()
    w, _, st = G.weights()
    idx, cnt = G.neighbors()
    preds = {}
    for name, params in (("trained", trained), ("untrained", untrained)):
        G.set_network(params)
        out = torch.empty((G.N, G.k), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        G.predict_device(out.data_ptr(), tensor_cores=False)  # writes every entry; returns when done
        preds[name] = out.cpu().numpy().astype(np.float64)
    G.close()
    kr = np.nonzero((st == 0) & (cnt >= 8))[0]
    err = {name: np.median([np.linalg.norm(pr[g, :cnt[g]] - w[g, :cnt[g]]) / np.linalg.norm(w[g, :cnt[g]])
                            for g in kr]) for name, pr in preds.items()}
    err["zero"] = 1.0
    print("median relative start error: " + ", ".join(f"{k} {v:.3f}" for k, v in err.items()))
    assert err["trained"] < 0.9 * err["zero"] and err["trained"] < err["untrained"]
    # CG iterations from each start on a sample of the systems
    grid = wl.domain
    pts = grid.centroids()
    v = p.variogram
    rng = np.random.default_rng(0)
    sample = rng.choice(kr, 120, replace=False)
    its = {"zero": [], "trained": [], "1e-1": [], "1e-2": [], "1e-3": [], "1e-4": []}
    for g in sample:
        n = int(cnt[g])
        X = pts[idx[g, :n]]
        lags = (X[:, None, :] - X[None, :, :]).reshape(-1, 3)
        K = np.array([oracle_mod.covariance(v, 3, l) for l in lags]).reshape(n, n)
        c = np.array([oracle_mod.covariance(v, 3, l) for l in X - pts[g]])
        ws = np.linalg.solve(K, c)
        its["zero"].append(_cg_iterations(K, c, np.zeros(n)))
        its["trained"].append(_cg_iterations(K, c, preds["trained"][g, :n]))
        for e in ("1e-1", "1e-2", "1e-3", "1e-4"):
            x0 = ws + float(e) * np.linalg.norm(ws) * rng.standard_normal(n) / np.sqrt(n)
            its[e].append(_cg_iterations(K, c, x0))
    mean = {k: float(np.mean(x)) for k, x in its.items()}
    print("mean CG iterations to 1e-6: " + ", ".join(f"{k} {v:.1f}" for k, v in mean.items()))
    assert mean["trained"] <= mean["zero"] + 0.5
    assert mean["1e-1"] > mean["1e-2"] > mean["1e-3"] > mean["1e-4"]

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

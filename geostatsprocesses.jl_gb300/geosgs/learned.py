"""Learned warm start of the kriging weights: training-data generation,
training and use, on the GPU through the library's own kernels
(sgs_plan_features_device, sgs_nn_forward, sgs_nn_backward, sgs_nn_adam).

The training systems are the ones the method itself solves: a plan is
prepared for a workload, the features of every kriged node and the weights
its solver produced become one training example.  Device buffers are torch
tensors (plumbing only); all arithmetic runs in libgeosgs kernels.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _abi
from .model import (CartesianGrid, ExponentialVariogram, GaussianProcess, GaussianVariogram, MetricBall, RandomPath,
                    RotZ, SphericalVariogram)
from .plan import Plan
from .problem import build_problem
from .simulation import GPUSEQSIM

F, H = _abi.SGS_NN_FEATURES, 32
NPARAMS = _abi.SGS_NN_PARAMS


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initial parameters (float32, layout of csrc/learned.cu)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS)
    w1, b1 = 0, H * F
    w2a = b1 + H
    w2b = w2a + H * H
    b2 = w2b + H * H
    w3 = b2 + H
    b3 = w3 + H
    p[w1:b1] = rng.standard_normal(H * F) * math.sqrt(2.0 / F)
    p[w2a:w2b] = rng.standard_normal(H * H) * math.sqrt(1.0 / H)
    p[w2b:b2] = rng.standard_normal(H * H) * math.sqrt(1.0 / H)
    p[w3:b3] = rng.standard_normal(H) * math.sqrt(1.0 / H) * 0.1
    return p.astype(np.float32)


def random_training_workload(rng: np.random.Generator, dims=(48, 48, 32), k: int = 32, precision: str = "fp32"):
    """A 3D grid with a random variogram: family in {spherical, exponential,
    gaussian}, major range log-uniform in [5, 100] cells, anisotropy ratios in
    [1, 10], random azimuth, nugget fraction in [0, 0.2]; unconditional."""
    cls = [SphericalVariogram, ExponentialVariogram, GaussianVariogram][rng.integers(3)]
    r0 = float(np.exp(rng.uniform(np.log(5.0), np.log(100.0))))
    r1 = r0 / rng.uniform(1.0, 10.0)
    r2 = r0 / rng.uniform(1.0, 10.0)
    ball = MetricBall((r0, max(r1, 1.0), max(r2, 1.0)), RotZ(float(rng.uniform(0.0, 180.0))))
    nug = float(rng.uniform(0.0, 0.2))
    proc = GaussianProcess(cls(ball, sill=1.0, nugget=nug), 0.0)
    method = GPUSEQSIM(path=RandomPath(int(rng.integers(1 << 30))), maxneighbors=k, neighborhood=ball,
                       precision=precision)
    return proc, CartesianGrid(tuple(dims)), method


def plan_systems(plan: Plan, torch):
    """(features [S, k, F], counts [S], target weights [S, k]) of the kriged
    nodes of a prepared plan, as device tensors."""
    N, k = plan.N, plan.k
    feat = torch.empty((N, k, F), dtype=torch.float32, device="cuda")
    plan._check(plan.lib.sgs_plan_features_device(plan.h, C.c_void_p(feat.data_ptr()), None))
    w, _, st = plan.weights()
    _, cnt = plan.neighbors()
    keep = np.nonzero(st == _abi.SGS_NODE_KRIGED)[0]
    sel = torch.from_numpy(keep).cuda()
    return (feat.index_select(0, sel).contiguous(),
            torch.from_numpy(cnt[keep].astype(np.int32)).cuda(),
            torch.from_numpy(w[keep].astype(np.float32)).cuda())


def generate(nsystems: int, seed: int, torch, dims=(48, 48, 32), k: int = 32):
    """At least `nsystems` training systems from random workloads."""
    rng = np.random.default_rng(seed)
    parts = []
    total = 0
    while total < nsystems:
        proc, grid, method = random_training_workload(rng, dims, k)
        p, keep = build_problem(proc, grid, None, method)
        plan = Plan(p, keep).prepare()
        f, c, t = plan_systems(plan, torch)
        plan.close()
        parts.append((f, c, t))
        total += f.shape[0]
    return (torch.cat([p[0] for p in parts])[:nsystems], torch.cat([p[1] for p in parts])[:nsystems],
            torch.cat([p[2] for p in parts])[:nsystems])


def _check(lib, rc):
    if rc != _abi.SGS_OK:
        raise _abi.GeoSGSError(rc, lib.sgs_last_error(None).decode())


def loss_and_grad(params, feat, count, target, torch):
    """Summed per-system loss and gradient on the device (float32 tensors)."""
    lib = _abi.load_library()
    grad = torch.zeros(NPARAMS, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    k = feat.shape[1]
    _check(lib, lib.sgs_nn_backward(params.data_ptr(), feat.data_ptr(), count.data_ptr(), target.data_ptr(),
                                    feat.shape[0], k, grad.data_ptr(), loss.data_ptr(), None))
    torch.cuda.synchronize()
    return float(loss.item()), grad


def predict(params, feat, count, torch):
    lib = _abi.load_library()
    k = feat.shape[1]
    pred = torch.empty((feat.shape[0], k), dtype=torch.float32, device="cuda")
    _check(lib, lib.sgs_nn_forward(params.data_ptr(), feat.data_ptr(), count.data_ptr(), feat.shape[0], k,
                                   pred.data_ptr(), None))
    torch.cuda.synchronize()
    return pred


def train(feat, count, target, torch, epochs: int = 4, batch: int = 16384, lr: float = 3e-3, seed: int = 0,
          log=None):
    """Adam on mini-batches with the library's backward and Adam kernels.
    Returns (params as float32 numpy, per-epoch mean loss)."""
    lib = _abi.load_library()
    params = torch.from_numpy(init_params(seed)).cuda()
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    grad = torch.zeros_like(params)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    S, k = feat.shape[0], feat.shape[1]
    gen = torch.Generator(device="cpu").manual_seed(seed)
    step = 0
    history = []
    for ep in range(epochs):
        perm = torch.randperm(S, generator=gen).cuda()
        loss.zero_()
        for b0 in range(0, S, batch):
            idx = perm[b0:b0 + batch]
            fb, cb, tb = feat.index_select(0, idx), count.index_select(0, idx), target.index_select(0, idx)
            grad.zero_()
            _check(lib, lib.sgs_nn_backward(params.data_ptr(), fb.data_ptr(), cb.data_ptr(), tb.data_ptr(),
                                            fb.shape[0], k, grad.data_ptr(), loss.data_ptr(), None))
            step += 1
            _check(lib, lib.sgs_nn_adam(params.data_ptr(), grad.data_ptr(), m.data_ptr(), v.data_ptr(), step,
                                        C.c_float(lr), C.c_float(1.0 / fb.shape[0]), None))
        torch.cuda.synchronize()
        history.append(float(loss.item()) / S)
        if log:
            log(f"epoch {ep}: mean loss {history[-1]:.3e}")
    return params.cpu().numpy(), history

"""Full-depth parity at the benchmark configurations: every node of the path,
not a prefix or a sample.

A value's error can grow along the path: a node's kriged mean sums the
values of earlier nodes, each carrying its own error, so the deepest levels
are where a precision problem would show.  These tests run the FP64 oracle
over every node of

  * the 200x200x100 conditional anisotropic grid (4 M nodes, 5,000 data,
    k = 48), 16 realizations;
  * the 256^3 unconditional anisotropic grid (16.8 M nodes, k = 32),
    8 realizations;
  * all 1,000 domains of the uneven batch (354 M nodes, k 8-48, 0-500 data),
    8 realizations;

and compare the CUDA path through the C ABI: neighbour indices and counts
bit-exact for every node, node status identical, weights and conditional
standard deviations within 1e-6 absolute, values within 1e-6 relative
(rel = max |v_gpu - v_oracle| / max(|v_oracle|, 1) per element), for the
plain FP64 path, the FP32 + refinement path and the FP32 path warm-started by
a trained network.  Each comparison prints one FULLDEPTH line with the
measured maxima, by path decile for the values."""
import concurrent.futures as cf
import time

import numpy as np
import pytest

import geosgs
from geosgs import _abi, learned, workloads

pytestmark = pytest.mark.gpu

VALUE_TOL = 1e-6
WEIGHT_TOL = 1e-6
SIGMA_TOL = 1e-6


def rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1.0)


def report(name, **kv):
    print("FULLDEPTH " + name + " " + " ".join(f"{k}={v:.3e}" if isinstance(v, float) else f"{k}={v}"
                                               for k, v in kv.items()), flush=True)


@pytest.fixture(scope="module")
def network(geosgs_lib):
    """A warm-start network trained on systems the method generates (the
    bench's recipe: 600,000 systems from random 3D workloads, 8 epochs)."""
    torch = pytest.importorskip("torch")
    feat, count, target = learned.generate(600_000, seed=11, torch=torch, dims=(48, 48, 32))
    params, hist = learned.train(feat, count, target, torch, epochs=8, batch=16384, lr=3e-3)
    del feat, count, target
    torch.cuda.empty_cache()
    return params


def _oracle(oracle_mod, wl, nreals, zseed):
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    t0 = time.perf_counter()
    O = oracle_mod.OraclePlan(p, keep).prepare()
    z = np.random.default_rng(zseed).standard_normal((nreals, O.N))
    vo = O.simulate(nreals, z)
    io, co = O.neighbors()
    wo, so, sto = O.weights()
    print(f"oracle {wl.name}: {time.perf_counter() - t0:.1f} s", flush=True)
    return dict(p=p, keep=keep, N=O.N, z=z, vo=vo, io=io, co=co, wo=wo, so=so, sto=sto)


def _check_plan(name, wl, ref, nreals, precision, params=None):
    wl.method.precision = precision
    wl.method.warm_start = params is not None
    p, keep = geosgs.build_problem(wl.process, wl.domain, wl.data, wl.method)
    G = geosgs.Plan(p, keep)
    if params is not None:
        G.set_network(params)
    G.prepare()
    ig, cg = G.neighbors()
    assert np.array_equal(cg, ref["co"]), name
    assert np.array_equal(ig, ref["io"]), name
    del ig, cg
    wg, sg, stg = G.weights()
    assert np.array_equal(stg, ref["sto"]), name
    werr = float(np.max(np.abs(wg - ref["wo"])))
    serr = float(np.max(np.abs(sg - ref["so"])))
    del wg, sg
    vg = G.simulate(nreals, ref["z"])
    info = G.info()
    G.close()
    e = rel(vg, ref["vo"]).max(axis=0)  # per node
    del vg
    path = wl.method.path.permutation(ref["N"])
    dec = [float(e[path[int(ref["N"] * i / 10):int(ref["N"] * (i + 1) / 10)]].max()) for i in range(10)]
    report(name, nodes=ref["N"], reals=nreals, weights=werr, sigma=serr, values=float(e.max()),
           first_decile=dec[0], last_decile=dec[-1], values_fp64=int(info.values_fp64),
           weight_l1_max=float(info.weight_l1_max), warm=int(info.n_warm_accepted),
           fp64_fallback=int(info.n_fp64_fallback))
    print("  values by path decile: " + " ".join(f"{d:.2e}" for d in dec), flush=True)
    assert werr <= WEIGHT_TOL, (name, werr)
    assert serr <= SIGMA_TOL, (name, serr)
    assert float(e.max()) <= VALUE_TOL, (name, float(e.max()))


@pytest.mark.parametrize("config", ["c3", "c4"])
def test_full_depth_plans(config, oracle_mod, network):
    if config == "c3":
        wl, R = workloads.c3(precision="fp32", nreals=16), 16
    else:
        wl, R = workloads.c4(precision="fp32", nreals=8), 8
    ref = _oracle(oracle_mod, wl, R, zseed=31)
    _check_plan(f"{wl.name} fp64", wl, ref, R, "fp64")
    _check_plan(f"{wl.name} fp32", wl, ref, R, "fp32")
    _check_plan(f"{wl.name} learned+fp32", wl, ref, R, "fp32", params=network)


def test_full_depth_all_c5_domains(oracle_mod, geosgs_lib):
    """Every node of every one of the 1,000 domains, 8 realizations.  The
    domains run as batches of 100 (host memory for the given draws and the
    FP64 output stays near 5 GB); a domain's results do not depend on the
    other domains of its batch, apart from the batch-wide value precision,
    which the comparison reports."""
    bw = workloads.c5("fp32", nreals=8, ndomains=1000)
    R = 8
    chunk = 100
    worst = dict(values=0.0, weights=0.0, sigma=0.0)
    nodes = 0
    t0 = time.perf_counter()

    def oracle_domain(args):
        p, keep, z = args
        O = oracle_mod.OraclePlan(p, keep).prepare(nthreads=2)
        io, co = O.neighbors()
        wo, so, sto = O.weights()
        return io, co, wo, so, sto, O.simulate(R, z, nthreads=2)

    with cf.ThreadPoolExecutor(max_workers=8) as pool:
        for c0 in range(0, len(bw.items), chunk):
            items = bw.items[c0:c0 + chunk]
            probs = [geosgs.build_problem(w.process, w.domain, w.data, w.method) for w in items]
            B = geosgs.Batch(probs).prepare()
            zs = [np.random.default_rng(7000 + c0 + d).standard_normal((R, int(n))) for d, n in enumerate(B.sizes)]
            vals = B.simulate(R, z=zs)
            fp64 = B.values_fp64()
            # largest domains first, so the chunk does not wait on one late straggler
            futs = {d: pool.submit(oracle_domain, (probs[d][0], probs[d][1], zs[d]))
                    for d in sorted(range(len(probs)), key=lambda d: -int(B.sizes[d]))}
            for d in range(len(probs)):
                io, co, wo, so, sto, vo = futs[d].result()
                ig, cg = B.neighbors(d)
                assert np.array_equal(cg, co) and np.array_equal(ig, io), f"domain {c0 + d}"
                wg, sg, stg = B.weights(d)
                assert np.array_equal(stg, sto), f"domain {c0 + d}"
                worst["weights"] = max(worst["weights"], float(np.max(np.abs(wg - wo))) if wo.size else 0.0)
                worst["sigma"] = max(worst["sigma"], float(np.max(np.abs(sg - so))))
                worst["values"] = max(worst["values"], float(rel(vals[d], vo).max()))
                nodes += vo.shape[1]
            report(f"c5 domains {c0}-{c0 + len(items) - 1}", values_fp64=int(fp64),
                   domains_fp64=int(B.info().domains_fp64), **worst)
            B.close()
    report("c5_batch_1000_domains all", nodes=nodes, reals=R, seconds=time.perf_counter() - t0, **worst)
    assert nodes == bw.nodes()
    assert worst["weights"] <= WEIGHT_TOL
    assert worst["sigma"] <= SIGMA_TOL
    assert worst["values"] <= VALUE_TOL

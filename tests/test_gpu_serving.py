"""Uneven batches and continuous batching (geopvi_gb300.scheduler) on the GPU.

Each request's result must be the same alone and in the mix: the server runs
requests of different grids, acquisitions and time axes concurrently on
several streams or fused into one call, merges queued requests of one
inversion into one batch and picks full storage or checkpoints by its HBM
budget -- none of which may change a single bit of any result.
"""
import os
import time

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.dirname(cases.__file__)
NAMES = ["fwi_o8", "fwi_o8_nti2", "fwi_ragged", "fwi_o12"]


def load(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def models(z, n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([z["start"] + rng.uniform(-30, 30, z["start"].shape).astype(np.float32) for _ in range(n)])


def alone(p, vel, obs):
    from geopvi_gb300.engine import Fwi2dEngine
    eng = Fwi2dEngine(p, device="cuda:0", graph=False)
    r = eng.run(torch.from_numpy(vel).cuda(), torch.from_numpy(obs).cuda(), want_syn=True)
    torch.cuda.synchronize()
    return r.misfit.cpu().numpy().copy(), r.grad.cpu().numpy().copy(), r.syn.cpu().numpy().copy()


@pytest.mark.parametrize("budget,at_once", [(150 << 30, False), (6 << 20, False), (150 << 30, True),
                                             (2 << 20, True)])
def test_uneven_batch_matches_each_job_alone(engine_lib, cuda, budget, at_once):
    """at_once: every job reaches the dispatcher together, so the inversions
    share one fused call (in waves, when the budget is small)."""
    from geopvi_gb300.scheduler import FwiServer
    jobs = []
    for k, name in enumerate(NAMES):
        z = load(name)
        p = cases.params_from_npz(z)
        vel = models(z, 2 + k, seed=k)
        jobs.append((name, p, vel, z["obs"]))
    expect = {name: alone(p, vel, obs) for name, p, vel, obs in jobs}
    with FwiServer(device="cuda:0", hbm_budget=budget, streams=3) as srv:
        for name, p, vel, obs in jobs:
            srv.register(name, p, obs)
        if at_once:
            futs = dict(zip([j[0] for j in jobs], srv.submit_many([(name, vel) for name, _, vel, _ in jobs],
                                                                  want_syn=True)))
        else:
            futs = {name: srv.submit(name, vel, want_syn=True) for name, p, vel, obs in jobs}
        res = {name: f.result(timeout=300) for name, f in futs.items()}
    for name, _, _, _ in jobs:
        m, g, s = expect[name]
        assert np.array_equal(res[name]["misfit"].numpy(), m), name
        assert np.array_equal(res[name]["grad"].numpy(), g), name
        assert np.array_equal(res[name]["syn"].numpy(), s), name


def test_continuous_batching_same_alone_and_in_the_mix(engine_lib, cuda):
    from geopvi_gb300.scheduler import FwiServer, latency_summary
    za, zb = load("fwi_o8"), load("fwi_o10_nti3")
    pa, pb = cases.params_from_npz(za), cases.params_from_npz(zb)
    reqs = [("a", models(za, n, 10 + i)) if i % 2 == 0 else ("b", models(zb, n, 10 + i))
            for i, n in enumerate([3, 2, 4, 1, 2, 3, 1, 2])]
    with FwiServer(device="cuda:0", streams=2) as srv:
        srv.register("a", pa, za["obs"])
        srv.register("b", pb, zb["obs"])
        futs = []
        for name, vel in reqs:  # staggered arrivals while earlier batches run
            futs.append(srv.submit(name, vel))
            time.sleep(0.003)
        out = [f.result(timeout=300) for f in futs]
        stats = latency_summary(srv.completed)
    assert stats["count"] == len(reqs)
    for (name, vel), res in zip(reqs, out):
        p, z = (pa, za) if name == "a" else (pb, zb)
        m, g, _ = alone(p, vel, z["obs"])
        assert np.array_equal(res["misfit"].numpy(), m)
        assert np.array_equal(res["grad"].numpy(), g)

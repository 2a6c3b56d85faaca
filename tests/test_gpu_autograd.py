"""The autograd path of the 300 x 600 batch (log_prob -> backward) against Posterior.fwi.

ForwardModel (posterior.py:8-24) saves the solver's gradient and scales it in
backward by the incoming per-sample gradient; log_prob is -loss/sigma^2 plus
the prior (posterior.py:151-166).  Here the autograd path runs with sqrt(nt)
checkpoints and Posterior.fwi with the whole forward field stored, on two
shots of the full 300 x 600, nt 4000, dt 0.8 ms geometry: the backward
gradient must equal -(1/sigma^2) times fwi's gradient bit for bit (the
recomputed segments reproduce the stored field exactly, and the prior is
uniform), and the log posterior must equal -loss/sigma^2 plus the prior's
constant.
"""
import configparser
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def fwi_config(p):
    cfg = configparser.ConfigParser()
    cfg["FWI"] = {"nx": str(p.nx), "nz": str(p.nz), "pml": str(p.pml0), "Lc": str(p.Lc),
                  "laplace_slover": str(p.laplace_solver), "ns": str(p.ns), "nt": str(p.nt), "ds": str(p.ds),
                  "ns0": str(p.ns0), "depths": str(p.depths), "depthr": str(p.depthr), "nr": str(p.nr),
                  "dr": str(p.dr), "nr0": str(p.nr0), "nt_interval": str(p.nt_interval), "dx": repr(p.dx),
                  "dz": repr(p.dz), "dt": repr(p.dt), "f0": repr(p.f0)}
    return cfg


def test_checkpointed_autograd_gradient_equals_fwi(engine_lib, cuda, tmp_path):
    from geopvi_gb300 import vi, workloads
    from geopvi_gb300.engine import Fwi2dEngine
    from geopvi_gb300.posterior import Posterior

    w = workloads.cfg3(nsamples=2)
    p = w.params.replace(ns=2)
    dev = torch.device("cuda:0")
    eng = Fwi2dEngine(p, device=dev, graph=False)
    zeros = torch.zeros(p.data_len, dtype=torch.float32, device=dev)
    obs = eng.run(torch.from_numpy(w.truth).to(dev).unsqueeze(0), zeros, forward_only=True).syn[0].cpu().numpy()
    del eng
    sigma = 0.01 * float(np.abs(obs).max())
    prior = vi.Uniform(lower=np.full(p.ncell, 1400.0), upper=np.full(p.ncell, 5000.0))
    cfg = fwi_config(p)

    ck = Posterior(obs, cfg, sigma=sigma, log_prior=prior.log_prob, paramfile=str(tmp_path / "a.txt"),
                   device=dev, graph=False, checkpoint=True)
    x = torch.from_numpy(w.samples.astype(np.float64)).requires_grad_(True)
    logp = ck.log_prob(x)
    logp.sum().backward()
    assert ck.engine.status() == 0
    g_auto = x.grad.clone()
    del ck
    torch.cuda.empty_cache()

    full = Posterior(obs, cfg, sigma=sigma, log_prior=prior.log_prob, paramfile=str(tmp_path / "b.txt"),
                     device=dev, graph=False)
    loss, grad = full.fwi(w.samples.astype(np.float64))
    assert full.engine.status() == 0
    expected = (-1.0 / sigma ** 2) * torch.from_numpy(grad)
    assert torch.equal(g_auto, expected), float((g_auto - expected).abs().max())
    logp_expected = -torch.from_numpy(loss) / sigma ** 2 + prior.log_prob(x.detach())
    assert torch.equal(logp.detach(), logp_expected)
    assert np.abs(grad).max() > 0

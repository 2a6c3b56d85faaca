"""3-D engine on the GPU against the 3-D oracle: data and gradient bit for bit.

Cases cover 8th, 12th and 6th order; grids whose sides are not multiples of
the 32 x 8 tile or the 32-plane z chunk; duplicate receiver cells (injected
in receiver order); stored steps every 2nd step; checkpointed and multi-wave
runs (same values as one wave with the whole field stored); and the
reference-compatible Posterior.
"""
import configparser
from types import SimpleNamespace

import numpy as np
import pytest
import torch

from geopvi_gb300 import fwi3d
from oracle import oracle3d as O

pytestmark = pytest.mark.gpu


def ricker(nt, dt, f0):
    t = np.arange(nt) * dt - 1.0 / f0
    a = (np.pi * f0 * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def make_case(nx, ny, nz, nt, Lc, pml0, nti, ns, nr, nsamples, seed):
    p = fwi3d.Fwi3dParams(nx=nx, ny=ny, nz=nz, nt=nt, dt=1e-3, dx=10.0, dy=12.0, dz=9.0, pml0=pml0, Lc=Lc,
                          nt_interval=nti, ns=ns, nr=nr)
    rng = np.random.default_rng(seed)
    src = np.stack([rng.integers(0, nx, ns), rng.integers(0, ny, ns), rng.integers(0, min(3, nz), ns)], 1)
    rec = np.stack([rng.integers(0, nx, nr), rng.integers(0, ny, nr), rng.integers(0, min(2, nz), nr)], 1)
    rec[nr // 2] = rec[1]  # a shared receiver cell
    wav = ricker(nt, p.dt, 20.0)
    truth = (1800 + 600 * rng.random((ny, nx, nz))).astype(np.float32)
    vel = np.clip(truth[None] + 150 * rng.standard_normal((nsamples, ny, nx, nz)), 1500, 2600).astype(np.float32)
    obs, _, _ = O.run(p, src, rec, wav, truth)
    return SimpleNamespace(p=p, src=src, rec=rec, wav=wav, vel=vel.reshape(nsamples, -1), obs=obs)


CASES = {
    "o8": dict(nx=12, ny=11, nz=9, nt=120, Lc=4, pml0=5, nti=1, ns=2, nr=14, nsamples=2, seed=0),
    "o12_ragged": dict(nx=37, ny=9, nz=40, nt=90, Lc=6, pml0=3, nti=2, ns=2, nr=9, nsamples=2, seed=1),
    "o6": dict(nx=10, ny=14, nz=11, nt=100, Lc=3, pml0=4, nti=1, ns=3, nr=6, nsamples=1, seed=2),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    return request.param, make_case(**CASES[request.param])


def oracle_all(c):
    out = [O.run(c.p, c.src, c.rec, c.wav, v, c.obs, grad=True) for v in c.vel]
    return (np.stack([o[0] for o in out]), np.stack([o[1] for o in out]), np.array([o[2] for o in out]))


def test_data_and_gradient_bit_exact(engine_lib, cuda, case):
    name, c = case
    syn_o, grad_o, mis_o = oracle_all(c)
    eng = fwi3d.Fwi3dEngine(c.p, c.src, c.rec, c.wav, device=cuda)
    r = eng.run(torch.from_numpy(c.vel).to(cuda), torch.from_numpy(c.obs).to(cuda), want_syn=True)
    torch.cuda.synchronize()
    assert np.array_equal(r.syn.cpu().numpy(), syn_o), name
    assert np.array_equal(r.grad.cpu().numpy(), grad_o), name
    assert np.allclose(r.misfit.cpu().numpy(), mis_o, rtol=1e-12, atol=0), name
    assert np.abs(grad_o).max() > 0 and r.launches > 2 * c.p.nt


def test_forward_only_matches(engine_lib, cuda):
    c = make_case(**CASES["o8"])
    eng = fwi3d.Fwi3dEngine(c.p, c.src, c.rec, c.wav, device=cuda)
    r = eng.run(torch.from_numpy(c.vel).to(cuda), forward_only=True)
    syn_o = np.stack([O.run(c.p, c.src, c.rec, c.wav, v)[0] for v in c.vel])
    assert np.array_equal(r.syn.cpu().numpy(), syn_o) and r.grad is None


def test_edge_geometries(engine_lib, cuda):
    """One shot and one receiver at opposite model corners, a one-cell absorbing
    strip, 10th order, stored steps every 3rd of a 101-step run (also
    checkpointed), and every receiver of another case in one cell."""
    p = fwi3d.Fwi3dParams(nx=9, ny=7, nz=8, nt=101, dt=1e-3, dx=10.0, dy=10.0, dz=10.0, pml0=1, Lc=5,
                          nt_interval=3, ns=1, nr=1)
    src, rec = np.array([[0, 0, 0]]), np.array([[8, 6, 7]])
    wav = ricker(p.nt, p.dt, 25.0)
    rng = np.random.default_rng(9)
    truth = (1800 + 500 * rng.random(p.ncell)).astype(np.float32)
    vel = (truth + rng.uniform(-80, 80, (2, p.ncell))).astype(np.float32)
    obs = O.run(p, src, rec, wav, truth)[0]
    outs = [O.run(p, src, rec, wav, v, obs, grad=True) for v in vel]
    for ck in (False, True):
        r = fwi3d.Fwi3dEngine(p, src, rec, wav, device=cuda, checkpoint=ck).run(
            torch.from_numpy(vel).to(cuda), torch.from_numpy(obs).to(cuda), want_syn=True)
        assert np.array_equal(r.syn.cpu().numpy(), np.stack([o[0] for o in outs]))
        assert np.array_equal(r.grad.cpu().numpy(), np.stack([o[1] for o in outs]))
        assert np.abs(outs[0][1]).max() > 0
    # every receiver in one cell: injected one after another in receiver order
    c = make_case(**CASES["o8"])
    rec_same = np.repeat(c.rec[:1], 5, axis=0)
    q = c.p.replace(nr=5)
    obs5 = O.run(q, c.src, rec_same, c.wav, c.vel[0] * 0 + 1900)[0]
    obs5 = obs5 + np.linspace(0, 1e-3, 5, dtype=np.float32)  # distinct residuals per receiver
    ref = O.run(q, c.src, rec_same, c.wav, c.vel[0], obs5, grad=True)
    r = fwi3d.Fwi3dEngine(q, c.src, rec_same, c.wav, device=cuda).run(
        torch.from_numpy(c.vel[:1]).to(cuda), torch.from_numpy(np.ascontiguousarray(obs5)).to(cuda), want_syn=True)
    assert np.array_equal(r.syn[0].cpu().numpy(), ref[0])
    assert np.array_equal(r.grad[0].cpu().numpy(), ref[1])


@pytest.mark.parametrize("checkpoint,resident", [(True, None), (False, 1), (True, 3)])
def test_checkpoint_and_waves_identical(engine_lib, cuda, checkpoint, resident):
    c = make_case(**{**CASES["o8"], "nt": 150, "nsamples": 3})
    vel = torch.from_numpy(c.vel).to(cuda)
    obs = torch.from_numpy(c.obs).to(cuda)
    base = fwi3d.Fwi3dEngine(c.p, c.src, c.rec, c.wav, device=cuda).run(vel, obs, want_syn=True)
    other = fwi3d.Fwi3dEngine(c.p, c.src, c.rec, c.wav, device=cuda, checkpoint=checkpoint,
                              max_resident=resident).run(vel, obs, want_syn=True)
    assert torch.equal(base.syn, other.syn)
    assert torch.equal(base.grad, other.grad)
    assert torch.equal(base.misfit, other.misfit)


def test_posterior_drop_in(engine_lib, cuda, tmp_path):
    """The reference's Posterior(args, config, mask, log_prior): the same random
    shot subset for the same seed, 0.5 * loss * scale and grad * scale, and
    autograd through log_prob on the device."""
    c = make_case(**{**CASES["o8"], "ns": 5, "nsamples": 3})
    nshots = 5
    shots = c.src
    data = np.stack([O.run(c.p.replace(ns=1), shots[i:i + 1], c.rec, c.wav,
                           (1800 + 0 * c.vel[0]).astype(np.float32))[0][0] for i in range(nshots)])
    np.save(tmp_path / "source.npy", shots)
    np.save(tmp_path / "data.npy", data)
    np.save(tmp_path / "rec.npy", c.rec)
    np.save(tmp_path / "wavelet.npy", c.wav)
    cfg = configparser.ConfigParser()
    cfg["FWI"] = dict(nx=str(c.p.nx), ny=str(c.p.ny), nz=str(c.p.nz), dx="10", dy="12", dz="9", dt="0.001",
                      pml=str(c.p.pml0), Lc="4", shot_batch="2", vel_fixed="1500",
                      recfile=str(tmp_path / "rec.npy"), waveletfile=str(tmp_path / "wavelet.npy"))
    cfg["path"] = dict(inpath=str(tmp_path), outpath=str(tmp_path), srcfile=str(tmp_path / "source.npy"),
                       datafile=str(tmp_path / "data.npy"))
    mask = np.ones((c.p.ny, c.p.nx, c.p.nz), bool)
    mask[:, :, 0] = False  # top layer fixed
    mask = mask.ravel()
    post = fwi3d.Posterior(SimpleNamespace(sigma=0.5), cfg, mask=mask, log_prior=lambda x: -0.0 * x.sum(1),
                           device=cuda)
    x = torch.from_numpy(c.vel[:, mask].astype(np.float64)).to(cuda).requires_grad_(True)
    np.random.seed(11)
    logp = post.log_prob(x)
    logp.sum().backward()
    np.random.seed(11)
    sl = np.sort(np.random.choice(nshots, size=2, replace=False))
    full = np.full((3, mask.size), 1500.0, np.float32)
    full[:, mask] = c.vel[:, mask]
    sub = c.p.replace(ns=2)
    ref = [O.run(sub, shots[sl], c.rec, c.wav, v, data[sl], grad=True) for v in full]
    scale = nshots / 2
    loss = np.array([r[2] for r in ref]) * scale
    grad = np.stack([r[1][mask] for r in ref]).astype(np.float64) * scale
    assert logp.is_cuda and x.grad.is_cuda
    assert np.allclose(-logp.detach().cpu().numpy() * 0.25, loss, rtol=1e-10)
    assert np.array_equal(x.grad.cpu().numpy(), -grad / 0.25)
    # a second call draws another subset; the engine and its workspace are reused
    np.random.seed(5)
    sl2 = np.sort(np.random.choice(nshots, size=2, replace=False))
    assert not np.array_equal(sl2, sl)
    np.random.seed(5)
    l2, g2 = post.fwi3d(x.detach())
    ref2 = [O.run(sub, shots[sl2], c.rec, c.wav, v, data[sl2], grad=True) for v in full]
    assert np.allclose(l2.cpu().numpy(), np.array([r[2] for r in ref2]) * scale, rtol=1e-10)
    assert np.array_equal(g2.cpu().numpy(), np.stack([r[1][mask] for r in ref2]).astype(np.float64) * scale)

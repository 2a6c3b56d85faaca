"""GPU exact discrete adjoint (GB_FWI2D_EXACT_GRADIENT) against the oracle.

The FP64 oracle's exact gradient is itself checked against central finite
differences with h = 1e-2 m/s on 50 random cells plus the model's corners
and edges (test_oracle_exact_adjoint.py).  A central difference in FP32 at
that h is dominated by rounding (the FP32 forward, bit-identical to the
engine's, gives ~90% error at h = 1e-2 on the 8th-order case), so on the GPU
the bars are:
  * gradient: relative L2 <= 1e-4 against the FP64 oracle's exact gradient;
  * a Taylor test of the engine's own misfit along its own gradient,
    J(v + h d) - J(v - h d) vs g . (2 h d) with d = g / max|g| and h = 2 m/s,
    relative error <= 2e-3 (FP32 rounding of J is the floor);
  * checkpointed, plain and multi-wave runs bit-identical to the batched one.
"""
import os

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.dirname(cases.__file__)
GRAD_TOL = 1e-4
TAYLOR_H = 2.0
TAYLOR_TOL = 2e-3
FWI_CASES = sorted(n for n, c in cases.SMALL.items() if c["run_fwi"])


def load(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oparams(O, p):
    return O.Params(**cases.params_to_dict(p))


def misfit32(O, op, vel, obs):
    """The engine's misfit: float residual of the FP32 forward, squares summed in double."""
    syn = O.forward_f32(op, np.asarray(vel, np.float32))
    r = (syn - np.asarray(obs, np.float32)).astype(np.float64)
    return 0.5 * float(np.sum(r * r))


def engine_for(p, **kw):
    from geopvi_gb300.engine import Fwi2dEngine
    return Fwi2dEngine(p, device="cuda:0", **kw)


def run_exact(eng, vel, obs, **kw):
    v = torch.from_numpy(np.ascontiguousarray(np.atleast_2d(vel), dtype=np.float32)).cuda()
    o = torch.from_numpy(np.ascontiguousarray(obs, dtype=np.float32)).cuda()
    r = eng.run(v, o, exact=True, **kw)
    torch.cuda.synchronize()
    assert eng.status() == 0
    return r.misfit.cpu().numpy().copy(), r.grad.cpu().numpy().copy()


@pytest.mark.parametrize("name", FWI_CASES)
def test_exact_gradient_matches_oracle(engine_lib, cuda, oracle, name):
    z = load(name)
    p = cases.params_from_npz(z)
    eng = engine_for(p, graph=False)
    J, g = run_exact(eng, z["start"], z["obs"])
    Jo, go = oracle.exact_grad_f64(oparams(oracle, p), z["start"].astype(np.float64), z["obs"].astype(np.float64))
    e = rel(g[0], go)
    assert e <= GRAD_TOL, f"exact gradient rel L2 {e:.3e} against the FP64 oracle"
    assert abs(J[0] - float(z["misfit"])) <= 1e-5 * abs(float(z["misfit"]))
    # same misfit as the reference-gradient mode, bit for bit (same forward)
    v = torch.from_numpy(np.atleast_2d(z["start"]).astype(np.float32)).cuda()
    o = torch.from_numpy(z["obs"].astype(np.float32)).cuda()
    assert eng.run(v, o).misfit.cpu().numpy()[0] == J[0]


def test_exact_gradient_batch_of_samples(engine_lib, cuda, oracle):
    """Several samples x shots in one launch sequence; each sample's gradient
    is its own (no cross-talk between solves of a wave)."""
    z = load("fwi_o8")
    p = cases.params_from_npz(z)
    rng = np.random.default_rng(4)
    # not the true model: its FP32 residual is exactly zero, the FP64 oracle's is not
    vel = np.stack([z["start"], 0.5 * (z["start"] + z["truth"]),
                    z["start"] + rng.uniform(-40, 40, p.ncell)]).astype(np.float32)
    eng = engine_for(p, graph=True)
    J, g = run_exact(eng, vel, z["obs"])
    op = oparams(oracle, p)
    for s in range(3):
        Jo, go = oracle.exact_grad_f64(op, vel[s].astype(np.float64), z["obs"].astype(np.float64))
        assert rel(g[s], go) <= GRAD_TOL, s
        assert J[s] == pytest.approx(misfit32(oracle, op, vel[s], z["obs"]), rel=1e-12), s


@pytest.mark.parametrize("name", ["fwi_o8", "fwi_ragged", "fwi_pml1"])
def test_taylor_along_own_gradient(engine_lib, cuda, name):
    z = load(name)
    p = cases.params_from_npz(z)
    eng = engine_for(p, graph=False)
    v0 = z["start"].astype(np.float32)
    _, g = run_exact(eng, v0, z["obs"])
    g = g[0].astype(np.float64)
    d = g / np.max(np.abs(g))
    vp = (v0 + TAYLOR_H * d).astype(np.float32)
    vm = (v0 - TAYLOR_H * d).astype(np.float32)
    Jpm, _ = run_exact(eng, np.stack([vp, vm]), z["obs"])
    fd = Jpm[0] - Jpm[1]
    pred = float(g @ (vp.astype(np.float64) - vm.astype(np.float64)))
    assert abs(fd - pred) <= TAYLOR_TOL * abs(pred), (fd, pred)


def test_checkpointed_plain_and_waves_identical(engine_lib, cuda):
    z = load("fwi_o8_nti2")  # nt = 301: the last segment is short
    p = cases.params_from_npz(z)
    vel = np.stack([z["start"], z["truth"]]).astype(np.float32)
    J0, g0 = run_exact(engine_for(p, graph=False), vel, z["obs"])
    for kw in (dict(checkpoint=True), dict(plain=True), dict(max_resident=4), dict(checkpoint=True, max_resident=5),
               dict(graph=True)):
        J, g = run_exact(engine_for(p, **kw), vel, z["obs"])
        assert np.array_equal(g, g0), kw
        assert np.array_equal(J, J0), kw


def test_posterior_exact_gradient(engine_lib, cuda, oracle, tmp_path):
    """Posterior(gradient='exact'): loss and d loss / d x on the free cells."""
    import configparser
    from geopvi_gb300.posterior import Posterior
    z = load("fwi_o8")
    p = cases.params_from_npz(z)
    cfg = configparser.ConfigParser()
    cfg["FWI"] = {k: str(v) for k, v in cases.params_to_dict(p).items()}
    cfg["FWI"]["laplace_slover"] = cfg["FWI"].pop("laplace_solver")
    cfg["FWI"]["pml"] = cfg["FWI"].pop("pml0")
    mask = np.ones(p.ncell, bool)
    mask[: 2 * p.nx] = False  # two fixed rows
    vel = z["start"].astype(np.float64)
    vfix = 1950.0
    vel[~mask] = vfix
    post = Posterior(z["obs"], cfg, vel_fixed=vfix, mask=mask, paramfile=str(tmp_path / "p.txt"),
                     gradient="exact")
    loss, grad = post.fwi(vel[mask][None, :])
    Jo, go = oracle.exact_grad_f64(oparams(oracle, p), vel.astype(np.float32).astype(np.float64),
                                   z["obs"].astype(np.float64))
    assert rel(grad[0], go[mask]) <= GRAD_TOL
    assert loss[0] == pytest.approx(misfit32(oracle, oparams(oracle, p), vel, z["obs"]), rel=1e-12)
    with pytest.raises(ValueError):
        Posterior(z["obs"], cfg, mask=mask, paramfile=str(tmp_path / "q.txt"), gradient="adjoint")


def test_exact_with_imaging_is_rejected(engine_lib, cuda):
    z = load("fwi_o8")
    p = cases.params_from_npz(z)
    eng = engine_for(p, graph=False)
    v = torch.from_numpy(np.atleast_2d(z["start"]).astype(np.float32)).cuda()
    o = torch.from_numpy(z["obs"].astype(np.float32)).cuda()
    with pytest.raises(ValueError):
        eng.run(v, o, exact=True, imaging=True)

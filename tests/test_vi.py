"""geopvi_gb300.vi against golden vectors from the reference's own modules.

tests/golden/make_vi_golden.py ran the reference's flows.py, models.py,
prior.py and utils.py (imported from the reference source tree) and stored
their outputs; here the device-resident restatement reproduces them on the
CPU (to double round-off: the structured kernel sums its bands in another
order), and on the GPU a full VI iteration through Posterior stays on the
device.
"""
import os

import numpy as np
import pytest
import torch

import cases
from geopvi_gb300 import vi

GOLDEN = os.path.join(os.path.dirname(cases.__file__), "vi_golden.npz")
TOL = 1e-12


@pytest.fixture(scope="module")
def g():
    return np.load(GOLDEN)


@pytest.fixture(autouse=True)
def float64_default():
    old = torch.get_default_dtype()
    torch.set_default_dtype(torch.float64)
    yield
    torch.set_default_dtype(old)


def close(a, b, tol=TOL):
    a = np.asarray(a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() <= tol * max(1.0, np.abs(b).max())


def test_linear_flows(g):
    dim = g["x"].shape[1]
    x = torch.from_numpy(g["x"])
    f = vi.Linear(dim, kernel="diagonal", param=g["diag_param"])
    z, ld = f(x)
    assert close(z, g["diag_z"]) and close(ld, g["diag_ld"])
    xi, li = f.inverse(z)
    assert close(xi, g["diag_xi"]) and close(li, g["diag_li"])
    f = vi.Linear(dim, kernel="fullrank", param=g["full_param"])
    z, ld = f(x)
    assert close(z, g["full_z"]) and close(ld, g["full_ld"])
    assert close(f.inverse(z)[0], g["x"], 1e-10)
    f = vi.Linear(dim, kernel="structured", mask=g["psvi_mask"], param=g["psvi_param"])
    z, ld = f(x)
    assert close(z, g["psvi_z"]) and close(ld, g["psvi_ld"])
    assert close(f.inverse(z)[0], g["x"], 1e-10)


def test_psvi_mask_matches(g):
    nz, nx = 5, 6
    assert np.array_equal(vi.psvi_mask_2D(np.ones((3, 3)), nz * nx, nx=nx, nz=nz), g["psvi_mask"])


def test_constraint_transforms_and_distribution(g):
    dim = g["x"].shape[1]
    x = torch.from_numpy(g["x"])
    r2c = vi.Real2Constr(dim, lower=g["lower"], upper=g["upper"])
    z, ld = r2c(x)
    assert close(z, g["r2c_z"]) and close(ld, g["r2c_ld"])
    xi, li = r2c.inverse(z)
    assert close(xi, g["r2c_xi"], 1e-9) and close(li, g["r2c_li"])
    c2r = vi.Constr2Real(dim, lower=0.0, upper=1.0)
    z, ld = c2r(torch.from_numpy(g["ub"]))
    assert close(z, g["c2r_z"]) and close(ld, g["c2r_ld"])
    q = vi.FlowsBasedDistribution([vi.Linear(dim, kernel="structured", mask=g["psvi_mask"], param=g["psvi_param"]),
                                   vi.Real2Constr(dim, lower=g["lower"], upper=g["upper"])], base="Normal")
    zq, lq = q(x)
    assert close(zq, g["q_z"]) and close(lq, g["q_logq"])


def test_priors_with_smoothing(g):
    nz, nx = 5, 6
    S = vi.smooth_matrix_2D(nx, nz, 2.0, 3.0)
    for prior, key in ((vi.Uniform(lower=g["lower"], upper=g["upper"], smooth_matrix=S), "unif"),
                       (vi.Normal(loc=0.5 * (g["lower"] + g["upper"]),
                                  std=np.sqrt((g["upper"] - g["lower"]) ** 2 / 12), smooth_matrix=S), "norm")):
        xm = torch.from_numpy(g["xm"]).requires_grad_(True)
        lp = prior.log_prob(xm)
        lp.sum().backward()
        assert close(lp, g[f"{key}_logp"]) and close(xm.grad, g[f"{key}_grad"])


def test_vi_update_reproduces_reference_iterations(g):
    dim = g["x"].shape[1]
    mu_t = torch.from_numpy(g["mu_t"])
    torch.manual_seed(123)
    q = vi.FlowsBasedDistribution([vi.Linear(dim, kernel="diagonal")], base="Normal")
    inv = vi.VariationalInversion(q, lambda zs: -0.5 * ((zs - mu_t) ** 2).sum(axis=1) / 0.25)
    loss = inv.update(lr=0.05, n_iter=5, nsample=8)
    assert close(loss, g["vi_loss"], 1e-10)
    assert close(q.flows[0].u, g["vi_u"], 1e-10) and close(q.flows[0].diag, g["vi_diag"], 1e-10)


def test_flow_param_round_trip(g):
    """get_flow_param -> Linear(param=...) starts the next frequency band from the last."""
    dim = g["x"].shape[1]
    x = torch.from_numpy(g["x"])
    for kw in (dict(kernel="diagonal", param=g["diag_param"]), dict(kernel="fullrank", param=g["full_param"]),
               dict(kernel="structured", mask=g["psvi_mask"], param=g["psvi_param"])):
        f = vi.Linear(dim, **kw)
        f2 = vi.Linear(dim, **{**kw, "param": vi.get_flow_param(f)})
        assert torch.allclose(f(x)[0], f2(x)[0], rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_waveform_generation(engine_lib, cuda, tmp_path):
    """generate_waveform: the reference's (ns, nt, nr) float32 waveform.npy, bit-exact data."""
    from geopvi_gb300.data import generate_waveform
    z = np.load(os.path.join(os.path.dirname(cases.__file__), "fwi_o8.npz"))
    p = cases.params_from_npz(z)
    path = str(tmp_path / "waveform.npy")
    data = generate_waveform(p, z["truth"].astype(np.float64), path=path, device=cuda)
    back = np.load(path)
    assert back.dtype == np.float32 and back.shape == (p.ns, p.nt, p.nr)
    assert np.array_equal(back.ravel(), z["obs"]) and np.array_equal(data, back)


@pytest.mark.gpu
def test_vi_iteration_on_the_device(engine_lib, cuda, tmp_path):
    """A PSVI iteration of a small FWI posterior: every tensor of the step
    stays on the GPU (the misfit and gradient come from the engine)."""
    import configparser
    from geopvi_gb300.posterior import Posterior
    z = np.load(os.path.join(os.path.dirname(cases.__file__), "fwi_o8.npz"))
    p = cases.params_from_npz(z)
    cfg = configparser.ConfigParser()
    cfg["FWI"] = {k: str(v) for k, v in cases.params_to_dict(p).items()}
    cfg["FWI"]["laplace_slover"] = cfg["FWI"].pop("laplace_solver")
    cfg["FWI"]["pml"] = cfg["FWI"].pop("pml0")
    water = 2
    mask = np.ones((p.nz, p.nx), bool)
    mask[:water] = False
    ndim = int(mask.sum())
    lower = np.full(ndim, 1500.0)
    upper = np.full(ndim, 4000.0)
    S = vi.smooth_matrix_2D(p.nx, p.nz - water, 2.0, 2.0)
    prior = vi.Uniform(lower=lower, upper=upper, smooth_matrix=S, device=cuda)
    post = Posterior(z["obs"], cfg, vel_fixed=1950.0, sigma=0.1, log_prior=prior.log_prob, mask=mask.ravel(),
                     paramfile=str(tmp_path / "p.txt"), device=cuda)
    psvi = vi.psvi_mask_2D(np.ones((3, 3)), ndim, nx=p.nx, nz=p.nz - water)
    q = vi.FlowsBasedDistribution([vi.Linear(ndim, kernel="structured", mask=psvi),
                                   vi.Real2Constr(ndim, lower=lower, upper=upper)], base="Normal").to(cuda)
    inv = vi.VariationalInversion(q, post.log_prob)
    optim = torch.optim.Adam(q.parameters(), lr=0.01)
    losses = [inv.step(optim, nsample=4) for _ in range(3)]
    assert all(l.is_cuda for l in losses)
    assert all(p.is_cuda and torch.isfinite(p).all() for p in q.parameters())
    assert torch.isfinite(torch.stack(losses)).all()
    samples = q.sample_tensor(6)
    assert samples.is_cuda and samples.shape == (6, ndim)
    assert bool(((samples > 1500.0) & (samples < 4000.0)).all())

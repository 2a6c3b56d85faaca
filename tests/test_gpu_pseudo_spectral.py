"""GPU pseudo-spectral mode (laplace_solver = 1) against the oracle.

The engine transforms with cuFFT (double, real-to-complex), the oracle with
a direct DFT (double); both round the double Laplacian to float every step,
so the data agree to the scheme's round-off spread rather than bit for bit.
That spread is intrinsic: two oracle builds differing only in the DFT's
summation order (plain vs compensated) differ by 2.7-4.4e-6 on these cases,
the FP32 and FP64 schemes by 3-5e-6, and the engine lands 1.9-8.2e-6 from
the oracle.  Bars: synthetic data relative L2 <= 1e-5, gradient <= 1e-4
(the tolerances stated for this path), misfit <= 1e-5.  The same bars hold
against the reference's own pseudo-spectral code (fixtures pstd_*.npz, made by
running fdtd2D_modelling.c with FFTW stand-ins that evaluate the transform's
definition directly; tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.dirname(cases.__file__)
DATA_TOL = 1e-5
GRAD_TOL = 1e-4


def load(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oparams(O, p):
    return O.Params(**cases.params_to_dict(p))


def run(p, vel, obs, **kw):
    from geopvi_gb300.engine import Fwi2dEngine
    eng = Fwi2dEngine(p, device="cuda:0", **{k: kw.pop(k) for k in ("plain", "checkpoint", "max_resident", "graph")
                                            if k in kw})
    v = torch.from_numpy(np.ascontiguousarray(np.atleast_2d(vel), dtype=np.float32)).cuda()
    o = torch.from_numpy(np.ascontiguousarray(obs, dtype=np.float32)).cuda()
    r = eng.run(v, o, **kw)
    torch.cuda.synchronize()
    assert eng.status() == 0
    out = {"misfit": r.misfit.cpu().numpy().copy()}
    if r.grad is not None:
        out["grad"] = r.grad.cpu().numpy().copy()
    if r.syn is not None:
        out["syn"] = r.syn.cpu().numpy().copy()
    return out


@pytest.mark.parametrize("name", ["fwi_o8", "fwi_ragged", "img_o6", "fwi_o10_nti3"])
def test_pseudo_spectral_against_oracle(engine_lib, cuda, oracle, name):
    z = load(name)
    base = cases.params_from_npz(z)
    p = base.replace(laplace_solver=1)
    op = oparams(oracle, p)
    imaging = int(z["run_fwi"]) == 0
    obs_o = oracle.forward_f32(op, z["truth"])
    fwd = run(p, z["truth"], np.zeros(p.data_len, np.float32), forward_only=True)
    assert rel(fwd["syn"][0], obs_o) <= DATA_TOL
    syn_o, grad_o = oracle.fwi_f32(op, z["start"], obs_o, 0 if imaging else 1)
    out = run(p, z["start"], obs_o, imaging=imaging, want_syn=True)
    assert rel(out["syn"][0], syn_o) <= DATA_TOL
    e = rel(out["grad"][0], grad_o)
    assert e <= GRAD_TOL, f"gradient rel L2 {e:.3e}"
    if not imaging:
        r = (syn_o - obs_o).astype(np.float64)
        assert abs(out["misfit"][0] - 0.5 * np.sum(r * r)) <= DATA_TOL * 0.5 * np.sum(r * r)


@pytest.mark.parametrize("name", sorted(cases.PSTD))
def test_pseudo_spectral_against_reference(engine_lib, cuda, name):
    """The engine against the reference's own pstd_2d_calculate_p (fixtures pstd_*.npz):
    forward data, synthetic data, gradient and misfit at the path's tolerances."""
    z = load(name)
    p = cases.params_from_npz(z)
    assert p.laplace_solver == 1
    imaging = int(z["run_fwi"]) == 0
    fwd = run(p, z["truth"], np.zeros(p.data_len, np.float32), forward_only=True)
    e = rel(fwd["syn"][0], z["obs"])
    assert e <= DATA_TOL, f"forward data rel L2 {e:.3e}"
    out = run(p, z["start"], z["obs"], imaging=imaging, want_syn=True)
    e = rel(out["syn"][0], z["syn"])
    assert e <= DATA_TOL, f"synthetic data rel L2 {e:.3e}"
    e = rel(out["grad"][0], z["grad"])
    assert e <= GRAD_TOL, f"gradient rel L2 {e:.3e}"
    m = float(z["misfit"])
    assert abs(out["misfit"][0] - m) <= DATA_TOL * abs(m)


def test_pseudo_spectral_waves_plain_checkpoint(engine_lib, cuda, oracle):
    """Several samples in waves, one solve per launch, and checkpointing give
    the batched result (transforms of different batch sizes agree to
    round-off; the rest of the step is deterministic)."""
    z = load("fwi_o8_nti2")
    p = cases.params_from_npz(z).replace(laplace_solver=1)
    vel = np.stack([z["start"], 0.5 * (z["start"] + z["truth"])]).astype(np.float32)
    obs = oracle.forward_f32(oparams(oracle, p), z["truth"])
    ref = run(p, vel, obs, graph=False)
    for kw in (dict(max_resident=4), dict(plain=True), dict(checkpoint=True), dict(checkpoint=True, max_resident=5),
               dict(graph=True)):
        out = run(p, vel, obs, **kw)
        assert rel(out["grad"], ref["grad"]) <= 1e-6, kw
        assert np.allclose(out["misfit"], ref["misfit"], rtol=1e-9), kw


def test_pseudo_spectral_rejects_exact_gradient(engine_lib, cuda):
    from geopvi_gb300 import _native
    z = load("fwi_o8")
    p = cases.params_from_npz(z).replace(laplace_solver=1)
    with pytest.raises(_native.EngineError):
        run(p, z["start"], z["obs"], exact=True)

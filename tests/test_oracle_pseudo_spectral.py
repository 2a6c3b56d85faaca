"""The oracle's pseudo-spectral Laplacian (laplace_solver = 1), CPU only.

pstd_2d_calculate_p (fdtd2D_modelling.c:783-830) transforms the padded field
with FFTW in double, multiplies by -|k|^2 (wavenumber, :1127-1184) and
transforms back; in this mode the reference sets Lc = 0, so its absorbing
strips start at the grid's edge (pml = pml0, :75-78).  The restatement (a
direct separable DFT in double) is checked against the mathematics -- exact on
a plane wave up to the float rounding of |k|^2, equal to numpy's FFT to double
round-off -- and against the reference's own pseudo-spectral code, run with
FFTW stand-ins that evaluate the transform's definition directly
(oracle/stub/fftw3_stub.c; fixtures pstd_*.npz by tests/golden/make_golden.py).
Two evaluations of the double transform agree only to their last bits, which
every step's float rounding amplifies, so the fixtures are met at the path's
stated tolerances: synthetic data relative L2 <= 1e-5, gradient <= 1e-4.
"""
import os

import numpy as np
import pytest

import cases

GOLDEN = os.path.dirname(cases.__file__)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", sorted(cases.PSTD))
def test_restatement_against_reference_pseudo_spectral(oracle, name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    p = cases.params_from_npz(z)
    assert p.laplace_solver == 1 and p.pml == p.pml0
    op = oparams(oracle, p)
    obs = oracle.forward_f32(op, z["truth"])
    assert rel(obs, z["obs"]) <= 1e-5
    syn, grad = oracle.fwi_f32(op, z["start"], z["obs"], int(z["run_fwi"]))
    assert rel(syn, z["syn"]) <= 1e-5
    assert rel(grad, z["grad"]) <= 1e-4


def oparams(O, p):
    return O.Params(**cases.params_to_dict(p))


def wavenumber_np(ntx, ntz, dx, dz):
    """wavenumber() with its float roundings, in numpy."""
    dkz = np.float32(1.0 / ntz / dz)
    dkx = np.float32(1.0 / ntx / dx)
    ax = ntx // 2 + (ntx % 2)
    az = ntz // 2 + (ntz % 2)
    jz = np.where(np.arange(ntz) < az, np.arange(ntz), ntz - np.arange(ntz))
    jx = np.where(np.arange(ntx) < ax, np.arange(ntx), ntx - np.arange(ntx))
    kz = (2 * 3.1415926 * np.float64(dkz) * jz).astype(np.float32).astype(np.float64)
    kx = (2 * 3.1415926 * np.float64(dkx) * jx).astype(np.float32).astype(np.float64)
    return (kx[None, :] ** 2 + kz[:, None] ** 2).astype(np.float32)


@pytest.mark.parametrize("shape,d", [((30, 44), (10.0, 12.0)), ((27, 33), (8.0, 8.0))])
def test_plane_wave(oracle, shape, d):
    ntz, ntx = shape
    dx, dz = d
    iz, ix = np.meshgrid(np.arange(ntz), np.arange(ntx), indexing="ij")
    for mz, mx in ((3, 5), (0, 1), (ntz // 2 - 1, 2)):
        f = np.cos(2 * np.pi * (mx * ix / ntx + mz * iz / ntz))
        k2 = (2 * np.pi * mx / (ntx * dx)) ** 2 + (2 * np.pi * mz / (ntz * dz)) ** 2
        lap = oracle.pstd_laplacian(f, dx, dz)
        assert np.abs(lap + k2 * f).max() <= 1e-6 * max(k2, 1e-30)


def test_matches_numpy_fft(oracle):
    rng = np.random.default_rng(0)
    for ntz, ntx in ((30, 44), (27, 33)):
        g = rng.standard_normal((ntz, ntx))
        ref = np.real(np.fft.ifft2(np.fft.fft2(g) * -wavenumber_np(ntx, ntz, 10.0, 12.0).astype(np.float64)))
        got = oracle.pstd_laplacian(g, 10.0, 12.0)
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_pseudo_spectral_runs_close_to_fd(oracle):
    """Both Laplacians approximate the same wave equation: data within a few percent."""
    z = np.load(f"{cases.__file__.rsplit('/', 1)[0]}/fwi_o8.npz")
    p = cases.params_from_npz(z)
    op = oparams(oracle, p.replace(laplace_solver=1))
    obs = oracle.forward_f32(op, z["truth"])
    assert np.isfinite(obs).all()
    rel = np.linalg.norm(obs - z["obs"]) / np.linalg.norm(z["obs"])
    assert 1e-4 < rel < 0.1
    with pytest.raises(ValueError):
        oracle.exact_grad_f64(op, z["start"].astype(np.float64), obs.astype(np.float64))

"""3-D engine: the oracle's properties, the C ABI's host side, the file helpers.

The reference's 3-D posterior (geopvi/forward/fwi3d/posterior.py) calls an
external executable it does not ship, so there is no reference output to pin
the 3-D scheme to.  The oracle (oracle/fwi3d_oracle.cpp) is checked here for
what the scheme must satisfy: exact mirror symmetry, linearity in the source,
and a gradient that matches central differences of the misfit where the
absorbing strips are far from the acquisition.  No GPU.
"""
import ctypes
import os
import re
from types import SimpleNamespace

import numpy as np
import pytest

from geopvi_gb300 import _native, fwi3d
from oracle import oracle3d as O

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "geopvi_fwi3d.h")


def ricker(nt, dt, f0):
    t = np.arange(nt) * dt - 1.0 / f0
    a = (np.pi * f0 * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def small(nx=12, ny=11, nz=9, nt=120, Lc=4, pml0=5, nti=1, ns=2, nr=14, seed=0):
    p = SimpleNamespace(nx=nx, ny=ny, nz=nz, pml0=pml0, Lc=Lc, ns=ns, nr=nr, nt=nt, nt_interval=nti,
                        dx=10.0, dy=12.0, dz=9.0, dt=1e-3)
    rng = np.random.default_rng(seed)
    src = np.stack([rng.integers(0, nx, ns), rng.integers(0, ny, ns), rng.integers(0, 3, ns)], 1)
    rec = np.stack([rng.integers(0, nx, nr), rng.integers(0, ny, nr), np.zeros(nr, int)], 1)
    wav = ricker(nt, p.dt, 20.0)
    vel = (1800 + 600 * rng.random((ny, nx, nz))).astype(np.float32)
    return p, src, rec, wav, vel


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"^\s*#.*$", "", text, flags=re.M)
    return sorted(set(re.findall(r"\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text)))


def test_header_lists_every_export(engine_lib):
    assert set(declared_functions()) == set(fwi3d.EXPORTED_SYMBOLS)
    for name in declared_functions():
        assert hasattr(engine_lib, name), f"{name} not exported"


def test_oracle_mirror_symmetry_in_y():
    """A model, sources and receivers mirrored in y give mirrored data bit for
    bit: the stencil pairs p[+m] + p[-m] and the y-min / y-max strips are
    disjoint mirror images."""
    p, _, _, wav, vel = small(ny=12)
    vel = (0.5 * (vel + vel[::-1])).astype(np.float32)  # symmetric in y
    rec = np.array([[x, y, 0] for x in (2, 6, 9) for y in (1, 3, 5)] +
                   [[x, 11 - y, 0] for x in (2, 6, 9) for y in (1, 3, 5)])
    p.ns, p.nr = 1, rec.shape[0]
    d0, _, _ = O.run(p, np.array([[5, 3, 1]]), rec, wav, vel)
    d1, _, _ = O.run(p, np.array([[5, 11 - 3, 1]]), rec, wav, vel)
    half = rec.shape[0] // 2
    assert np.abs(d0).max() > 0
    assert np.array_equal(d0[0][:, :half], d1[0][:, half:])
    assert np.array_equal(d0[0][:, half:], d1[0][:, :half])


def test_oracle_zero_source_and_linearity():
    p, src, rec, wav, vel = small()
    z, _, _ = O.run(p, src, rec, np.zeros_like(wav), vel)
    assert not z.any()
    d1, _, _ = O.run(p, src, rec, wav, vel)
    d2, _, _ = O.run(p, src, rec, 2 * wav, vel)
    assert np.array_equal(d2, 2 * d1)  # scaling by 2 is exact in binary floating point


def test_oracle_gradient_against_central_differences():
    """With sources and receivers in the interior the gradient is dJ/dv: central
    differences (h = 4 m/s, FP32 misfit) on interior cells agree within 15 %
    (measured 0.98-1.10), and the median ratio within 5 %."""
    p = SimpleNamespace(nx=20, ny=18, nz=20, pml0=8, Lc=4, ns=2, nr=30, nt=300, nt_interval=1,
                        dx=10.0, dy=10.0, dz=10.0, dt=1e-3)
    rng = np.random.default_rng(0)
    src = np.array([[5, 9, 10], [14, 8, 10]])
    rec = np.stack([rng.integers(2, p.nx - 2, p.nr), rng.integers(2, p.ny - 2, p.nr), np.full(p.nr, 10)], 1)
    wav = ricker(p.nt, p.dt, 15.0)
    truth = (2000 + 300 * rng.random((p.ny, p.nx, p.nz))).astype(np.float32)
    obs, _, _ = O.run(p, src, rec, wav, truth)
    v0 = np.full(truth.shape, 2150.0, np.float32)
    _, g, _ = O.run(p, src, rec, wav, v0, obs, grad=True)
    G = g.reshape(p.ny, p.nx, p.nz)
    ratios = []
    for _ in range(6):
        iy, ix, iz = rng.integers(4, p.ny - 4), rng.integers(4, p.nx - 4), rng.integers(4, p.nz - 4)
        m = (iy * p.nx + ix) * p.nz + iz
        h = 4.0
        vp = v0.ravel().copy(); vp[m] += h
        vm = v0.ravel().copy(); vm[m] -= h
        fd = (O.run(p, src, rec, wav, vp, obs)[2] - O.run(p, src, rec, wav, vm, obs)[2]) / (2 * h)
        ratios.append(G[iy, ix, iz] / fd)
    ratios = np.array(ratios)
    assert np.all((ratios > 0.85) & (ratios < 1.15)), ratios
    assert abs(np.median(ratios) - 1) < 0.05, ratios


def _c(p, src, rec, wav):
    a = fwi3d.Acquisition(src, rec, wav)
    cp = fwi3d.CParams3(**{n: getattr(p, n) for n in fwi3d.INT_FIELDS + fwi3d.FLOAT_FIELDS})
    return cp, a


def test_validation_and_workspace(engine_lib):
    L = fwi3d.load()
    p, src, rec, wav, vel = small()
    cp, a = _c(p, src, rec, wav)
    assert L.gb_fwi3d_validate(ctypes.byref(cp), ctypes.byref(a.c)) == _native.OK
    for bad in (dict(Lc=2), dict(Lc=7), dict(nx=0), dict(pml0=0), dict(nt_interval=0), dict(dt=0.0),
                dict(dx=float("nan"))):
        q = SimpleNamespace(**{**p.__dict__, **bad})
        cq, aq = _c(q, src, rec, wav)
        assert L.gb_fwi3d_validate(ctypes.byref(cq), ctypes.byref(aq.c)) == _native.EINVAL, bad
    bad_src = src.copy(); bad_src[0, 1] = p.ny
    cq, aq = _c(p, bad_src, rec, wav)
    assert L.gb_fwi3d_validate(ctypes.byref(cq), ctypes.byref(aq.c)) == _native.EINVAL
    bad_wav = wav.copy(); bad_wav[3] = np.inf
    cq, aq = _c(p, src, rec, bad_wav)
    assert L.gb_fwi3d_validate(ctypes.byref(cq), ctypes.byref(aq.c)) == _native.EINVAL

    def ws(nsamples, resident, flags=0):
        n = ctypes.c_size_t(0)
        assert L.gb_fwi3d_workspace_size(ctypes.byref(cp), ctypes.byref(a.c), nsamples, resident, flags,
                                         ctypes.byref(n)) == _native.OK
        return n.value
    assert ws(3, 1) < ws(3, 2) < ws(3, 6) == ws(3, 0)
    assert ws(3, 2, fwi3d.FORWARD_ONLY) < ws(3, 2)
    # checkpointing: a long run keeps 2 ceil(sqrt(nt)) padded levels and
    # ceil(sqrt(nt)) stored steps per solve instead of nt stored steps
    q = SimpleNamespace(**{**p.__dict__, "nt": 900, "nx": 40, "ny": 40, "nz": 40, "pml0": 2})
    cq, aq = _c(q, src, rec, ricker(900, q.dt, 20.0))
    n_full, n_ck = ctypes.c_size_t(0), ctypes.c_size_t(0)
    L.gb_fwi3d_workspace_size(ctypes.byref(cq), ctypes.byref(aq.c), 2, 2, 0, ctypes.byref(n_full))
    L.gb_fwi3d_workspace_size(ctypes.byref(cq), ctypes.byref(aq.c), 2, 2, fwi3d.CHECKPOINT, ctypes.byref(n_ck))
    assert n_ck.value < 0.25 * n_full.value
    budget = ws(3, 4)
    assert L.gb_fwi3d_max_resident(ctypes.byref(cp), ctypes.byref(a.c), 3, 0, budget) == 4
    assert L.gb_fwi3d_max_resident(ctypes.byref(cp), ctypes.byref(a.c), 3, 0, 1000) == 0


def test_file_helpers_round_trip(tmp_path):
    """prepare_samples / prepare_batch / cal_loss keep the reference's files."""
    nx, ny, nz = 4, 3, 5
    theta = np.arange(2 * nx * ny * nz, dtype=np.float64).reshape(2, -1)
    fwi3d.prepare_samples(theta, nx, ny, nz, datapath=str(tmp_path))
    back = np.load(tmp_path / "particles_1.npy")
    assert back.shape == (ny, nx, nz) and np.array_equal(back.ravel(), theta[1])
    shots = np.arange(30).reshape(10, 3)
    data = np.random.default_rng(1).random((10, 7, 4)).astype(np.float32)
    np.save(tmp_path / "source.npy", shots)
    np.save(tmp_path / "data.npy", data)
    np.random.seed(3)
    scale = fwi3d.prepare_batch(4, datapath=str(tmp_path), srcfile=str(tmp_path / "source.npy"),
                                datafile=str(tmp_path / "data.npy"))
    assert scale == 2.5
    np.random.seed(3)
    sl = np.sort(np.random.choice(10, size=4, replace=False))
    assert np.array_equal(np.load(tmp_path / "batch_src.npy"), shots[sl])
    assert np.array_equal(np.load(tmp_path / "batch_data.npy"), data[sl])
    np.save(tmp_path / "pred.npy", data[sl] + 1)
    assert fwi3d.cal_loss(str(tmp_path / "pred.npy"), str(tmp_path / "batch_data.npy")) == pytest.approx(4 * 7 * 4)


def test_posterior_reads_the_reference_config(tmp_path):
    """Posterior(args, config, ...) takes the reference's [FWI] / [path] keys plus
    dt (and optional pml, Lc, nt_interval); nt is the wavelet's length.  The
    engine is created on the first call, so construction needs no GPU."""
    import configparser
    shots = np.array([[1, 2, 0], [3, 1, 1], [0, 0, 2]])
    rec = np.array([[0, 0, 0], [2, 1, 0]])
    wav = ricker(57, 1e-3, 20.0)
    data = np.zeros((3, 57, 2), np.float32)
    for name, arr in (("source", shots), ("data", data), ("rec", rec), ("wavelet", wav)):
        np.save(tmp_path / f"{name}.npy", arr)
    cfg = configparser.ConfigParser()
    cfg["FWI"] = dict(nx="4", ny="3", nz="5", dx="10", dy="12", dz="9", dt="0.0008", shot_batch="2",
                      vel_fixed="1500", recfile=str(tmp_path / "rec.npy"), waveletfile=str(tmp_path / "wavelet.npy"))
    cfg["path"] = dict(inpath=str(tmp_path), outpath=str(tmp_path), srcfile=str(tmp_path / "source.npy"),
                       datafile=str(tmp_path / "data.npy"))
    post = fwi3d.Posterior(SimpleNamespace(sigma=0.3), cfg, device="cpu")
    p = post.params
    assert (p.nx, p.ny, p.nz, p.nt) == (4, 3, 5, 57) and p.dt == pytest.approx(0.0008)
    assert (p.dx, p.dy, p.dz) == (10.0, 12.0, 9.0)
    assert (p.pml0, p.Lc, p.nt_interval) == (10, 4, 1)  # defaults
    assert post.mask.shape == (60,) and post.mask.all() and post.sigma == 0.3 and post.batch == 2
    assert post.shots.shape == (3, 3) and post.rec.shape == (2, 3) and post.data.shape == (3, 57, 2)
    cfg["FWI"].update(pml="6", Lc="5", nt_interval="3")
    q = fwi3d.Posterior(SimpleNamespace(sigma=0.3), cfg, mask=np.arange(60) % 2 == 0, device="cpu").params
    assert (q.pml0, q.Lc, q.nt_interval) == (6, 5, 3)

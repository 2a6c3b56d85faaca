"""Parity cases pinned by the golden fixtures in this folder.

Each case is a solver configuration plus the seeds of its velocity models.
``make_golden.py`` runs the reference solver (compiled unmodified from its
C sources by oracle/Makefile) on them and stores the results here; the tests
check the oracle restatement and the GPU engine against those files.
"""
from __future__ import annotations

import numpy as np

from geopvi_gb300.params import Params
from geopvi_gb300 import workloads

# Small cases: every array is stored in full.
SMALL = {
    # 8th order, one snapshot per step, FWI gradient
    "fwi_o8": dict(params=Params(nx=40, nz=24, pml0=8, Lc=4, ns=3, nt=300, ds=12, ns0=5, depths=2,
                                 depthr=1, nr=36, dr=1, nr0=2, nt_interval=1, dx=10.0, dz=12.0,
                                 dt=1e-3, f0=15.0), run_fwi=1, seed=11),
    # odd nt with a snapshot every 2nd step (nt_save rounding)
    "fwi_o8_nti2": dict(params=Params(nx=40, nz=24, pml0=8, Lc=4, ns=3, nt=301, ds=12, ns0=5, depths=2,
                                      depthr=1, nr=36, dr=1, nr0=2, nt_interval=2, dx=10.0, dz=12.0,
                                      dt=1e-3, f0=15.0), run_fwi=1, seed=12),
    # 6th order, imaging condition (record = obs, psave = p)
    "img_o6": dict(params=Params(nx=33, nz=29, pml0=6, Lc=3, ns=2, nt=250, ds=15, ns0=3, depths=3,
                                 depthr=0, nr=33, dr=1, nr0=0, nt_interval=1, dx=10.0, dz=10.0,
                                 dt=1e-3, f0=20.0), run_fwi=0, seed=13),
    # 10th order, snapshot every 3rd step
    "fwi_o10_nti3": dict(params=Params(nx=36, nz=30, pml0=7, Lc=5, ns=2, nt=280, ds=14, ns0=4, depths=1,
                                       depthr=2, nr=18, dr=2, nr0=1, nt_interval=3, dx=10.0, dz=10.0,
                                       dt=1e-3, f0=15.0), run_fwi=1, seed=14),
    # 12th order, rectangular cells
    "fwi_o12": dict(params=Params(nx=31, nz=27, pml0=6, Lc=6, ns=2, nt=260, ds=13, ns0=2, depths=2,
                                  depthr=1, nr=31, dr=1, nr0=0, nt_interval=1, dx=12.0, dz=9.0,
                                  dt=1e-3, f0=15.0), run_fwi=1, seed=15),
    # ragged edges: source and receivers inside the absorbing strip, sparse receivers
    "fwi_ragged": dict(params=Params(nx=37, nz=19, pml0=5, Lc=4, ns=2, nt=240, ds=30, ns0=-2, depths=0,
                                     depthr=3, nr=11, dr=3, nr0=-3, nt_interval=1, dx=10.0, dz=10.0,
                                     dt=1e-3, f0=18.0), run_fwi=1, seed=16),
    # one-cell absorbing strip (w = 1, so the blend keeps only the extrapolation)
    "fwi_pml1": dict(params=Params(nx=30, nz=20, pml0=1, Lc=4, ns=1, nt=200, ds=1, ns0=15, depths=2,
                                   depthr=0, nr=30, dr=1, nr0=0, nt_interval=1, dx=10.0, dz=10.0,
                                   dt=1e-3, f0=20.0), run_fwi=1, seed=17),
    # a single receiver (dr = 0 is legal when nr = 1)
    "fwi_nr1": dict(params=Params(nx=28, nz=22, pml0=6, Lc=4, ns=2, nt=220, ds=10, ns0=4, depths=2,
                                  depthr=5, nr=1, dr=0, nr0=14, nt_interval=1, dx=10.0, dz=10.0,
                                  dt=1e-3, f0=15.0), run_fwi=1, seed=18),
}

# Full-size cases: hashes, norms, gradients and a trace subsample are stored.
FULL = {
    # benchmark configuration 1, one sample
    "cfg1": dict(params=workloads.cfg1().params, run_fwi=1, seed=1),
    # the reference example's own config.ini (examples/fwi2d/input/config.ini)
    "example": dict(params=Params(nx=250, nz=110, pml0=10, Lc=3, ns=12, nt=2001, ds=20, ns0=15,
                                  depths=1, depthr=9, nr=250, dr=1, nr0=0, nt_interval=2, dx=20.0,
                                  dz=20.0, dt=0.002, f0=10.0), run_fwi=1, seed=21),
}

# Pseudo-spectral Laplacian (laplace_solver = 1): the reference's own
# pstd_2d_calculate_p, with oracle/stub/fftw3_stub.c evaluating FFTW's
# transform definition directly.  Every array is stored in full; these are
# compared at tolerances, since two evaluations of the double transform
# agree only to their last bits, which each step's float rounding amplifies.
PSTD = {
    # FWI gradient; the absorbing strips start at the grid's edge (pml = pml0)
    "pstd_fwi": dict(params=Params(nx=40, nz=24, pml0=8, Lc=4, laplace_solver=1, ns=3, nt=260, ds=12, ns0=5,
                                   depths=2, depthr=1, nr=36, dr=1, nr0=2, nt_interval=1, dx=10.0, dz=12.0,
                                   dt=1e-3, f0=15.0), run_fwi=1, seed=31),
    # imaging condition on odd padded sizes (45 x 41), stored every 2nd step
    "pstd_img": dict(params=Params(nx=33, nz=29, pml0=6, Lc=3, laplace_solver=1, ns=2, nt=241, ds=15, ns0=3,
                                   depths=3, depthr=0, nr=33, dr=1, nr0=0, nt_interval=2, dx=10.0, dz=10.0,
                                   dt=1e-3, f0=20.0), run_fwi=0, seed=32),
    # source and receivers inside the absorbing strip, sparse receivers
    "pstd_ragged": dict(params=Params(nx=37, nz=19, pml0=5, Lc=4, laplace_solver=1, ns=2, nt=220, ds=30, ns0=-2,
                                      depths=0, depthr=3, nr=11, dr=3, nr0=-3, nt_interval=1, dx=10.0, dz=10.0,
                                      dt=1e-3, f0=18.0), run_fwi=1, seed=33),
}

SUBSAMPLE_TRACES = 10  # keep every 10th receiver of shot 0 in the full-size fixtures


def small_models(p: Params, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """(truth, starting model) float32, nz*nx each."""
    rng = np.random.default_rng(seed)
    z = np.linspace(0.0, 1.0, p.nz)[:, None]
    truth = 1800.0 + 1200.0 * z + 250.0 * rng.standard_normal((p.nz, p.nx)) * 0.3
    truth = truth + 300.0 * np.exp(-((np.arange(p.nz)[:, None] - p.nz / 2) ** 2 +
                                     (np.arange(p.nx)[None, :] - p.nx / 3) ** 2) / 20.0)
    start = workloads.smooth(truth, passes=2, half=2) + rng.uniform(-80.0, 80.0, truth.shape)
    return truth.astype(np.float32).ravel(), start.astype(np.float32).ravel()


def full_models(name: str) -> tuple[np.ndarray, np.ndarray]:
    if name == "cfg1":
        w = workloads.cfg1()
        return w.truth, w.samples[0]
    p = FULL[name]["params"]
    rng = np.random.default_rng(FULL[name]["seed"])
    truth = workloads.gradient_with_anomalies(p.nz, p.nx, p.dx, rng, vtop=2000.0, vbot=4000.0)
    truth[:10] = 1950.0  # fixed water layer (config.ini: layer_fixed = 10, vel_fixed = 1950)
    start = workloads.smooth(truth) + rng.uniform(-100.0, 100.0, truth.shape)
    start[:10] = 1950.0
    return truth.astype(np.float32).ravel(), start.astype(np.float32).ravel()


def params_to_dict(p: Params) -> dict:
    from dataclasses import asdict
    return asdict(p)


def params_from_npz(z) -> Params:
    import json
    return Params(**json.loads(str(z["params_json"])))

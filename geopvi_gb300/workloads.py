"""Seeded synthetic workloads for the benchmark configurations.

No public dataset is involved: the reference's example data (waveform.npy)
is not shipped, so every model is generated here from a seed with the
shapes, sizes and value ranges of the benchmark configurations:

* ``cfg1`` plain misfit+gradient: 120x250 grid, 10 m, nt 2000, dt 1 ms,
  8th order, pml0 20, 10 Ricker 10 Hz shots at 20 m depth, 250 surface
  receivers; truth = linear 1500->4000 m/s plus 3 Gaussian anomalies
  (+-300 m/s, radius 100-300 m); 4 samples = smoothed truth + U(+-200).
* ``cfg2`` batched VI iteration: 200x400, nt 3000, 20 shots of 8 Hz,
  400 receivers, 64 samples from N(smoothed layered 1500-4500, 100^2)
  clipped to [1400, 5000].
* ``cfg3`` autograd + checkpointing: 300x600, nt 4000, dt 0.8 ms, 32 shots,
  600 receivers, 16 samples from a diagonal Gaussian.
* ``cfg4`` uneven batch: 48 (grid, shots, nt, f0) instances.

Shots are placed by ``ds = nx // ns``, ``ns0 = (nx - (ns-1)*ds) // 2``.
Everything is float32 on output, numpy only (no scipy), deterministic for a
given seed.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .params import Params


def acquisition(nx: int, ns: int) -> tuple[int, int]:
    ds = nx // ns
    ns0 = (nx - (ns - 1) * ds) // 2
    return ds, ns0


def make_params(nz: int, nx: int, nt: int, dt: float, ns: int, f0: float, *, nr: int | None = None,
                dx: float = 10.0, Lc: int = 4, pml0: int = 20, depths: int = 2, depthr: int = 0,
                nt_interval: int = 1) -> Params:
    ds, ns0 = acquisition(nx, ns)
    nr = nx if nr is None else nr
    dr = max(1, nx // nr)
    nr0 = (nx - (nr - 1) * dr) // 2 if nr < nx else 0
    return Params(nx=nx, nz=nz, pml0=pml0, Lc=Lc, laplace_solver=0, ns=ns, nt=nt, ds=ds, ns0=ns0,
                  depths=depths, depthr=depthr, nr=nr, dr=dr, nr0=nr0, nt_interval=nt_interval,
                  dx=dx, dz=dx, dt=dt, f0=f0)


def smooth(model: np.ndarray, passes: int = 4, half: int = 4) -> np.ndarray:
    """Separable repeated box filter with edge replication (approximates a
    Gaussian of sigma ~ half*sqrt(passes/3) cells)."""
    out = np.asarray(model, dtype=np.float64)
    k = 2 * half + 1
    for _ in range(passes):
        for axis in (0, 1):
            pad = [(0, 0), (0, 0)]
            pad[axis] = (half + 1, half)
            c = np.cumsum(np.pad(out, pad, mode="edge"), axis=axis)
            if axis == 0:
                out = (c[k:, :] - c[:-k, :]) / k
            else:
                out = (c[:, k:] - c[:, :-k]) / k
    return out


def gradient_with_anomalies(nz: int, nx: int, dx: float, rng: np.random.Generator,
                            vtop: float = 1500.0, vbot: float = 4000.0, n_anom: int = 3) -> np.ndarray:
    z = np.arange(nz)[:, None] * dx
    x = np.arange(nx)[None, :] * dx
    model = vtop + (vbot - vtop) * (z / max(z.max(), 1.0)) * np.ones_like(x)
    for _ in range(n_anom):
        cz = rng.uniform(0.25, 0.85) * nz * dx
        cx = rng.uniform(0.15, 0.85) * nx * dx
        rad = rng.uniform(100.0, 300.0)
        amp = rng.choice([-300.0, 300.0])
        model = model + amp * np.exp(-((z - cz) ** 2 + (x - cx) ** 2) / (2 * rad ** 2))
    return model


def layered(nz: int, nx: int, dx: float, rng: np.random.Generator, vmin: float = 1500.0,
            vmax: float = 4500.0, nlayers: int = 6) -> np.ndarray:
    z = np.arange(nz)[:, None] * dx
    x = np.arange(nx)[None, :] * dx
    bounds = np.sort(rng.uniform(0.05, 0.95, nlayers - 1)) * nz * dx
    vels = np.linspace(vmin, vmax, nlayers) + rng.uniform(-150, 150, nlayers)
    model = np.full((nz, nx), vels[0])
    for b, v in zip(bounds, vels[1:]):
        undul = 0.04 * nz * dx * np.sin(2 * np.pi * x / (nx * dx) * rng.uniform(0.5, 2.0) + rng.uniform(0, 6.3))
        model = np.where(z >= b + undul, v, model)
    return model


@dataclass
class Workload:
    name: str
    params: Params
    truth: np.ndarray      # (nz*nx,) float32
    samples: np.ndarray    # (nsamples, nz*nx) float32


def cfg1(seed: int = 1, nsamples: int = 4) -> Workload:
    p = make_params(120, 250, 2000, 1e-3, 10, 10.0)
    rng = np.random.default_rng(seed)
    truth = gradient_with_anomalies(p.nz, p.nx, p.dx, rng)
    base = smooth(truth)
    samples = np.stack([base + rng.uniform(-200.0, 200.0, base.shape) for _ in range(nsamples)])
    return Workload("cfg1", p, truth.astype(np.float32).ravel(),
                    samples.reshape(nsamples, -1).astype(np.float32))


def cfg2(seed: int = 2, nsamples: int = 64) -> Workload:
    p = make_params(200, 400, 3000, 1e-3, 20, 8.0)
    rng = np.random.default_rng(seed)
    truth = layered(p.nz, p.nx, p.dx, rng)
    mean = smooth(truth, passes=4, half=6)
    samples = np.clip(mean[None] + 100.0 * rng.standard_normal((nsamples,) + mean.shape), 1400.0, 5000.0)
    return Workload("cfg2", p, truth.astype(np.float32).ravel(),
                    samples.reshape(nsamples, -1).astype(np.float32))


def cfg3(seed: int = 3, nsamples: int = 16) -> Workload:
    p = make_params(300, 600, 4000, 0.8e-3, 32, 10.0)
    rng = np.random.default_rng(seed)
    truth = layered(p.nz, p.nx, p.dx, rng, nlayers=8)
    mean = smooth(truth, passes=4, half=8)
    std = 50.0 + 50.0 * rng.random(mean.shape)
    samples = np.clip(mean[None] + std[None] * rng.standard_normal((nsamples,) + mean.shape), 1400.0, 5000.0)
    return Workload("cfg3", p, truth.astype(np.float32).ravel(),
                    samples.reshape(nsamples, -1).astype(np.float32))


def cfg4_instances(seed: int = 4, n: int = 48) -> list[Params]:
    """Uneven batch: grids from {100x200, 200x400, 300x600, 400x800}, 4-48
    shots, nt 1500-5000, Ricker 5-12 Hz, dt 1 ms, 10 m cells."""
    rng = np.random.default_rng(seed)
    grids = [(100, 200), (200, 400), (300, 600), (400, 800)]
    out = []
    for _ in range(n):
        nz, nx = grids[rng.integers(len(grids))]
        ns = int(rng.integers(4, 49))
        nt = int(rng.integers(1500, 5001))
        f0 = float(rng.uniform(5.0, 12.0))
        out.append(make_params(nz, nx, nt, 1e-3, ns, round(f0, 2)))
    return out


def scaled(p: Params, *, nz: int | None = None, nx: int | None = None, nt: int | None = None,
           ns: int | None = None) -> Params:
    """A smaller copy of a configuration (for tests), acquisition re-derived."""
    nz = nz or p.nz
    nx = nx or p.nx
    ns = ns or p.ns
    return make_params(nz, nx, nt or p.nt, p.dt, ns, p.f0, nr=min(p.nr, nx), dx=p.dx, Lc=p.Lc,
                       pml0=p.pml0, depths=p.depths, depthr=p.depthr, nt_interval=p.nt_interval)


@dataclass
class Workload3D:
    """A seeded 3-D inversion batch for the 3-D engine (fwi3d)."""
    name: str
    params: object          # fwi3d.Fwi3dParams
    src: np.ndarray         # (ns, 3) model cells
    rec: np.ndarray         # (nr, 3) model cells
    wavelet: np.ndarray     # (nt,)
    truth: np.ndarray       # (ny*nx*nz,) float32, (ny, nx, nz) order
    samples: np.ndarray     # (nsamples, ny*nx*nz) float32


def ricker(nt: int, dt: float, f0: float) -> np.ndarray:
    """Ricker wavelet (1 - 2a) exp(-a), a = (pi f0 (t - 1/f0))^2, in FP64 rounded to float32."""
    t = np.arange(nt) * dt - 1.0 / f0
    a = (np.pi * f0 * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def fwi3d_workload(n: int = 160, nt: int = 600, nsamples: int = 4, seed: int = 6) -> Workload3D:
    """n^3 cells of 10 m, dt 1 ms, 8th order, 10-cell absorbing strips; 8 shots
    on a 2 x 4 surface grid at 2 cells depth, receivers every 4 cells on the
    surface; truth: 1.6-3.0 km/s layers bending with depth plus a slow sphere;
    samples: the smoothed truth plus N(0, 100^2), clipped to [1500, 3000]."""
    from .fwi3d import Fwi3dParams
    rng = np.random.default_rng(seed)
    p = Fwi3dParams(nx=n, ny=n, nz=n, nt=nt, dt=1e-3, dx=10.0, dy=10.0, dz=10.0, pml0=10, Lc=4, nt_interval=1)
    sx = np.linspace(n // 8, n - 1 - n // 8, 4).astype(int)
    sy = np.linspace(n // 4, n - 1 - n // 4, 2).astype(int)
    src = np.array([[x, y, 2] for y in sy for x in sx])
    g = np.arange(0, n, 4)
    rec = np.array([[x, y, 0] for y in g for x in g])
    z = np.arange(n)[None, None, :]
    x = np.arange(n)[None, :, None]
    y = np.arange(n)[:, None, None]
    depth = z + 0.08 * n * np.sin(2 * np.pi * x / n) * np.cos(np.pi * y / n)
    truth = 1600.0 + 1400.0 * np.clip(depth / n, 0, 1)
    r2 = (x - n / 2) ** 2 + (y - n / 2) ** 2 + (z - 0.55 * n) ** 2
    truth = truth - 300.0 * np.exp(-r2 / (0.12 * n) ** 2)
    base = truth.copy()
    for axis in range(3):  # separable box smoothing, 9 cells
        c = np.cumsum(np.pad(base, [(5, 4) if a == axis else (0, 0) for a in range(3)], mode="edge"), axis=axis)
        base = (np.take(c, range(9, c.shape[axis]), axis=axis) - np.take(c, range(0, c.shape[axis] - 9), axis=axis)) / 9
    samples = np.clip(base[None] + 100.0 * rng.standard_normal((nsamples,) + base.shape), 1500.0, 3000.0)
    wav = ricker(nt, p.dt, 10.0)
    return Workload3D("fwi3d", p.replace(ns=src.shape[0], nr=rec.shape[0]), src, rec, wav,
                      truth.astype(np.float32).ravel(), samples.reshape(nsamples, -1).astype(np.float32))

"""3-D acoustic FWI on the GPU, a drop-in for geopvi/forward/fwi3d/posterior.py.

The reference's 3-D posterior (posterior.py:94-177) hands every sample to an
external FWI executable through files (run_fwi_i, :44-77) and a dask cluster.
Here the same ``Posterior`` (constructor, ``fwi3d``, ``log_prob``) runs every
(sample, shot) solve of a call on one GPU through the C ABI of
include/geopvi_fwi3d.h, with the scheme that header defines (the 2-D
reference solver's algorithm on three axes).  The reference's file helpers
``prepare_samples``, ``prepare_batch`` and ``cal_loss`` (:13-41) are kept with
their file formats for workflows that still exchange files.

Formats (the reference leaves them to the external code; these are the
engine's):
  models      (m, ny*nx*nz) in (ny, nx, nz) order, nz fastest, as
              ``vel.reshape(m, ny, nx, nz)`` in fwi3d (:140-141);
  srcfile     ``np.load`` -> (nshots, 3) integer model cells (ix, iy, iz);
  datafile    ``np.load`` -> (nshots, nt, nr) float32 observed data;
  recfile     ``np.load`` -> (nr, 3) integer model cells, common to all shots;
  waveletfile ``np.load`` -> (nt,) source time function.
Config keys: [FWI] nx, ny, nz, dx, dy, dz, shot_batch, vel_fixed, recfile,
waveletfile (as the reference) plus dt and, optionally, pml (absorbing strip
width, default 10), Lc (FD half order, default 4) and nt_interval (default 1);
[path] srcfile, datafile (and inpath for the file helpers).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np
import torch
from torch.autograd import Function

from . import _native

FORWARD_ONLY = 0x1
CHECKPOINT = 0x2

# Every function include/geopvi_fwi3d.h declares.
EXPORTED_SYMBOLS = ("gb_fwi3d_validate", "gb_fwi3d_workspace_size", "gb_fwi3d_max_resident", "gb_fwi3d_run",
                    "gb_fwi3d_last_launches")

INT_FIELDS = ("nx", "ny", "nz", "pml0", "Lc", "ns", "nr", "nt", "nt_interval")
FLOAT_FIELDS = ("dx", "dy", "dz", "dt")


class CParams3(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in INT_FIELDS] + [(n, ctypes.c_float) for n in FLOAT_FIELDS]


class CAcq3(ctypes.Structure):
    _fields_ = [("src", ctypes.POINTER(ctypes.c_int)), ("rec", ctypes.POINTER(ctypes.c_int)),
                ("wavelet", ctypes.POINTER(ctypes.c_float))]


@dataclass
class Fwi3dParams:
    nx: int
    ny: int
    nz: int
    nt: int
    dt: float
    dx: float = 10.0
    dy: float = 10.0
    dz: float = 10.0
    pml0: int = 10
    Lc: int = 4
    nt_interval: int = 1
    ns: int = 1
    nr: int = 1

    def replace(self, **kw) -> "Fwi3dParams":
        d = dict(self.__dict__)
        d.update(kw)
        return Fwi3dParams(**d)

    @property
    def ncell(self) -> int:
        return self.nx * self.ny * self.nz


_bound = False


def load() -> ctypes.CDLL:
    """The engine library with the 3-D entry points typed."""
    global _bound
    L = _native.load()
    if not _bound:
        P, A = ctypes.POINTER(CParams3), ctypes.POINTER(CAcq3)
        vp = ctypes.c_void_p
        L.gb_fwi3d_validate.argtypes = [P, A]
        L.gb_fwi3d_validate.restype = ctypes.c_int
        L.gb_fwi3d_workspace_size.argtypes = [P, A, ctypes.c_int, ctypes.c_int, ctypes.c_uint,
                                              ctypes.POINTER(ctypes.c_size_t)]
        L.gb_fwi3d_workspace_size.restype = ctypes.c_int
        L.gb_fwi3d_max_resident.argtypes = [P, A, ctypes.c_int, ctypes.c_uint, ctypes.c_size_t]
        L.gb_fwi3d_max_resident.restype = ctypes.c_int
        L.gb_fwi3d_run.argtypes = [P, A, ctypes.c_int, vp, vp, vp, vp, vp, vp, ctypes.c_size_t, ctypes.c_int,
                                   ctypes.c_uint, vp]
        L.gb_fwi3d_run.restype = ctypes.c_int
        L.gb_fwi3d_last_launches.argtypes = []
        L.gb_fwi3d_last_launches.restype = ctypes.c_longlong
        _bound = True
    return L


class Acquisition:
    """Host-side acquisition arrays kept alive for the C structs that point at them."""

    def __init__(self, src, rec, wavelet):
        self.src = np.ascontiguousarray(np.asarray(src).reshape(-1, 3), dtype=np.int32)
        self.rec = np.ascontiguousarray(np.asarray(rec).reshape(-1, 3), dtype=np.int32)
        self.wavelet = np.ascontiguousarray(np.asarray(wavelet, dtype=np.float32).ravel())
        ip = ctypes.POINTER(ctypes.c_int)
        self.c = CAcq3(self.src.ctypes.data_as(ip), self.rec.ctypes.data_as(ip),
                       self.wavelet.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))


@dataclass
class Result3:
    syn: torch.Tensor | None
    grad: torch.Tensor | None
    misfit: torch.Tensor | None
    launches: int


class Fwi3dEngine:
    """Batched 3-D misfit + gradient (or data) on one GPU.

    params: Fwi3dParams (ns and nr are taken from src and rec);
    src (ns, 3), rec (nr, 3): model cells (ix, iy, iz); wavelet (nt,);
    checkpoint: keep ceil(sqrt(nt))-step segments instead of the whole
    forward field (a third propagation per step); max_resident: solves in
    flight (default: as many as fit in `hbm_fraction` of free memory).
    """

    def __init__(self, params: Fwi3dParams, src, rec, wavelet, device=None, checkpoint: bool = False,
                 max_resident: int | None = None, hbm_fraction: float = 0.8):
        self.lib = load()
        self.acq = Acquisition(src, rec, wavelet)
        self.params = params.replace(ns=self.acq.src.shape[0], nr=self.acq.rec.shape[0])
        if self.acq.wavelet.shape[0] != self.params.nt:
            raise ValueError("wavelet length must equal nt")
        self.cp = CParams3(**{n: getattr(self.params, n) for n in INT_FIELDS + FLOAT_FIELDS})
        _native.check(self.lib.gb_fwi3d_validate(ctypes.byref(self.cp), ctypes.byref(self.acq.c)),
                      "gb_fwi3d_validate")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.checkpoint = checkpoint
        self.max_resident = max_resident
        self.hbm_fraction = hbm_fraction
        self._work = None
        self._key = None

    def set_sources(self, src) -> None:
        """Replace the shot positions (same number of shots): the workspace is reused."""
        acq = Acquisition(src, self.acq.rec, self.acq.wavelet)
        if acq.src.shape[0] != self.params.ns:
            raise ValueError(f"expected {self.params.ns} shots, got {acq.src.shape[0]}")
        _native.check(self.lib.gb_fwi3d_validate(ctypes.byref(self.cp), ctypes.byref(acq.c)), "gb_fwi3d_validate")
        self.acq = acq

    def _flags(self, forward_only: bool) -> int:
        return (FORWARD_ONLY if forward_only else 0) | (CHECKPOINT if self.checkpoint and not forward_only else 0)

    def workspace_bytes(self, nsamples: int, resident: int, forward_only: bool = False) -> int:
        n = ctypes.c_size_t(0)
        _native.check(self.lib.gb_fwi3d_workspace_size(ctypes.byref(self.cp), ctypes.byref(self.acq.c), nsamples,
                                                       resident, self._flags(forward_only), ctypes.byref(n)),
                      "gb_fwi3d_workspace_size")
        return int(n.value)

    def resident_for(self, nsamples: int, forward_only: bool = False) -> int:
        if self.max_resident:
            return int(self.max_resident)
        free, _ = torch.cuda.mem_get_info(self.device)
        r = int(self.lib.gb_fwi3d_max_resident(ctypes.byref(self.cp), ctypes.byref(self.acq.c), nsamples,
                                                self._flags(forward_only), int(free * self.hbm_fraction)))
        if r < 1:
            raise _native.EngineError(_native.ENOMEM, "Fwi3dEngine: one solve does not fit in device memory")
        ninst = nsamples * self.params.ns
        waves = -(-ninst // r)
        return -(-ninst // waves)  # equal waves

    def run(self, vel: torch.Tensor, obs: torch.Tensor | None = None, forward_only: bool = False,
            want_syn: bool = False) -> Result3:
        """vel (m, ny*nx*nz) float32 on the device; obs (ns, nt, nr) float32.
        Returns synthetic data (when forward_only or want_syn), the gradient
        dJ/dv (m, ny*nx*nz) and the misfit 0.5 sum((syn - obs)^2) (FP64, m)."""
        p = self.params
        vel = vel.to(self.device, torch.float32).contiguous()
        m = vel.shape[0]
        if vel.shape[1] != p.ncell:
            raise ValueError(f"models have {vel.shape[1]} cells, expected {p.ncell}")
        if obs is not None:
            obs = obs.to(self.device, torch.float32).contiguous()
            if obs.numel() != p.ns * p.nt * p.nr:
                raise ValueError("obs must hold (ns, nt, nr) values")
        if not forward_only and obs is None:
            raise ValueError("the gradient needs observed data")
        key = (m, forward_only)
        if self._key != key:
            self._resident = self.resident_for(m, forward_only)
            nbytes = self.workspace_bytes(m, self._resident, forward_only)
            self._work = None
            self._work = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._key = key
        syn = torch.empty((m, p.ns, p.nt, p.nr), dtype=torch.float32, device=self.device) \
            if (forward_only or want_syn) else None
        grad = None if forward_only else torch.empty((m, p.ncell), dtype=torch.float32, device=self.device)
        misfit = torch.empty(m, dtype=torch.float64, device=self.device) if obs is not None else None
        stream = torch.cuda.current_stream(self.device).cuda_stream
        ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        with torch.cuda.device(self.device):
            st = self.lib.gb_fwi3d_run(ctypes.byref(self.cp), ctypes.byref(self.acq.c), m, ptr(vel), ptr(obs),
                                       ptr(syn), ptr(grad), ptr(misfit), ptr(self._work), self._work.numel(),
                                       self._resident, self._flags(forward_only), ctypes.c_void_p(stream))
        _native.check(st, "gb_fwi3d_run")
        return Result3(syn, grad, misfit, int(self.lib.gb_fwi3d_last_launches()))


# ---- the reference's file helpers (posterior.py:13-41) ----

def prepare_samples(theta, nx, ny, nz, datapath="./", fname="particles", sep="_"):
    """One ``<fname><sep><i>.npy`` per sample (posterior.py:13-19)."""
    for i in range(theta.shape[0]):
        np.save(os.path.join(datapath, fname + sep + str(i) + ".npy"), theta[i, :].reshape((ny, nx, nz)))
    return 0


def prepare_batch(batch, datapath="input", srcfile="input/source.npy", datafile="input/data.npy"):
    """A random shot subset and its data as batch files; returns nshots / batch (posterior.py:21-33)."""
    shots = np.load(srcfile)
    slices = np.sort(np.random.choice(shots.shape[0], size=batch, replace=False))
    np.save(os.path.join(datapath, "batch_src.npy"), shots[slices, :, ])
    np.save(os.path.join(datapath, "batch_data.npy"), np.load(datafile)[slices, :, :])
    return shots.shape[0] * 1. / batch


def cal_loss(pred_file, data_file="input/batch_data.npy"):
    """sum((pred - data)^2) from two files (posterior.py:35-41)."""
    return np.sum((np.load(pred_file) - np.load(data_file)) ** 2)


class ForwardModel(Function):
    """loss = func(x) with the gradient computed alongside (posterior.py:80-92)."""

    @staticmethod
    def forward(ctx, input, func):
        output, grad = func(input)
        output = torch.as_tensor(output).to(input.device)
        grad = torch.as_tensor(grad).to(input.device)
        ctx.save_for_backward(input, grad.to(input.dtype))
        return output.to(input.dtype)

    @staticmethod
    def backward(ctx, grad_output):
        input, grad = ctx.saved_tensors
        return grad_output[..., None] * grad, None


class Posterior:
    """The reference's 3-D posterior (posterior.py:94-177) on the GPU engine.

    args: needs ``sigma``; config: as the reference (see the module docstring
    for the extra ``dt`` key); mask: cells updated (default all); log_prior:
    callable x -> log prior; client: accepted for compatibility (the GPU batch
    replaces the dask cluster); device: the GPU.
    """

    def __init__(self, args, config, mask=None, log_prior=None, client=None, device=None, checkpoint=False):
        self.args = args
        self.config = config
        self.sigma = args.sigma
        self.client = client
        self.vel_water = config.getfloat("FWI", "vel_fixed")
        self.log_prior = log_prior
        f = config["FWI"]
        self.nx, self.ny, self.nz = int(f["nx"]), int(f["ny"]), int(f["nz"])
        if mask is None:
            mask = np.full((self.ny * self.nx * self.nz), True)
        self.mask = np.asarray(mask, dtype=bool)
        self.params = Fwi3dParams(nx=self.nx, ny=self.ny, nz=self.nz, nt=1, dt=float(f["dt"]), dx=float(f["dx"]),
                                  dy=float(f["dy"]), dz=float(f["dz"]), pml0=int(f.get("pml", 10)),
                                  Lc=int(f.get("Lc", 4)), nt_interval=int(f.get("nt_interval", 1)))
        self.shots = np.asarray(np.load(config.get("path", "srcfile"))).reshape(-1, 3)
        self.data = np.asarray(np.load(config.get("path", "datafile")), dtype=np.float32)
        self.rec = np.asarray(np.load(f["recfile"])).reshape(-1, 3)
        self.wavelet = np.asarray(np.load(f["waveletfile"]), dtype=np.float32).ravel()
        self.params = self.params.replace(nt=self.wavelet.shape[0])
        self.batch = config.getint("FWI", "shot_batch")
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.checkpoint = checkpoint
        self._mask_dev = torch.as_tensor(self.mask, device=self.device)
        self._data_dev = torch.as_tensor(self.data, device=self.device)
        self._eng = None

    def _engine(self, slices) -> Fwi3dEngine:
        """One engine (and workspace) for every shot subset: only the sources change."""
        if self._eng is None:
            self._eng = Fwi3dEngine(self.params, self.shots[slices], self.rec, self.wavelet, device=self.device,
                                    checkpoint=self.checkpoint)
        else:
            self._eng.set_sources(self.shots[slices])
        return self._eng

    def fwi3d(self, x):
        """x (m, ndim) -> (0.5 * loss * scale (m,), grad * scale (m, ndim)) for a
        random subset of shot_batch shots, scale = nshots / shot_batch
        (posterior.py:122-149); numpy for CPU input, CUDA tensors for CUDA input."""
        on_device = isinstance(x, torch.Tensor) and x.is_cuda
        xt = torch.as_tensor(x.detach() if isinstance(x, torch.Tensor) else np.asarray(x, dtype=np.float64))
        m = xt.shape[0]
        vel = torch.full((m, self.mask.size), float(self.vel_water), dtype=torch.float64, device=self.device)
        vel[:, self._mask_dev] = xt.to(self.device, torch.float64)
        nshots = self.shots.shape[0]
        slices = np.sort(np.random.choice(nshots, size=self.batch, replace=False))
        scale = nshots * 1. / self.batch
        obs = self._data_dev[torch.as_tensor(slices, device=self.device)]
        r = self._engine(slices).run(vel.to(torch.float32), obs)
        loss = r.misfit * scale
        grad = r.grad[:, self._mask_dev].to(torch.float64) * scale
        if on_device:
            return loss, grad
        return loss.cpu().numpy(), grad.cpu().numpy()

    def log_prob(self, x):
        """Unnormalised log posterior per sample (posterior.py:151-177)."""
        if torch.isnan(x).any():
            raise ValueError("NaN occured in sample!")
        loss = ForwardModel.apply(x, self.fwi3d)
        logp = -loss / self.sigma ** 2
        if self.log_prior is not None:
            logp = logp + self.log_prior(x)
        return logp

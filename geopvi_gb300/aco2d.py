"""Drop-in for the Cython module ``aco2d`` (geopvi/forward/fwi2d/pyacofwi2D.pyx).

Same functions, signatures, dtypes and return values:

* ``fwi(vel, record_obs, paramfile, is_fwi, verbose) -> (record_syn, grad)``
  (pyacofwi2D.pyx:11-30)
* ``forward(vel, dim, paramfile, verbose) -> record_syn``  (pyacofwi2D.pyx:33-48)

Both call the engine's C entry points ``fwi_2D`` / ``forward_2D``, which keep
the reference's C signatures (pyacofwi2D.h:2-3) and run every shot on the GPU.
A NaN velocity prints the reference's message and raises SystemExit, as the
Cython module's ``exit()`` does; a missing parameter file raises
FileNotFoundError where the reference's C calls exit(0)
(fdtd2D_modelling.c:1335).
"""
from __future__ import annotations

import ctypes
import sys

import numpy as np

from . import _native
from .params import read_paramfile

_f32p = ctypes.POINTER(ctypes.c_float)


def _as_f64_vector(vel) -> np.ndarray:
    vel = np.asarray(vel)
    if vel.dtype != np.float64 or vel.ndim != 1 or not vel.flags.c_contiguous:
        raise TypeError("vel must be a 1-D C-contiguous float64 array (pyacofwi2D.pyx:11)")
    return vel


def _nan_exit(vel: np.ndarray) -> None:
    if np.isnan(vel).any():
        print("NaN occured in python")
        sys.exit()


def fwi(vel, record_obs, paramfile="./input/input_param.txt", is_fwi=1, verbose=0):
    """Synthetic data and gradient for one velocity model (pyacofwi2D.pyx:11-30)."""
    vel = _as_f64_vector(vel)
    record_obs = np.asarray(record_obs)
    if record_obs.dtype != np.float32 or record_obs.ndim != 1 or not record_obs.flags.c_contiguous:
        raise TypeError("record_obs must be a 1-D C-contiguous float32 array (pyacofwi2D.pyx:12)")
    _nan_exit(vel)
    p = read_paramfile(paramfile)
    if vel.shape[0] != p.ncell or record_obs.shape[0] != p.data_len:
        raise ValueError(f"sizes: vel {vel.shape[0]} (nz*nx = {p.ncell}), "
                         f"record_obs {record_obs.shape[0]} (ns*nt*nr = {p.data_len})")
    vel_f = np.float32(vel)
    grad = np.zeros(vel_f.shape[0], dtype=np.float32)
    record_syn = np.zeros(record_obs.shape[0], dtype=np.float32)
    lib = _native.load()
    st = lib.fwi_2D(paramfile.encode(), vel_f.ctypes.data_as(_f32p), record_syn.ctypes.data_as(_f32p),
                    record_obs.ctypes.data_as(_f32p), grad.ctypes.data_as(_f32p), int(is_fwi), int(verbose))
    _native.check(st, "fwi_2D")
    return record_syn, grad


def forward(vel, dim=1, paramfile="./input/input_param.txt", verbose=0):
    """Synthetic data only (pyacofwi2D.pyx:33-48); ``dim`` = ns*nt*nr."""
    vel = _as_f64_vector(vel)
    _nan_exit(vel)
    p = read_paramfile(paramfile)
    if vel.shape[0] != p.ncell:
        raise ValueError(f"vel has {vel.shape[0]} cells, expected nz*nx = {p.ncell}")
    if dim < p.data_len:
        raise ValueError(f"dim = {dim} is smaller than ns*nt*nr = {p.data_len}")
    vel_f = np.float32(vel)
    record_syn = np.zeros(dim, dtype=np.float32)
    lib = _native.load()
    st = lib.forward_2D(paramfile.encode(), vel_f.ctypes.data_as(_f32p), record_syn.ctypes.data_as(_f32p),
                        1, int(verbose))
    _native.check(st, "forward_2D")
    return record_syn

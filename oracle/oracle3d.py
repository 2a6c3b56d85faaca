"""ctypes front end for the 3-D scheme's CPU restatement (TEST INFRASTRUCTURE ONLY).

Only tests/ and bench.py's cpu_baseline leg import this module; the engine in
``geopvi_gb300`` never does.  ``liboracle_fwi3d.so`` (oracle/fwi3d_oracle.cpp)
follows include/geopvi_fwi3d.h's scheme operation by operation in FP32.

Parameters are read by attribute (nx, ny, nz, pml0, Lc, ns, nr, nt,
nt_interval, dx, dy, dz, dt), so any object with those fields works.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle_fwi3d.so")

INT_FIELDS = ("nx", "ny", "nz", "pml0", "Lc", "ns", "nr", "nt", "nt_interval")
FLOAT_FIELDS = ("dx", "dy", "dz", "dt")


class CParams3(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in INT_FIELDS] + [(n, ctypes.c_float) for n in FLOAT_FIELDS]


class CAcq3(ctypes.Structure):
    _fields_ = [("src", ctypes.POINTER(ctypes.c_int)), ("rec", ctypes.POINTER(ctypes.c_int)),
                ("wavelet", ctypes.POINTER(ctypes.c_float))]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            subprocess.run(["make", "-s", "-C", ORACLE_DIR, "oracle"], check=True)
        L = ctypes.CDLL(_LIB_PATH)
        f32 = ctypes.POINTER(ctypes.c_float)
        L.oracle3d_run.argtypes = [ctypes.POINTER(CParams3), ctypes.POINTER(CAcq3), f32, f32, f32, f32,
                                   ctypes.POINTER(ctypes.c_double)]
        L.oracle3d_run.restype = ctypes.c_int
        _lib = L
    return _lib


def run(p, src, rec, wavelet, vel, obs=None, grad: bool = False):
    """One sample: (syn [ns][nt][nr] float32, grad [ny*nx*nz] float32 or None,
    misfit float or None).  vel is in (ny, nx, nz) order, nz fastest."""
    cp = CParams3(**{n: getattr(p, n) for n in INT_FIELDS + FLOAT_FIELDS})
    src = np.ascontiguousarray(src, dtype=np.int32).reshape(-1, 3)
    rec = np.ascontiguousarray(rec, dtype=np.int32).reshape(-1, 3)
    wav = np.ascontiguousarray(wavelet, dtype=np.float32).ravel()
    vel = np.ascontiguousarray(vel, dtype=np.float32).ravel()
    acq = CAcq3(src.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), rec.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                wav.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    syn = np.zeros(p.ns * p.nt * p.nr, np.float32)
    g = np.zeros(vel.shape[0], np.float32) if grad else None
    mis = ctypes.c_double(0.0)
    f32 = ctypes.POINTER(ctypes.c_float)
    ob = None
    if obs is not None:
        ob = np.ascontiguousarray(obs, dtype=np.float32).ravel()
    st = lib().oracle3d_run(ctypes.byref(cp), ctypes.byref(acq), vel.ctypes.data_as(f32),
                            ob.ctypes.data_as(f32) if ob is not None else None, syn.ctypes.data_as(f32),
                            g.ctypes.data_as(f32) if g is not None else None,
                            ctypes.byref(mis) if ob is not None else None)
    if st:
        raise ValueError(f"oracle3d_run status {st}")
    return syn.reshape(p.ns, p.nt, p.nr), g, (mis.value if ob is not None else None)

"""ctypes front end for the CPU checkers (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the cpu_baseline / reference legs
of ``bench.py`` import this module.  The engine in ``geopvi_gb300`` never
does: it has no CPU path.

Two checkers sit behind it:

* ``liboracle_fwi2d.so`` -- the project's C++ restatement of the reference
  solver (``oracle/fwi2d_oracle.cpp``), in the reference's FP32 arithmetic and
  in FP64;
* ``_ref/libref_fwi2d.so`` -- the reference's own ``fdtd2D_modelling.c``
  compiled unmodified (only where its sources were present at build time).

The reference reads its parameters from a positional text file
(``read_parameters``, geopvi/forward/fwi2d/fdtd2D_modelling.c:1328-1379),
written by ``prepare_fwi_parameters`` (geopvi/forward/fwi2d/posterior.py:27-68);
``write_paramfile`` produces the same layout.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
import tempfile
from dataclasses import dataclass, fields

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle_fwi2d.so")
_REF_PATH = os.path.join(ORACLE_DIR, "_ref", "libref_fwi2d.so")

INT_FIELDS = ("nx", "nz", "pml0", "Lc", "laplace_solver", "ns", "nt", "ds", "ns0",
              "depths", "depthr", "nr", "dr", "nr0", "nt_interval")
FLOAT_FIELDS = ("dx", "dz", "dt", "f0")

# Comment lines of prepare_fwi_parameters (posterior.py:29-65), one per value.
_COMMENTS = {
    "nx": "--grid points in x direction (nx)",
    "nz": "--grid points in z direction (nz)",
    "pml0": "--pml points (pml0)",
    "Lc": "--Finite difference order (Lc)",
    "laplace_solver": "--Method to calculate Laplace operator: 0 for FDM and 1 for PSM, (laplace_slover)",
    "ns": "--Total number of sources (ns)",
    "nt": "--Total time steps (nt)",
    "ds": "--Shot interval in grid points (ds)",
    "ns0": "--Grid number of the first shot to the left of the model (ns0)",
    "depths": "--Depth of source in grid points (depths)",
    "depthr": "--Depth of receiver in grid points (depthr)",
    "nr": "--Total number of receivers (nr)",
    "dr": "--Receiver interval in grid points (dr)",
    "nr0": "--Grid number of the first receiver to the left of the model (nr0)",
    "nt_interval": "--Time step interval of saved wavefield during forward (nt_interval)",
    "dx": "--Grid spacing in x direction (dx)",
    "dz": "--Grid spacing in z direction (dz)",
    "dt": "--Time step (dt)",
    "f0": "--Dominant frequency (f0)",
}


class CParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in INT_FIELDS] + [(n, ctypes.c_float) for n in FLOAT_FIELDS]


@dataclass
class Params:
    nx: int
    nz: int
    pml0: int = 20
    Lc: int = 4
    laplace_solver: int = 0
    ns: int = 1
    nt: int = 100
    ds: int = 1
    ns0: int = 0
    depths: int = 2
    depthr: int = 0
    nr: int = 1
    dr: int = 1
    nr0: int = 0
    nt_interval: int = 1
    dx: float = 10.0
    dz: float = 10.0
    dt: float = 1e-3
    f0: float = 10.0

    def c(self) -> CParams:
        return CParams(**{f.name: getattr(self, f.name) for f in fields(self)})

    @property
    def pml(self) -> int:
        # pseudo-spectral mode: the reference sets Lc = 0 first (fdtd2D_modelling.c:75-78)
        return self.pml0 if self.laplace_solver == 1 else self.pml0 + self.Lc + 1

    @property
    def data_len(self) -> int:
        return self.ns * self.nt * self.nr


def write_paramfile(path: str, p: Params) -> None:
    with open(path, "w") as f:
        for name in INT_FIELDS + FLOAT_FIELDS:
            f.write(_COMMENTS[name] + "\n")
            f.write(f"{getattr(p, name)}\n")


# Where this checkout keeps the reference solver's sources (read-only); the
# GEOPVI_REFERENCE_FWI2D environment variable overrides it.  Absent on
# machines that only hold this repository: the reference is then not built.
REFERENCE_FWI2D = os.environ.get("GEOPVI_REFERENCE_FWI2D", "/root/reference/geopvi/forward/fwi2d")


def build() -> None:
    """Compile the restatement (and the reference, if its sources exist)."""
    cmd = ["make", "-s", "-C", ORACLE_DIR, "all"]
    if os.path.isfile(os.path.join(REFERENCE_FWI2D, "fdtd2D_modelling.c")):
        cmd.append(f"REF_SRC={REFERENCE_FWI2D}")
    # make's messages go to stderr: a bench run's stdout carries one JSON line
    subprocess.run(cmd, check=True, stdout=sys.stderr)


_lib = None
_ref = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER(CParams)
        fp32 = ctypes.POINTER(ctypes.c_float)
        fp64 = ctypes.POINTER(ctypes.c_double)
        L.oracle_fwi2d_f32.argtypes = [P, fp32, fp32, fp32, fp32, ctypes.c_int]
        L.oracle_fwi2d_f64.argtypes = [P, fp64, fp64, fp64, fp64, ctypes.c_int]
        L.oracle_forward2d_f32.argtypes = [P, fp32, fp32]
        L.oracle_forward2d_f64.argtypes = [P, fp64, fp64]
        L.oracle_exact_grad_f64.argtypes = [P, fp64, fp64, fp64, fp64]
        L.oracle_pstd_laplacian.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, fp64, fp64]
        L.oracle_read_params.argtypes = [ctypes.c_char_p, P]
        L.oracle_ricker_f32.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float, fp32]
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_get_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(_REF_PATH)


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError("reference solver not built (oracle/_ref)")
        R = ctypes.CDLL(_REF_PATH)
        fp32 = ctypes.POINTER(ctypes.c_float)
        R.fwi_2D.argtypes = [ctypes.c_char_p, fp32, fp32, fp32, fp32, ctypes.c_int, ctypes.c_int]
        R.fwi_2D.restype = None
        R.forward_2D.argtypes = [ctypes.c_char_p, fp32, fp32, ctypes.c_int, ctypes.c_int]
        R.forward_2D.restype = None
        _ref = R
    return _ref


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def get_threads() -> int:
    return int(lib().oracle_get_threads())


def fwi_f32(p: Params, vel, obs, run_fwi: int = 1):
    """(syn f32[ns*nt*nr], grad f32[nz*nx]) in the reference's FP32 arithmetic."""
    vel = np.ascontiguousarray(vel, dtype=np.float32).ravel()
    obs = np.ascontiguousarray(obs, dtype=np.float32).ravel()
    syn = np.zeros(p.data_len, np.float32)
    grad = np.zeros(p.nz * p.nx, np.float32)
    cp = p.c()
    st = lib().oracle_fwi2d_f32(ctypes.byref(cp), _ptr(vel, ctypes.c_float), _ptr(obs, ctypes.c_float),
                                _ptr(syn, ctypes.c_float), _ptr(grad, ctypes.c_float), int(run_fwi))
    if st:
        raise ValueError(f"oracle_fwi2d_f32 status {st}")
    return syn, grad


def fwi_f64(p: Params, vel, obs, run_fwi: int = 1):
    """(syn f64, grad f64): the same scheme carried out in double precision."""
    vel = np.ascontiguousarray(vel, dtype=np.float64).ravel()
    obs = np.ascontiguousarray(obs, dtype=np.float64).ravel()
    syn = np.zeros(p.data_len, np.float64)
    grad = np.zeros(p.nz * p.nx, np.float64)
    cp = p.c()
    st = lib().oracle_fwi2d_f64(ctypes.byref(cp), _ptr(vel, ctypes.c_double), _ptr(obs, ctypes.c_double),
                                _ptr(syn, ctypes.c_double), _ptr(grad, ctypes.c_double), int(run_fwi))
    if st:
        raise ValueError(f"oracle_fwi2d_f64 status {st}")
    return syn, grad


def forward_f32(p: Params, vel):
    vel = np.ascontiguousarray(vel, dtype=np.float32).ravel()
    syn = np.zeros(p.data_len, np.float32)
    cp = p.c()
    st = lib().oracle_forward2d_f32(ctypes.byref(cp), _ptr(vel, ctypes.c_float), _ptr(syn, ctypes.c_float))
    if st:
        raise ValueError(f"oracle_forward2d_f32 status {st}")
    return syn


def forward_f64(p: Params, vel):
    vel = np.ascontiguousarray(vel, dtype=np.float64).ravel()
    syn = np.zeros(p.data_len, np.float64)
    cp = p.c()
    st = lib().oracle_forward2d_f64(ctypes.byref(cp), _ptr(vel, ctypes.c_double), _ptr(syn, ctypes.c_double))
    if st:
        raise ValueError(f"oracle_forward2d_f64 status {st}")
    return syn


def exact_grad_f64(p: Params, vel, obs):
    """(misfit, dJ/dv f64[nz*nx]): the exact gradient of the discrete scheme
    (double precision) for J = 0.5 * sum((syn - obs)^2) over all shots."""
    vel = np.ascontiguousarray(vel, dtype=np.float64).ravel()
    obs = np.ascontiguousarray(obs, dtype=np.float64).ravel()
    grad = np.zeros(p.nz * p.nx, np.float64)
    J = ctypes.c_double(0.0)
    cp = p.c()
    st = lib().oracle_exact_grad_f64(ctypes.byref(cp), _ptr(vel, ctypes.c_double), _ptr(obs, ctypes.c_double),
                                     _ptr(grad, ctypes.c_double), ctypes.byref(J))
    if st:
        raise ValueError(f"oracle_exact_grad_f64 status {st}")
    return J.value, grad


def pstd_laplacian(field, dx: float, dz: float) -> np.ndarray:
    """The pseudo-spectral Laplacian of a [ntz, ntx] field (float64)."""
    f = np.ascontiguousarray(field, dtype=np.float64)
    out = np.zeros_like(f)
    st = lib().oracle_pstd_laplacian(f.shape[0], f.shape[1], float(dx), float(dz), _ptr(f, ctypes.c_double),
                                     _ptr(out, ctypes.c_double))
    if st:
        raise ValueError(f"oracle_pstd_laplacian status {st}")
    return out


def misfit_f64(p: Params, vel, obs) -> float:
    syn = forward_f64(p, vel)
    return float(0.5 * np.sum((syn - np.asarray(obs, np.float64).ravel()) ** 2))


def ricker_f32(nt: int, dt: float, f0: float) -> np.ndarray:
    out = np.zeros(nt, np.float32)
    lib().oracle_ricker_f32(int(nt), float(dt), float(f0), _ptr(out, ctypes.c_float))
    return out


def read_params(path: str) -> Params:
    cp = CParams()
    st = lib().oracle_read_params(path.encode(), ctypes.byref(cp))
    if st:
        raise ValueError(f"oracle_read_params status {st}")
    return Params(**{n: getattr(cp, n) for n in INT_FIELDS + FLOAT_FIELDS})


def ref_fwi(p: Params, vel, obs, run_fwi: int = 1):
    """The reference's own fwi_2D (fdtd2D_modelling.c:18), as aco2d.fwi calls it
    (pyacofwi2D.pyx:11-30: float64 velocity cast to float32, zeroed outputs)."""
    vel = np.ascontiguousarray(np.float32(np.asarray(vel, dtype=np.float64))).ravel()
    obs = np.ascontiguousarray(obs, dtype=np.float32).ravel()
    syn = np.zeros(obs.shape[0], np.float32)
    grad = np.zeros(vel.shape[0], np.float32)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "input_param.txt")
        write_paramfile(path, p)
        ref().fwi_2D(path.encode(), _ptr(vel, ctypes.c_float), _ptr(syn, ctypes.c_float),
                     _ptr(obs, ctypes.c_float), _ptr(grad, ctypes.c_float), int(run_fwi), 0)
    return syn, grad


def ref_forward(p: Params, vel):
    """The reference's forward_2D (fdtd2D_modelling.c:356), as aco2d.forward calls it."""
    vel = np.ascontiguousarray(np.float32(np.asarray(vel, dtype=np.float64))).ravel()
    syn = np.zeros(p.data_len, np.float32)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "input_param.txt")
        write_paramfile(path, p)
        ref().forward_2D(path.encode(), _ptr(vel, ctypes.c_float), _ptr(syn, ctypes.c_float), 1, 0)
    return syn

"""Solver parameters: the 19 values of the reference's positional parameter file.

``prepare_fwi_parameters`` writes the file from an INI ``[FWI]`` section
exactly as geopvi/forward/fwi2d/posterior.py:27-68 does, and ``read_paramfile``
parses it with the engine's own reader (the C ABI's gb_fwi2d_read_params,
which restates read_parameters, fdtd2D_modelling.c:1328-1379).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, fields, replace

from . import _native

INT_FIELDS = _native.INT_FIELDS
FLOAT_FIELDS = _native.FLOAT_FIELDS

# (comment line, INI key) per value, in file order (posterior.py:29-66).
_FILE_LAYOUT = (
    ("nx", "--grid points in x direction (nx)", "nx"),
    ("nz", "--grid points in z direction (nz)", "nz"),
    ("pml0", "--pml points (pml0)", "pml"),
    ("Lc", "--Finite difference order (Lc)", "Lc"),
    ("laplace_solver", "--Method to calculate Laplace operator: 0 for FDM and 1 for PSM, (laplace_slover)",
     "laplace_slover"),
    ("ns", "--Total number of sources (ns)", "ns"),
    ("nt", "--Total time steps (nt)", "nt"),
    ("ds", "--Shot interval in grid points (ds)", "ds"),
    ("ns0", "--Grid number of the first shot to the left of the model (ns0)", "ns0"),
    ("depths", "--Depth of source in grid points (depths)", "depths"),
    ("depthr", "--Depth of receiver in grid points (depthr)", "depthr"),
    ("nr", "--Total number of receivers (nr)", "nr"),
    ("dr", "--Receiver interval in grid points (dr)", "dr"),
    ("nr0", "--Grid number of the first receiver to the left of the model (nr0)", "nr0"),
    ("nt_interval", "--Time step interval of saved wavefield during forward (nt_interval)", "nt_interval"),
    ("dx", "--Grid spacing in x direction (dx)", "dx"),
    ("dz", "--Grid spacing in z direction (dz)", "dz"),
    ("dt", "--Time step (dt)", "dt"),
    ("f0", "--Dominant frequency (f0)", "f0"),
)


@dataclass(frozen=True)
class Params:
    """One solver configuration.  ``Lc`` is the file's value (half the FD
    order); ``pml0`` the absorbing-strip width in cells."""
    nx: int
    nz: int
    pml0: int = 20
    Lc: int = 4
    laplace_solver: int = 0
    ns: int = 1
    nt: int = 1000
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

    # ---- derived sizes (fdtd2D_modelling.c:70, 75-78, 85-89, 167-169) ----
    @property
    def pml(self) -> int:
        # The pseudo-spectral Laplacian has no stencil halo: the reference sets
        # Lc = 0 before pml = pml0 + Lc (fdtd2D_modelling.c:75-78).
        return self.pml0 if self.laplace_solver == 1 else self.pml0 + self.Lc + 1

    @property
    def ntz(self) -> int:
        return self.nz + 2 * self.pml

    @property
    def ntx(self) -> int:
        return self.nx + 2 * self.pml

    @property
    def ntp(self) -> int:
        return self.ntz * self.ntx

    @property
    def ncell(self) -> int:
        return self.nz * self.nx

    @property
    def data_len(self) -> int:
        return self.ns * self.nt * self.nr

    @property
    def nt_save(self) -> int:
        return self.nt // self.nt_interval + (1 if self.nt % self.nt_interval else 0)

    def c(self) -> _native.CParams:
        return _native.CParams(**{f.name: getattr(self, f.name) for f in fields(self)})

    def replace(self, **kw) -> "Params":
        return replace(self, **kw)

    def validate(self) -> None:
        lib = _native.load()
        cp = self.c()
        _native.check(lib.gb_fwi2d_validate(ctypes.byref(cp)), "gb_fwi2d_validate")

    @staticmethod
    def from_config(config) -> "Params":
        """From a configparser holding the example's ``[FWI]`` section."""
        vals = {}
        for name, _, key in _FILE_LAYOUT:
            raw = config.get("FWI", key)
            vals[name] = int(raw) if name in INT_FIELDS else float(raw)
        return Params(**vals)


def write_paramfile(path: str, p: Params) -> None:
    """The file layout of prepare_fwi_parameters (posterior.py:27-68)."""
    with open(path, "w") as f:
        for name, comment, _ in _FILE_LAYOUT:
            f.write(comment + "\n")
            f.write(f"{getattr(p, name)}\n")


def prepare_fwi_parameters(paramfile: str, config) -> None:
    """Same behaviour as posterior.py:27-68: copy the INI strings verbatim."""
    with open(paramfile, "w") as f:
        for _, comment, key in _FILE_LAYOUT:
            f.write(comment + "\n")
            f.write(config.get("FWI", key) + "\n")


def read_paramfile(path: str) -> Params:
    lib = _native.load()
    cp = _native.CParams()
    st = lib.gb_fwi2d_read_params(path.encode(), ctypes.byref(cp))
    if st == _native.ENOENT:
        raise FileNotFoundError(f"Cannot open {path}!")
    _native.check(st, f"read_paramfile({path})")
    return Params(**{n: getattr(cp, n) for n in INT_FIELDS + FLOAT_FIELDS})

"""ctypes binding of the engine's C ABI (include/geopvi_fwi2d.h).

The shared library is built in-tree by ``geopvi_gb300.build``.  There is no
CPU implementation behind this module: if the library is missing, or no CUDA
device is present when a solve is requested, the call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

INT_FIELDS = ("nx", "nz", "pml0", "Lc", "laplace_solver", "ns", "nt", "ds", "ns0",
              "depths", "depthr", "nr", "dr", "nr0", "nt_interval")
FLOAT_FIELDS = ("dx", "dz", "dt", "f0")

OK = 0
ENOENT = -2
E2BIG = -7
ENOMEM = -12
EINVAL = -22
ENOTSUP = -95
ENAN = -1001
ECUDA = -1002
ETIMEOUT = -1003

FLAG_IMAGING = 0x1
FLAG_PLAIN = 0x2
FLAG_GRAPH = 0x4
FLAG_CHECKPOINT = 0x8
FLAG_FORWARD_ONLY = 0x10
FLAG_PROFILE = 0x20
FLAG_EXACT_GRADIENT = 0x40
VARIANT_SHIFT = 8
NUM_STEP_VARIANTS = 4


def flag_variant(v: int) -> int:
    """Force FD step variant v (0-3); 0 in the flags lets the tuner choose."""
    return (v + 1) << VARIANT_SHIFT

STATIC_SCRATCH_BYTES = 64 << 20

STATUS_NAMES = {ENOENT: "ENOENT (parameter file missing)", E2BIG: "E2BIG (batch exceeds the static scratch)", ENOMEM: "ENOMEM (device memory)",
                EINVAL: "EINVAL (invalid parameters or buffers)",
                ENOTSUP: "ENOTSUP (combination not supported, or cuFFT missing for laplace_solver = 1)",
                ENAN: "ENAN (NaN in velocity)", ECUDA: "ECUDA (CUDA runtime error)",
                ETIMEOUT: "ETIMEOUT (a bounded device wait gave up)"}

# Every symbol the header declares; tests check that the library exports each.
EXPORTED_SYMBOLS = (
    "gb_fwi2d_read_params", "gb_fwi2d_validate", "fwi_2D", "forward_2D",
    "gb_fwi2d_workspace_bytes", "gb_fwi2d_batch", "gb_fwi2d_last_launch_count",
    "gb_fwi2d_release_caches", "gb_fwi2d_version", "gb_fwi2d_profile_step_ms", "gb_fwi2d_status",
    "gb_fwi2d_batch_noalloc", "gb_fwi2d_tuned_variant", "gb_fwi2d_instances_workspace_bytes",
    "gb_fwi2d_run_instances", "gb_fwi2d_side_stream_count", "gb_fwi2d_instances_waves",
)


class CParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in INT_FIELDS] + [(n, ctypes.c_float) for n in FLOAT_FIELDS]


class CInstance(ctypes.Structure):
    """gb_fwi2d_instance: one entry of an uneven batch (device pointers)."""
    _fields_ = [("params", CParams), ("nsamples", ctypes.c_int), ("vel", ctypes.c_void_p),
                ("obs", ctypes.c_void_p), ("syn", ctypes.c_void_p), ("grad", ctypes.c_void_p),
                ("misfit", ctypes.c_void_p)]


class EngineError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: status {status} {STATUS_NAMES.get(status, '')}".strip())


_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB_PATH


def load() -> ctypes.CDLL:
    """Load the engine library; raise if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise ImportError(f"GB300 engine library missing ({path}); run geopvi_gb300.build.build()")
        L = ctypes.CDLL(path)
        P = ctypes.POINTER(CParams)
        f32 = ctypes.POINTER(ctypes.c_float)
        L.gb_fwi2d_read_params.argtypes = [ctypes.c_char_p, P]
        L.gb_fwi2d_read_params.restype = ctypes.c_int
        L.gb_fwi2d_validate.argtypes = [P]
        L.gb_fwi2d_validate.restype = ctypes.c_int
        L.fwi_2D.argtypes = [ctypes.c_char_p, f32, f32, f32, f32, ctypes.c_int, ctypes.c_int]
        L.fwi_2D.restype = ctypes.c_int
        L.forward_2D.argtypes = [ctypes.c_char_p, f32, f32, ctypes.c_int, ctypes.c_int]
        L.forward_2D.restype = ctypes.c_int
        L.gb_fwi2d_workspace_bytes.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_uint]
        L.gb_fwi2d_workspace_bytes.restype = ctypes.c_size_t
        L.gb_fwi2d_batch.argtypes = [P, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        L.gb_fwi2d_batch.restype = ctypes.c_int
        L.gb_fwi2d_batch_noalloc.argtypes = [P, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p]
        L.gb_fwi2d_batch_noalloc.restype = ctypes.c_int
        L.gb_fwi2d_last_launch_count.argtypes = []
        L.gb_fwi2d_last_launch_count.restype = ctypes.c_longlong
        L.gb_fwi2d_profile_step_ms.argtypes = [ctypes.POINTER(ctypes.c_longlong)]
        L.gb_fwi2d_profile_step_ms.restype = ctypes.c_double
        L.gb_fwi2d_status.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.gb_fwi2d_status.restype = ctypes.c_int
        L.gb_fwi2d_tuned_variant.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_uint]
        L.gb_fwi2d_tuned_variant.restype = ctypes.c_int
        I = ctypes.POINTER(CInstance)
        L.gb_fwi2d_instances_workspace_bytes.argtypes = [I, ctypes.c_int, ctypes.c_int, ctypes.c_uint]
        L.gb_fwi2d_instances_workspace_bytes.restype = ctypes.c_size_t
        L.gb_fwi2d_run_instances.argtypes = [I, ctypes.c_int, ctypes.c_uint, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_size_t, ctypes.c_void_p]
        L.gb_fwi2d_run_instances.restype = ctypes.c_int
        L.gb_fwi2d_instances_waves.argtypes = [I, ctypes.c_int, ctypes.c_uint, ctypes.c_int, ctypes.c_size_t]
        L.gb_fwi2d_instances_waves.restype = ctypes.c_int
        L.gb_fwi2d_side_stream_count.argtypes = []
        L.gb_fwi2d_side_stream_count.restype = ctypes.c_int
        L.gb_fwi2d_release_caches.argtypes = []
        L.gb_fwi2d_release_caches.restype = None
        L.gb_fwi2d_version.argtypes = []
        L.gb_fwi2d_version.restype = ctypes.c_char_p
        _lib = L
        return L


def check(status: int, where: str) -> None:
    if status != OK:
        raise EngineError(status, where)

"""Build the engine's shared library in-tree with nvcc (sm_103a only).

``python -m geopvi_gb300.build`` compiles ``csrc/*.cu`` into
``geopvi_gb300/_lib/libgeopvi_fwi2d.so``.  The library exports the C ABI of
``include/geopvi_fwi2d.h``; Python reaches it through ctypes
(``geopvi_gb300._native``).

Host code is compiled with FMA contraction off: the Ricker table and other
host-side tables must round exactly like the reference's C on both x86-64 and
aarch64 (where GCC contracts by default).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_NAME = "libgeopvi_fwi2d.so"
LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--fmad=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-Xptxas", "-v",
]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine has no CPU path and must be compiled")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".inc"))]
    deps += [os.path.join(REPO_DIR, "include", h) for h in ("geopvi_fwi2d.h", "geopvi_fwi3d.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def _defines() -> list[str]:
    """Extra preprocessor definitions, e.g. GEOPVI_GB300_DEFINES="NAME=VALUE"."""
    return ["-D" + d for d in os.environ.get("GEOPVI_GB300_DEFINES", "").split() if d]


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every .cu in csrc/ into one shared library; return its path."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = nvcc_path()
    objs = []
    procs = []
    for src in sources():
        obj = os.path.join(LIB_DIR, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *_defines(), "-I", os.path.join(REPO_DIR, "include"), "-c", src, "-o", obj]
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(obj)
    logs = []
    for src, p in procs:
        out, _ = p.communicate()
        logs.append(out)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{out}")
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}")
    os.replace(tmp, LIB_PATH)
    with open(os.path.join(LIB_DIR, "ptxas.log"), "w") as f:
        f.write("\n".join(logs))
    if verbose:
        print("\n".join(logs))
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))

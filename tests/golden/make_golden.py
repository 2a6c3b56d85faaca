"""Generate the golden fixtures from the reference solver itself.

The reference's geopvi/forward/fwi2d/fdtd2D_modelling.c is compiled,
unmodified, by oracle.build() into oracle/_ref/libref_fwi2d.so (with
oracle/stub's FFTW stand-ins, whose transform evaluates FFTW's definition of
the 2-D DFT directly, for the pseudo-spectral cases) and driven through its
own entry points fwi_2D / forward_2D, the way the Cython module aco2d does
(pyacofwi2D.pyx: float64 velocity cast to float32, zeroed outputs).

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py fwi_o8     # selected cases

Run in a checkout where the reference sources are present; the GPU machine only
reads the .npz files written here.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
import cases  # noqa: E402


def to_oracle(p):
    return O.Params(**cases.params_to_dict(p))


def misfit_like_reference(syn: np.ndarray, obs: np.ndarray) -> float:
    """posterior.py:109: 0.5 * np.sum((data_syn - self.data)**2) on float32."""
    return float(0.5 * np.sum((syn - obs) ** 2))


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_small(name: str) -> None:
    c = cases.SMALL[name] if name in cases.SMALL else cases.PSTD[name]
    p = c["params"]
    op = to_oracle(p)
    truth, start = cases.small_models(p, c["seed"])
    obs = O.ref_forward(op, truth.astype(np.float64))
    syn, grad = O.ref_fwi(op, start.astype(np.float64), obs, c["run_fwi"])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), params_json=json.dumps(cases.params_to_dict(p)),
                        run_fwi=c["run_fwi"], truth=truth, start=start, obs=obs, syn=syn, grad=grad,
                        misfit=misfit_like_reference(syn, obs))
    print(f"{name}: |obs| {np.linalg.norm(obs):.4g} |syn| {np.linalg.norm(syn):.4g} |grad| {np.linalg.norm(grad):.4g}")


def make_full(name: str) -> None:
    c = cases.FULL[name]
    p = c["params"]
    op = to_oracle(p)
    truth, start = cases.full_models(name)
    obs = O.ref_forward(op, truth.astype(np.float64))
    syn, grad = O.ref_fwi(op, start.astype(np.float64), obs, c["run_fwi"])
    shot0 = lambda d: d.reshape(p.ns, p.nt, p.nr)[0, :, ::cases.SUBSAMPLE_TRACES].copy()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), params_json=json.dumps(cases.params_to_dict(p)),
                        run_fwi=c["run_fwi"], truth=truth, start=start,
                        obs_sha256=sha(obs), syn_sha256=sha(syn), obs_norm=np.linalg.norm(obs.astype(np.float64)),
                        syn_norm=np.linalg.norm(syn.astype(np.float64)), obs_shot0=shot0(obs),
                        syn_shot0=shot0(syn), grad=grad, misfit=misfit_like_reference(syn, obs))
    print(f"{name}: obs {sha(obs)[:16]} syn {sha(syn)[:16]} |grad| {np.linalg.norm(grad):.4g}")


def main(names):
    if not O.ref_available():
        O.build()
    if not O.ref_available():
        raise SystemExit("reference solver not built: are the reference sources present?")
    for n in names or list(cases.SMALL) + list(cases.PSTD) + list(cases.FULL):
        (make_full if n in cases.FULL else make_small)(n)


if __name__ == "__main__":
    main(sys.argv[1:])

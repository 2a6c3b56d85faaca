"""Observed-data generation in the reference's file format.

The FWI example loads its observed data from ``waveform.npy`` (an
``(ns, nt, nr)`` float32 array, the C layout of record_syn,
fdtd2D_modelling.c:273) and flattens it (examples/fwi2d/fwi2d.py:129-130);
the reference makes such data with ``aco2d.forward`` on the true model.
``generate_waveform`` does the same on the GPU engine, all shots in one
batch: the same float32 values as ``aco2d.forward`` (the forward data are
bit-exact with the reference's solver).
"""
from __future__ import annotations

import numpy as np
import torch

from .engine import Fwi2dEngine
from .params import Params


def generate_waveform(source, vel, path: str | None = None, device=None) -> np.ndarray:
    """source: a Params or a configparser holding the ``[FWI]`` section;
    vel: the true model, nz*nx values (row-major [iz][ix]) of any float type.
    Returns the (ns, nt, nr) float32 data, also saved to ``path`` (.npy) if given."""
    p = source if isinstance(source, Params) else Params.from_config(source)
    v = np.asarray(vel, dtype=np.float64).reshape(-1)
    if v.size != p.ncell:
        raise ValueError(f"vel has {v.size} values, expected nz*nx = {p.ncell}")
    dev = torch.device(device if device is not None else "cuda")
    eng = Fwi2dEngine(p, device=dev, graph=False)
    vt = torch.from_numpy(v.astype(np.float32)[None]).to(dev)
    syn = eng.run(vt, torch.zeros(p.data_len, dtype=torch.float32, device=dev), forward_only=True).syn
    data = syn[0].reshape(p.ns, p.nt, p.nr).cpu().numpy().copy()
    if path is not None:
        np.save(path, data)
    return data

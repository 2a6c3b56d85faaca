"""Small, self-contained run of the time-step kernel for ncu captures.

    python -m geopvi_gb300.profile_step --config cfg2 --solves 140 --nt 400 --nt-interval 10

Runs one misfit + gradient batch of ``solves`` (sample, shot) solves of the
named configuration with ``nt`` shortened, all solves resident at once, no
CUDA graph, then exits.  The wavefield state of 140 cfg2 solves (~200 MB)
exceeds the 129 MB L2, so DRAM counters stay meaningful, while storing every
10th step keeps the stored forward field near 2 GB.  A capture late in the
run (forward launch 300, adjoint launch 699 = time index 100, both stored
steps) sees a developed wavefield rather than the mostly-zero early field.
Prints the device time of the step kernels.
"""
from __future__ import annotations

import argparse
import json

import numpy as np
import torch

from . import workloads
from .engine import Fwi2dEngine


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="cfg2", choices=["cfg1", "cfg2", "cfg3"])
    ap.add_argument("--solves", type=int, default=128)
    ap.add_argument("--nt", type=int, default=100)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--nz", type=int, default=None, help="override the grid (acquisition re-derived)")
    ap.add_argument("--nx", type=int, default=None)
    ap.add_argument("--ns", type=int, default=None)
    ap.add_argument("--nt-interval", type=int, default=None,
                    help="store every n-th step (keeps the stored field small for multi-pass captures)")
    ap.add_argument("--variant", type=int, default=None, help="force a step-kernel variant (default: the tuner)")
    args = ap.parse_args()
    w = getattr(workloads, args.config)()
    p = w.params.replace(nt=args.nt)
    if args.nz or args.nx or args.ns:
        p = workloads.scaled(p, nz=args.nz, nx=args.nx, ns=args.ns)
        base = workloads.smooth(np.ones((p.nz, p.nx)) * 2500.0 + np.linspace(0, 1500, p.nz)[:, None])
        w.samples = np.stack([base.ravel().astype(np.float32)] * w.samples.shape[0])
    if args.nt_interval:
        p = p.replace(nt_interval=args.nt_interval)
    nsamples = max(1, -(-args.solves // p.ns))
    dev = torch.device("cuda:0")
    eng = Fwi2dEngine(p, device=dev, graph=False, max_resident=nsamples * p.ns, variant=args.variant)
    idx = np.arange(nsamples) % w.samples.shape[0]
    vel = torch.from_numpy(np.ascontiguousarray(w.samples[idx])).to(dev)
    obs = torch.zeros(p.data_len, dtype=torch.float32, device=dev)
    for _ in range(args.repeat):
        eng.run(vel, obs, profile=True)
    torch.cuda.synchronize()
    ms, launches = eng.step_profile()
    cells = p.ntp * nsamples * p.ns
    print(json.dumps({"config": args.config, "grid": [p.nz, p.nx], "variant": args.variant, "nt": p.nt,
                      "solves": nsamples * p.ns,
                      "step_launches": launches, "step_ms": ms, "ms_per_launch": ms / max(launches, 1),
                      "padded_cells_per_wave": cells, "gcells_per_s": cells * 2 * p.nt * args.repeat / ms / 1e6}))


if __name__ == "__main__":
    main()

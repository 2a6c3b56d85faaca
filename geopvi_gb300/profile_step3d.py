"""Small, self-contained run of the 3-D engine for ncu captures and timing.

    python -m geopvi_gb300.profile_step3d --n 150 --solves 8 --nt 200 [--forward-only] [--nt-interval 50]

One batch of ``solves`` (sample, shot) solves of an n^3 model
(workloads.fwi3d_workload geometry, 8 shots per sample), all resident, then
exits.  ``--forward-only`` keeps no stored field, and a large
``--nt-interval`` keeps only a few stored steps, so a capture stays within a
few GB of device memory.  Prints the CUDA-event time and cell-updates/s of
the second of two runs.
"""
from __future__ import annotations

import argparse
import json

import torch

from . import fwi3d, workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=150)
    ap.add_argument("--solves", type=int, default=8)
    ap.add_argument("--nt", type=int, default=200)
    ap.add_argument("--nt-interval", type=int, default=1)
    ap.add_argument("--forward-only", action="store_true")
    args = ap.parse_args()
    w = workloads.fwi3d_workload(n=args.n, nt=args.nt, nsamples=max(1, -(-args.solves // 8)))
    p = w.params.replace(nt_interval=args.nt_interval)
    nsamples = w.samples.shape[0]
    dev = torch.device("cuda", 0)
    eng = fwi3d.Fwi3dEngine(p, w.src, w.rec, w.wavelet, device=dev, max_resident=nsamples * p.ns)
    vel = torch.from_numpy(w.samples).to(dev)
    obs = None if args.forward_only else torch.zeros(p.ns * p.nt * p.nr, device=dev)
    for _ in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        r = eng.run(vel, obs, forward_only=args.forward_only)
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    pad = 2 * (p.pml0 + p.Lc + 1)
    ntp = (p.nx + pad) * (p.ny + pad) * (p.nz + pad)
    cu = nsamples * p.ns * p.nt * ntp * (1 if args.forward_only else 2)
    print(json.dumps({"n": args.n, "solves": nsamples * p.ns, "nt": p.nt, "forward_only": args.forward_only,
                      "nt_interval": p.nt_interval, "ms": ms, "launches": r.launches,
                      "gcells_per_s": cu / ms / 1e6}))


if __name__ == "__main__":
    main()

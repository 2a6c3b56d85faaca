#!/usr/bin/env python
"""Benchmark of the GB300 FWI engine: one VI iteration's misfit + gradient batch.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--config cfg2]

A "step" is one pass of the forward/adjoint path over one batch: every
(sample, shot) solve of the configuration (default: the batched VI
iteration, 64 samples x 20 shots on a 200x400 grid, nt 3000), followed by the
per-sample gradient and FP64 misfit reductions.  Inputs are seeded synthetic
models of the configuration's shapes (no dataset is shipped).

Printed as one JSON line by rank 0:
  value   useful FD cell-updates/s (2*ns*nt*ntp per sample), device-timed,
          inputs resident in HBM; max over ranks, summed over replicas
  e2e     the same metric through the public Posterior.fwi call with host
          float64 samples in and host loss/gradient out (copies timed)
  roofline  the time-step kernel: algorithmic bytes per launch / its average
          launch time (CUDA events around the step loops), against the
          measured HBM copy bandwidth
  cpu_baseline  the oracle port of the reference solver (FP32, OpenMP on all
          host cores) on a bounded sample of the same workload
Multi-GPU: replicas only -- each rank solves its own batch, no collective on
the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="cfg2",
                    choices=["cfg1", "cfg2", "cfg3", "cfg4", "cfg5", "fwi3d", "exact"],
                    help="cfg4: uneven batch of 48 instances; cfg5: serving loop; fwi3d: the 3-D engine; "
                         "exact: the exact-gradient mode against the reference gradient (each its own JSON line)")
    ap.add_argument("--requests", type=int, default=40,
                    help="cfg5: requests served at each load (a request is ~6 s of GPU time at capacity)")
    ap.add_argument("--below-saturation", type=float, default=0.7,
                    help="cfg5: the second load, as a fraction of the capacity the first run measured")
    ap.add_argument("--rate", type=float, default=200.0, help="cfg5: mean Poisson arrival rate (req/s)")
    ap.add_argument("--cpu-shots", type=int, default=4, help="shots per sample in the bounded CPU sample")
    ap.add_argument("--cpu-samples", type=int, default=3, help="samples timed in the CPU baseline (median reported)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--hbm-budget-gb", type=float, default=None)
    ap.add_argument("--nt", type=int, default=None, help="shorten the time axis (profiling runs only)")
    return ap.parse_args()


def workload(name: str, nt: int | None = None):
    from geopvi_gb300 import workloads
    if name not in ("cfg1", "cfg2", "cfg3"):
        name = "cfg2"  # the reference arm times the batched VI iteration's per-shot cost
    w = {"cfg1": workloads.cfg1, "cfg2": workloads.cfg2, "cfg3": workloads.cfg3}[name]()
    if nt:
        w.params = w.params.replace(nt=nt)
    return w


WORKLOAD_NAMES = {
    "cfg1": "plain fwi2d misfit+gradient, 120x250 grid, nt 2000, 10 shots, 250 receivers, 4 samples",
    "cfg2": "batched VI iteration, 200x400 grid, nt 3000, 20 shots, 400 receivers, 64 samples",
    "cfg3": "autograd batch, 300x600 grid, nt 4000, dt 0.8 ms, 32 shots, 600 receivers, 16 samples",
}


def cell_updates_per_sample(p) -> int:
    return 2 * p.ns * p.nt * p.ntp


def algorithmic_bytes_per_sample(p) -> int:
    """16 B per propagation cell-update (read p0, p1, v*dt; write p2) plus,
    per interior cell per stored step, 4 B written forward and 12 B in the
    adjoint (read the stored field, read-modify-write the accumulator)."""
    return p.ns * (2 * p.nt * 16 * p.ntp + p.nt_save * 16 * p.ncell)


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle port (or the compiled reference where it loads)
# ---------------------------------------------------------------------------
def cpu_sample(p, vel: np.ndarray, obs_shots: np.ndarray, shots: int):
    """Time the reference arithmetic on the host for `shots` shots of one
    sample; returns (cell-updates/s, seconds, kind, threads, description)."""
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    O.set_threads(threads)
    sub = p.replace(ns=shots)
    op = O.Params(**{k: getattr(sub, k) for k in O.INT_FIELDS + O.FLOAT_FIELDS})
    obs = np.ascontiguousarray(obs_shots.reshape(p.ns, p.nt, p.nr)[:shots]).ravel()
    kind = "port"
    t0 = time.perf_counter()
    if O.ref_available():
        try:
            O.ref_fwi(op, vel.astype(np.float64), obs, 1)
            kind = "reference"
        except OSError:
            O.fwi_f32(op, vel, obs, 1)
    else:
        O.fwi_f32(op, vel, obs, 1)
    dt = time.perf_counter() - t0
    cu = 2 * shots * p.nt * p.ntp
    desc = (f"1 sample x {shots} of {p.ns} shots ({p.nz}x{p.nx}, nt {p.nt}); "
            f"{'compiled reference fdtd2D_modelling.c' if kind == 'reference' else 'FP32 C++ port of fdtd2D_modelling.c'}"
            f", OpenMP {O.get_threads()} threads; cost is linear in shots and samples")
    return cu / dt, dt, kind, O.get_threads(), desc


def cpu_baseline(p, samples: np.ndarray, obs: np.ndarray, shots: int, nsamples: int) -> dict:
    """The CPU baseline line: `nsamples` samples of `shots` shots each, timed
    one after another; the median rate is reported with the spread."""
    runs = [cpu_sample(p, samples[i % len(samples)], obs, shots) for i in range(nsamples)]
    rates = [r[0] for r in runs]
    v = float(statistics.median(rates))
    kind, threads, desc = runs[0][2], runs[0][3], runs[0][4]
    desc = desc.replace("1 sample x", f"median of {nsamples} samples x", 1)
    return {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": kind, "sample": desc,
            "seconds": float(sum(r[1] for r in runs)), "spread": [float(min(rates)), float(max(rates))],
            "sample_gradients_per_s": v / cell_updates_per_sample(p)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    w = workload(args.config, args.nt)
    p = w.params
    # observed data from the truth on the host, with the same port (bounded: the sampled shots only)
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    sub = p.replace(ns=args.cpu_shots)
    op = O.Params(**{k: getattr(sub, k) for k in O.INT_FIELDS + O.FLOAT_FIELDS})
    obs_sub = O.forward_f32(op, w.truth)
    obs = np.zeros(p.data_len, np.float32)
    obs[: obs_sub.size] = obs_sub
    vals = []
    info = None
    for i in range(args.warmup + args.steps):
        v, dt, kind, threads, desc = cpu_sample(p, w.samples[i % len(w.samples)], obs, args.cpu_shots)
        if i >= args.warmup:
            vals.append((v, dt))
        info = (kind, threads, desc)
    value = float(statistics.median([v for v, _ in vals]))  # steps are single samples: the median is steadier
    ms = float(statistics.median([dt for _, dt in vals]) * 1e3)
    kind, threads, desc = info
    out = {
        "impl": "reference", "metric": "FD cell-updates/s (misfit+gradient, fwd+adjoint)", "value": value,
        "unit": "cell-updates/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD_NAMES.get(args.config, WORKLOAD_NAMES["cfg2"]), "sample": desc},
        "sample_gradients_per_s": value / cell_updates_per_sample(p),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": threads, "kind": kind, "sample": desc},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def traffic_per_cell(name: str = "k_step_traffic.json"):
    """DRAM bytes per padded cell-update from a committed ncu summary, or None."""
    path = os.path.join(REPO, "profiles", name)
    if not os.path.exists(path):
        return None
    try:
        t = json.load(open(path))
        return float(t["dram_bytes_per_launch"]) / float(t["padded_cells_per_launch"])
    except (KeyError, ValueError, ZeroDivisionError):
        return None


def load_traffic(p, nres_avg: float):
    """DRAM bytes per step launch from the committed ncu summary, scaled to
    this workload by padded cells per launch (traffic grows in proportion)."""
    per_cell = traffic_per_cell()
    return None if per_cell is None else per_cell * p.ntp * nres_avg


def fwi_config(p):
    """The example's [FWI] config section (config.ini keys) for a parameter set."""
    import configparser
    cfg = configparser.ConfigParser()
    cfg["FWI"] = {"nx": str(p.nx), "nz": str(p.nz), "pml": str(p.pml0), "Lc": str(p.Lc),
                  "laplace_slover": str(p.laplace_solver), "ns": str(p.ns), "nt": str(p.nt), "ds": str(p.ds),
                  "ns0": str(p.ns0), "depths": str(p.depths), "depthr": str(p.depthr), "nr": str(p.nr),
                  "dr": str(p.dr), "nr0": str(p.nr0), "nt_interval": str(p.nt_interval), "dx": repr(p.dx),
                  "dz": repr(p.dz), "dt": repr(p.dt), "f0": repr(p.f0)}
    return cfg


def peak_hbm():
    """(GB/s, 'measured' | 'fallback') from MEASURED_PEAKS.json."""
    pk_path = os.path.join(REPO, "MEASURED_PEAKS.json")
    peaks = json.load(open(pk_path)) if os.path.exists(pk_path) else {}
    return float(peaks.get("hbm_gbs", 6800.0)), ("measured" if "hbm_gbs" in peaks else "fallback")


def run_gpu(args):
    import torch

    from geopvi_gb300.replicas import ReplicaGroup

    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    grp = ReplicaGroup(dev)  # replicas: one batch per rank, host-side barrier and max-time only
    world, rank = grp.world, grp.rank

    from geopvi_gb300.engine import Fwi2dEngine
    w = workload(args.config, args.nt)
    p = w.params
    budget = int(args.hbm_budget_gb * 2**30) if args.hbm_budget_gb else None
    eng = Fwi2dEngine(p, device=dev, graph=False, hbm_budget=budget)
    vel = torch.from_numpy(w.samples).to(dev)
    zeros = torch.zeros(p.data_len, dtype=torch.float32, device=dev)
    obs = eng.run(torch.from_numpy(w.truth).to(dev).unsqueeze(0), zeros, forward_only=True).syn[0].clone()
    nsamples = vel.shape[0]

    barrier = grp.barrier

    for _ in range(args.warmup):
        eng.run(vel, obs, profile=True)
    resident = eng._resident
    torch.cuda.synchronize(dev)
    eng.step_profile()  # discard warm-up spans
    barrier()
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(dev.index if dev.index is not None else 0)
    sampler.start()
    stream = torch.cuda.current_stream(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    launches = 0
    e0.record(stream)
    for _ in range(args.steps):
        r = eng.run(vel, obs, profile=True)
        launches += r.launches
    e1.record(stream)
    torch.cuda.synchronize(dev)
    clocks = sampler.stop()
    barrier()
    ms = e0.elapsed_time(e1)
    step_ms, step_launches = eng.step_profile()
    device_status = eng.status()
    step_variant = eng.tuned_variant(nsamples)  # -1: the tuner was still trying variants
    ms_max = grp.max_seconds(ms / 1e3) * 1e3
    cu_batch = cell_updates_per_sample(p) * nsamples
    value = grp.throughput(args.steps * cu_batch, ms_max / 1e3)
    sgrad = grp.throughput(args.steps * nsamples, ms_max / 1e3)

    # roofline of the time-step kernel
    alg_total = algorithmic_bytes_per_sample(p) * nsamples * args.steps
    achieved = alg_total / (step_ms / 1e3) / 1e9
    peak, peak_src = peak_hbm()
    # step_launches counts time steps of a wave; a wave of many resident
    # solves runs each step as two concurrent launches (one per half of the
    # solves, on two streams), so the per-step figures cover both.
    avg_launch_ms = step_ms / max(step_launches, 1)
    ninst = nsamples * p.ns
    waves = -(-ninst // resident)
    # kernels per run: k_prepare, the step launches, the gradient reduction, two misfit kernels
    kernels_per_step = (launches / args.steps - 4) / (waves * 2 * p.nt)
    nres_avg = ninst * 2 * p.nt * args.steps / max(step_launches, 1)
    traffic = load_traffic(p, nres_avg)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": peak_src, "kernel": "k_step (fused FD step)",
                "avg_launch_ms": avg_launch_ms, "step_share_of_region": step_ms / ms if ms else None,
                "algorithmic_bytes_per_launch": alg_total / max(step_launches, 1),
                "per": "time step of a wave", "kernel_launches_per_time_step": round(kernels_per_step, 3)}

    # plain comparator: one (sample, shot) per launch, shots in order, one sample
    plain = None
    if not args.no_plain:
        peng = Fwi2dEngine(p, device=dev, graph=False, plain=True)
        peng.run(vel[:1], obs)
        torch.cuda.synchronize(dev)
        q0 = torch.cuda.Event(enable_timing=True)
        q1 = torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        peng.run(vel[:1], obs)
        q1.record(stream)
        torch.cuda.synchronize(dev)
        pms = q0.elapsed_time(q1)
        plain = {"sample_gradients_per_s": 1e3 / pms, "cell_updates_per_s": cell_updates_per_sample(p) / (pms / 1e3),
                 "ms_per_sample": pms}
        del peng
        torch.cuda.empty_cache()

    # end to end through the public Posterior.fwi: host float64 samples in, host loss/grad out
    e2e = None
    if not args.no_e2e:
        from geopvi_gb300.posterior import Posterior
        cfg = fwi_config(p)
        del eng
        torch.cuda.empty_cache()
        with tempfile.TemporaryDirectory() as td:
            post = Posterior(obs.cpu().numpy(), cfg, sigma=1.0, paramfile=os.path.join(td, "p.txt"),
                             device=dev, graph=False, hbm_budget=budget)
            x = torch.from_numpy(w.samples.astype(np.float64))
            loss, grad = post.fwi(x)  # warm-up (workspace allocation)
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                loss, grad = post.fwi(x)
            t1 = time.perf_counter()
            e2e_s = t1 - t0
            e2e_s = grp.max_seconds(e2e_s)
            e2e = {"value": args.steps * cu_batch * world / e2e_s, "unit": "cell-updates/s",
                   "h2d_bytes_per_step": int(x.numel() * 8), "d2h_bytes_per_step": int(loss.nbytes + grad.nbytes),
                   "api": "geopvi_gb300.posterior.Posterior.fwi (host float64 in, numpy out)",
                   "sample_gradients_per_s": args.steps * nsamples * world / e2e_s}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(p, w.samples, obs.cpu().numpy(), args.cpu_shots, args.cpu_samples)

    if rank == 0:
        out = {
            "metric": "FD cell-updates/s (misfit+gradient, fwd+adjoint)",
            "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded models)",
            "config": {"workload": WORKLOAD_NAMES[args.config] + (f" (nt shortened to {p.nt})" if args.nt else ""),
                       "samples": nsamples, "shots": p.ns,
                       "grid": f"{p.nz}x{p.nx} (padded {p.ntz}x{p.ntx})", "nt": p.nt, "fd_order": 2 * p.Lc,
                       "resident_solves": resident, "waves": -(-ninst // resident),
                       "fd_step_variant": step_variant,
                       "l2": "inputs larger than L2 (wavefield state of the resident solves >> 129 MB)",
                       "parallelism": f"replicas x{world}"},
            "sample_gradients_per_s": sgrad,
            "plain": plain,
            "batched_vs_plain": (sgrad / world) / plain["sample_gradients_per_s"] if plain else None,
            "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
            "gpu_launches": launches, "device_status": device_status,
        }
        print(json.dumps(out), flush=True)
    grp.close()


# ---------------------------------------------------------------------------
# cfg3: the autograd path with sqrt(nt) checkpoints
# ---------------------------------------------------------------------------
def run_exact(args):
    """The exact discrete-adjoint gradient (GB_FWI2D_EXACT_GRADIENT) against
    the reference's gradient on the same batch: the 200x400, nt 3000, 20-shot
    geometry with 2 samples, full storage, device-resident inputs; CUDA events
    around `steps` calls of each mode after `warmup`."""
    import torch
    from geopvi_gb300.engine import Fwi2dEngine
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    w = workload("cfg2", args.nt)
    p = w.params
    vel = torch.from_numpy(w.samples[:2]).to(dev)
    eng = Fwi2dEngine(p, device=dev, graph=False)
    zeros = torch.zeros(p.data_len, dtype=torch.float32, device=dev)
    obs = eng.run(torch.from_numpy(w.truth).to(dev).unsqueeze(0), zeros, forward_only=True).syn[0].clone()

    def timed(exact):
        for _ in range(args.warmup):
            eng.run(vel, obs, exact=exact)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        launches = 0
        for _ in range(args.steps):
            launches += eng.run(vel, obs, exact=exact).launches
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / args.steps, launches

    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    ref_ms, _ = timed(False)
    ex_ms, launches = timed(True)
    clocks = sampler.stop()
    assert eng.status() == 0
    cells = cell_updates_per_sample(p) * 2
    print(json.dumps({
        "metric": "FD cell-updates/s (misfit + exact gradient, fwd+adjoint)", "value": cells / (ex_ms / 1e3),
        "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ex_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded models)",
        "config": {"workload": "exact gradient: 200x400 grid, nt 3000, 20 shots, 400 receivers, 2 samples, "
                               "full storage of every padded level", "samples": 2,
                   "l2": "inputs larger than L2 (the stored levels of one call: ~58 GB)"},
        "reference_gradient_ms": ref_ms, "exact_over_reference": ex_ms / ref_ms,
        "clocks": clocks, "gpu_launches": launches,
    }), flush=True)


def run_autograd(args):
    """cfg3: log_prob = uniform prior + L2 likelihood through ForwardModel, the
    forward state kept every ~sqrt(nt) steps and each segment recomputed in
    the adjoint.  value: device-resident engine runs (useful cell-updates;
    the recomputed steps are not counted); e2e: Posterior.log_prob(x) ->
    .sum().backward() with host float64 samples in and the host gradient out."""
    import torch
    from geopvi_gb300 import vi
    from geopvi_gb300.engine import Fwi2dEngine
    from geopvi_gb300.posterior import Posterior
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    w = workload("cfg3", args.nt)
    p = w.params
    nsamples = w.samples.shape[0]
    eng = Fwi2dEngine(p, device=dev, graph=False, checkpoint=True)
    zeros = torch.zeros(p.data_len, dtype=torch.float32, device=dev)
    obs = eng.run(torch.from_numpy(w.truth).to(dev).unsqueeze(0), zeros, forward_only=True).syn[0].clone()
    sigma = 0.01 * float(obs.abs().max())  # noise: 1 % of the largest trace amplitude
    vel = torch.from_numpy(w.samples).to(dev)

    def timed(engine, v, steps, warmup, profile=False):
        for _ in range(warmup):
            engine.run(v, obs, profile=profile)
        torch.cuda.synchronize(dev)
        if profile and warmup:
            engine.step_profile()  # discard the warm-up spans
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launches = 0
        e0.record()
        for _ in range(steps):
            launches += engine.run(v, obs, profile=profile).launches
        e1.record()
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1), launches

    for _ in range(args.warmup):
        eng.run(vel, obs, profile=True)
    torch.cuda.synchronize(dev)
    eng.step_profile()
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    ms, launches = timed(eng, vel, args.steps, 0, profile=True)
    clocks = sampler.stop()
    step_ms, step_launches = eng.step_profile()
    resident = eng._resident
    cu_batch = cell_updates_per_sample(p) * nsamples
    value = args.steps * cu_batch / (ms / 1e3)
    # roofline of the step kernel over every launched step (forward, recomputed forward, adjoint)
    alg = nsamples * p.ns * (3 * p.nt * 16 * p.ntp + p.nt_save * 16 * p.ncell) * args.steps
    peak, peak_src = peak_hbm()
    achieved = alg / (step_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": load_traffic(p, nsamples * p.ns * 3 * p.nt * args.steps / max(step_launches, 1)),
                "peak_source": peak_src, "kernel": "k_step (fused FD step)",
                "avg_launch_ms": step_ms / max(step_launches, 1), "step_share_of_region": step_ms / ms,
                "algorithmic_bytes_per_launch": alg / max(step_launches, 1),
                "per": "time step of a wave (forward, recomputed forward and adjoint steps alike)"}
    del eng
    torch.cuda.empty_cache()

    # checkpoint overhead on a resident subset: 8 shots x 2 samples, one wave, both storage modes
    sub = p.replace(ns=8)
    sub_obs = obs.view(p.ns, p.nt, p.nr)[:8].contiguous().view(-1)
    over = {}
    for ck in (False, True):
        e = Fwi2dEngine(sub, device=dev, graph=False, checkpoint=ck, max_resident=16)
        for _ in range(2):
            e.run(vel[:2], sub_obs)
        torch.cuda.synchronize(dev)
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        q0.record()
        e.run(vel[:2], sub_obs)
        q1.record()
        torch.cuda.synchronize(dev)
        over["checkpoint" if ck else "full"] = q0.elapsed_time(q1)
        del e
        torch.cuda.empty_cache()
    overhead = {"subset": "2 samples x 8 shots, 16 solves resident in one wave", "full_storage_ms": over["full"],
                "checkpointed_ms": over["checkpoint"], "ratio": over["checkpoint"] / over["full"]}

    # plain comparator: one (sample, shot) per launch, one sample
    pe = Fwi2dEngine(p, device=dev, graph=False, plain=True)
    pe.run(vel[:1], obs)
    pms, _ = timed(pe, vel[:1], 1, 0)
    plain = {"sample_gradients_per_s": 1e3 / pms, "cell_updates_per_s": cell_updates_per_sample(p) / (pms / 1e3),
             "ms_per_sample": pms}
    del pe
    torch.cuda.empty_cache()

    # end to end through autograd: host float64 samples in, host gradient out
    with tempfile.TemporaryDirectory() as td:
        prior = vi.Uniform(lower=np.full(p.ncell, 1400.0), upper=np.full(p.ncell, 5000.0))
        post = Posterior(obs.cpu().numpy(), fwi_config(p), sigma=sigma, log_prior=prior.log_prob,
                         paramfile=os.path.join(td, "p.txt"), device=dev, graph=False, checkpoint=True)
        x = torch.from_numpy(w.samples.astype(np.float64)).requires_grad_(True)
        for _ in range(2):
            x.grad = None
            post.log_prob(x).sum().backward()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            x.grad = None
            logp = post.log_prob(x)
            logp.sum().backward()
            g = x.grad.numpy()
        e2e_s = time.perf_counter() - t0
        e2e = {"value": args.steps * cu_batch / e2e_s, "unit": "cell-updates/s",
               "h2d_bytes_per_step": int(x.numel() * 8), "d2h_bytes_per_step": int(g.nbytes + logp.numel() * 8),
               "api": "Posterior.log_prob(x).sum().backward() (host float64 samples in, host x.grad out)",
               "sample_gradients_per_s": args.steps * nsamples / e2e_s}

    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(p, w.samples, obs.cpu().numpy(), args.cpu_shots, args.cpu_samples)
    sgrad = args.steps * nsamples / (ms / 1e3)
    print(json.dumps({
        "metric": "FD cell-updates/s (misfit+gradient, fwd+adjoint)", "value": value, "unit": "cell-updates/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded models)",
        "config": {"workload": WORKLOAD_NAMES["cfg3"] + (f" (nt shortened to {p.nt})" if args.nt else ""),
                   "samples": nsamples, "shots": p.ns, "grid": f"{p.nz}x{p.nx} (padded {p.ntz}x{p.ntx})",
                   "nt": p.nt, "storage": "sqrt(nt) checkpoints, segments recomputed in the adjoint",
                   "resident_solves": resident, "waves": -(-(nsamples * p.ns) // resident),
                   "sigma": sigma, "prior": "uniform [1400, 5000] m/s",
                   "l2": "inputs larger than L2 (wavefield state of the resident solves >> 129 MB)"},
        "sample_gradients_per_s": sgrad, "plain": plain, "batched_vs_plain": sgrad / plain["sample_gradients_per_s"],
        "checkpoint_overhead": overhead, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
        "clocks": clocks, "gpu_launches": launches,
    }), flush=True)


# ---------------------------------------------------------------------------
# cfg4 (uneven batch) and cfg5 (serving): whole-job runs through the scheduler
# ---------------------------------------------------------------------------
def _observed(p, truth, dev):
    import torch
    from geopvi_gb300.engine import Fwi2dEngine
    eng = Fwi2dEngine(p, device=dev, graph=False, hbm_budget=8 << 30)
    zeros = torch.zeros(p.data_len, dtype=torch.float32, device=dev)
    obs = eng.run(torch.from_numpy(truth).to(dev).unsqueeze(0), zeros, forward_only=True).syn[0].cpu()
    del eng, zeros
    torch.cuda.empty_cache()
    return obs


def _instance_models(p, rng, nsamples):
    from geopvi_gb300 import workloads
    truth = workloads.gradient_with_anomalies(p.nz, p.nx, p.dx, rng)
    base = workloads.smooth(truth)
    samples = np.stack([base + rng.uniform(-150.0, 150.0, base.shape) for _ in range(nsamples)])
    return truth.astype(np.float32).ravel(), samples.reshape(nsamples, -1).astype(np.float32)


def run_uneven(args):
    """cfg4: 48 instances of mixed grid, shots, nt and f0 submitted at once."""
    import torch
    from geopvi_gb300 import workloads
    from geopvi_gb300.scheduler import FwiServer
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    plist = workloads.cfg4_instances()
    rng = np.random.default_rng(40)
    jobs = []
    t_setup = time.perf_counter()
    for i, p in enumerate(plist):
        truth, samples = _instance_models(p, rng, 1)
        jobs.append((f"inst{i}", p, samples, _observed(p, truth, dev)))
    print(f"cfg4: observed data for {len(jobs)} instances in {time.perf_counter() - t_setup:.1f} s",
          file=sys.stderr, flush=True)
    cells = sum(cell_updates_per_sample(p) for _, p, _, _ in jobs)
    budget = int((args.hbm_budget_gb or 200) * (1 << 30))
    with FwiServer(device=dev, streams=4, hbm_budget=budget) as srv:
        for name, p, _, obs in jobs:
            srv.register(name, p, obs)
        torch.cuda.synchronize(dev)
        sampler = ClockSampler(dev.index or 0)
        sampler.start()
        t0 = time.perf_counter()
        futs = srv.submit_many([(name, vel) for name, _, vel, _ in jobs])
        for k, f in enumerate(futs):
            f.result(timeout=600)
            print(f"cfg4: {k + 1}/{len(futs)} done at {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
        wall = time.perf_counter() - t0
        clocks = sampler.stop()
    print(json.dumps({
        "metric": "FD cell-updates/s (misfit+gradient, fwd+adjoint)", "value": cells / wall,
        "unit": "cell-updates/s", "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": wall * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded models)",
        "config": {"workload": "uneven batch: 48 instances, grids {100x200..400x800}, 4-48 shots, "
                               "nt 1500-5000, Ricker 5-12 Hz, 1 model each, submitted at once",
                   "instances": len(jobs), "cell_updates": cells,
                   "storage": "one fused gb_fwi2d_run_instances call: full storage, waves of mixed instances",
                   "hbm_budget_gb": budget / (1 << 30)},
        "sample_gradients_per_s": len(jobs) / wall, "clocks": clocks,
        "e2e": {"value": cells / wall, "unit": "cell-updates/s",
                "h2d_bytes_per_step": int(sum(v.nbytes for _, _, v, _ in jobs)),
                "d2h_bytes_per_step": int(sum(8 + 4 * p.ncell for _, p, _, _ in jobs)),
                "api": "geopvi_gb300.scheduler.FwiServer (host models in, host results out)"},
    }), flush=True)


def _serve(dev, inv, reqs, gaps, label):
    """Submit `reqs` with the given inter-arrival gaps to a fresh server; wait for all."""
    import torch
    from geopvi_gb300.scheduler import FwiServer, latency_summary
    with FwiServer(device=dev, streams=4) as srv:
        for name, _, p, _, obs in inv:
            srv.register(name, p, obs)
        torch.cuda.synchronize(dev)
        sampler = ClockSampler(dev.index or 0)
        sampler.start()
        t0 = time.perf_counter()
        futs, t_next = [], t0
        for (name, p, vel), gap in zip(reqs, gaps):
            t_next += gap
            delay = t_next - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futs.append(srv.submit(name, vel))
        t_arrivals = time.perf_counter() - t0
        print(f"cfg5 {label}: {len(futs)} requests submitted in {t_arrivals:.1f} s", file=sys.stderr, flush=True)
        for k, f in enumerate(futs):
            f.result(timeout=3600)
            print(f"cfg5 {label}: {k + 1}/{len(futs)} done at {time.perf_counter() - t0:.1f} s",
                  file=sys.stderr, flush=True)
        wall = time.perf_counter() - t0
        clocks = sampler.stop()
        lat = latency_summary(srv.completed)
        queued = [r.t_start - r.t_submit for r in srv.completed]
    cells = sum(cell_updates_per_sample(p) * vel.shape[0] for _, p, vel in reqs)
    grads = sum(vel.shape[0] for _, _, vel in reqs)
    return {"offered_rate_req_per_s": len(reqs) / max(t_arrivals, 1e-9), "requests": len(reqs),
            "arrival_span_s": t_arrivals, "wall_s": wall, "requests_per_s": len(reqs) / wall,
            "sample_gradients_per_s": grads / wall, "cell_updates_per_s": cells / wall,
            "latency": lat, "queue_wait_p50_s": float(np.percentile(queued, 50)),
            "queue_wait_p99_s": float(np.percentile(queued, 99)), "clocks": clocks}


def run_serving(args):
    """cfg5: Poisson arrivals of misfit+gradient requests from 6 inversions,
    served twice: at the stated 200 req/s (far above capacity: latency is
    queueing) and at 0.7x the capacity that run measured (below saturation)."""
    import torch
    from geopvi_gb300 import workloads
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(50)
    grids = [(120, 250), (200, 400), (300, 600), (400, 800)]
    kinds = ["advi", "advi", "flow", "flow", "bvi", "bvi"]      # mean-field ADVI, flows, boosting VI
    batch = {"advi": (4, 8), "flow": (16, 32), "bvi": (8, 16)}  # samples per request
    inv = []
    for i, kind in enumerate(kinds):
        nz, nx = grids[rng.integers(len(grids))]
        p = workloads.make_params(nz, nx, int(rng.integers(2000, 5001)), 1e-3, int(rng.integers(10, 41)),
                                  round(float(rng.uniform(6.0, 12.0)), 2))
        truth, _ = _instance_models(p, rng, 1)
        inv.append((f"{kind}{i}", kind, p, truth, _observed(p, truth, dev)))
    reqs = []
    for _ in range(args.requests):
        name, kind, p, truth, _ = inv[rng.integers(len(inv))]
        lo, hi = batch[kind]
        n = int(rng.integers(lo, hi + 1))
        base = workloads.smooth(truth.reshape(p.nz, p.nx))
        vel = (base[None] + rng.normal(0.0, 60.0, (n,) + base.shape)).reshape(n, -1).astype(np.float32)
        reqs.append((name, p, vel))
    unit_gaps = rng.exponential(1.0, len(reqs))  # Poisson arrivals, scaled per load
    print(f"cfg5: {len(inv)} inversions registered, {len(reqs)} requests drawn", file=sys.stderr, flush=True)
    over = _serve(dev, inv, reqs, unit_gaps / args.rate, f"{args.rate} req/s")
    capacity = over["requests_per_s"]  # the server is busy throughout: its throughput is the capacity
    rate2 = args.below_saturation * capacity
    below = _serve(dev, inv, reqs, unit_gaps / rate2, f"{rate2:.3g} req/s")
    over["load"] = f"the stated {args.rate} req/s: {args.rate / capacity:.0f}x the capacity (queueing)"
    below["load"] = f"{args.below_saturation} x the measured capacity of {capacity:.3g} req/s (below saturation)"
    cells = sum(cell_updates_per_sample(p) * vel.shape[0] for _, p, vel in reqs)
    print(json.dumps({
        "metric": "FD cell-updates/s (misfit+gradient, fwd+adjoint)", "value": over["cell_updates_per_s"],
        "unit": "cell-updates/s", "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": over["wall_s"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded models)",
        "config": {"workload": f"serving: {len(reqs)} requests from 6 inversions (2 ADVI, 2 flow, 2 BVI), "
                               "4-32 samples, grids 120x250..400x800, 10-40 shots, nt 2000-5000, 150 GB "
                               "admission budget, 4 streams; Poisson arrivals at two offered loads",
                   "requests": len(reqs), "samples": int(sum(v.shape[0] for _, _, v in reqs)),
                   "cell_updates": cells},
        "sample_gradients_per_s": over["sample_gradients_per_s"],
        "latency": below["latency"], "loads": [over, below],
        "e2e": {"value": over["cell_updates_per_s"], "unit": "cell-updates/s",
                "h2d_bytes_per_step": int(sum(v.nbytes for _, _, v in reqs)),
                "d2h_bytes_per_step": int(sum(v.shape[0] * (8 + 4 * p.ncell) for _, p, v in reqs)),
                "api": "geopvi_gb300.scheduler.FwiServer (host models in, host results out)"},
        "clocks": below["clocks"],
    }), flush=True)


# ---------------------------------------------------------------------------
# fwi3d: the 3-D engine behind the fwi3d posterior boundary
# ---------------------------------------------------------------------------
def run_fwi3d(args):
    """Misfit + gradient of a batch of 3-D models (workloads.fwi3d_workload):
    device-timed engine runs, the same through the reference-compatible
    Posterior with host arrays, the CPU oracle on one shot."""
    import configparser
    from types import SimpleNamespace
    import torch
    from geopvi_gb300 import fwi3d, workloads
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    w = workloads.fwi3d_workload(nt=args.nt or 600)
    p = w.params
    eng = fwi3d.Fwi3dEngine(p, w.src, w.rec, w.wavelet, device=dev)
    obs = eng.run(torch.from_numpy(w.truth).to(dev).unsqueeze(0), forward_only=True).syn[0].contiguous()
    vel = torch.from_numpy(w.samples).to(dev)
    nsamples = vel.shape[0]
    for _ in range(args.warmup):
        r = eng.run(vel, obs)
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    e0.record()
    for _ in range(args.steps):
        r = eng.run(vel, obs)
        launches += r.launches
    e1.record()
    torch.cuda.synchronize(dev)
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    resident = eng._resident
    pad = 2 * (p.pml0 + p.Lc + 1)
    ntp = (p.nx + pad) * (p.ny + pad) * (p.nz + pad)
    ncell = p.nx * p.ny * p.nz
    nt_save = -(-p.nt // p.nt_interval)
    cu = 2 * p.ns * p.nt * ntp * nsamples * args.steps
    alg = p.ns * nsamples * args.steps * (2 * p.nt * 16 * ntp + nt_save * 16 * ncell)
    peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(REPO, "MEASURED_PEAKS.json")) else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg / (ms / 1e3) / 1e9
    tpc = traffic_per_cell("k3_step_traffic.json")
    traffic3 = None if tpc is None else tpc * ntp * resident
    # end to end through the Posterior: host float64 models in, numpy loss and gradient out
    e2e = None
    with tempfile.TemporaryDirectory() as d:
        for name, arr in (("source", w.src), ("data", obs.cpu().numpy()), ("rec", w.rec), ("wavelet", w.wavelet)):
            np.save(os.path.join(d, name + ".npy"), arr)
        cfg = configparser.ConfigParser()
        cfg["FWI"] = dict(nx=str(p.nx), ny=str(p.ny), nz=str(p.nz), dx=str(p.dx), dy=str(p.dy), dz=str(p.dz),
                          dt=str(p.dt), pml=str(p.pml0), Lc=str(p.Lc), shot_batch=str(p.ns), vel_fixed="1500",
                          recfile=os.path.join(d, "rec.npy"), waveletfile=os.path.join(d, "wavelet.npy"))
        cfg["path"] = dict(inpath=d, outpath=d, srcfile=os.path.join(d, "source.npy"),
                           datafile=os.path.join(d, "data.npy"))
        post = fwi3d.Posterior(SimpleNamespace(sigma=1.0), cfg, device=dev)
        x = w.samples.astype(np.float64)
        post.fwi3d(x)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            loss, grad = post.fwi3d(x)
        wall = time.perf_counter() - t0
        e2e = {"value": cu / wall, "unit": "cell-updates/s", "h2d_bytes_per_step": int(x.nbytes),
               "d2h_bytes_per_step": int(loss.nbytes + grad.nbytes),
               "api": "geopvi_gb300.fwi3d.Posterior.fwi3d (host float64 in, numpy out)"}
        del post
    del eng
    torch.cuda.empty_cache()
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle3d as O3
        sub_nt = min(p.nt, 150)
        sp = p.replace(ns=1, nt=sub_nt)
        obs_sub = O3.run(sp, w.src[:1], w.rec, w.wavelet[:sub_nt], w.truth)[0]
        t0 = time.perf_counter()
        O3.run(sp, w.src[:1], w.rec, w.wavelet[:sub_nt], w.samples[0], obs_sub, grad=True)
        sec = time.perf_counter() - t0
        cpu = {"value": 2 * sub_nt * ntp / sec, "unit": "cell-updates/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"1 sample x 1 of {p.ns} shots, nt {sub_nt} of {p.nt} (cost is linear in shots and "
                         f"steps); FP32 C++ oracle of the 3-D scheme, OpenMP", "seconds": sec}
    print(json.dumps({
        "metric": "FD cell-updates/s (3-D misfit+gradient, fwd+adjoint)", "value": cu / (ms / 1e3),
        "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded models)",
        "config": {"workload": f"3-D batch: {p.nx}x{p.ny}x{p.nz} cells, nt {p.nt}, {p.ns} shots, {p.nr} receivers, "
                               f"{nsamples} samples, 8th order", "resident_solves": resident,
                   "waves": -(-(nsamples * p.ns) // resident),
                   "l2": "inputs larger than L2 (one padded field is 28 MB; the stored field per solve ~10 GB)"},
        "sample_gradients_per_s": nsamples * args.steps / (ms / 1e3),
        "e2e": e2e,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic3, "kernel": "k3_step (3-D step) and its IO kernels, whole run",
                     "per": "time step of a wave: algorithmic and DRAM bytes of one step of the resident "
                            "solves (DRAM scaled from profiles/k3_step_traffic.json by padded cells)",
                     "algorithmic_bytes_per_launch": alg / (args.steps * 2 * p.nt * -(-(nsamples * p.ns) // resident))},
        "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": launches,
    }), flush=True)


def main():
    args = parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "cfg3":
        run_autograd(args)
    elif args.config == "cfg4":
        run_uneven(args)
    elif args.config == "cfg5":
        run_serving(args)
    elif args.config == "fwi3d":
        run_fwi3d(args)
    elif args.config == "exact":
        run_exact(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

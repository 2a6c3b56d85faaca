"""Continuous batching of misfit + gradient requests on one GPU.

GeoPVI evaluates its likelihood one VI iteration at a time, one sample after
another (geopvi/forward/fwi2d/posterior.py:112-149).  This module serves many
such evaluations at once: requests from several inversions (each with its own
grid, acquisition, time axis and observed data) arrive at any time; a
dispatcher thread admits them as HBM and streams free up and merges queued
requests of the same inversion into one batch.  Batches of several
inversions submitted together (submit_many) go to the engine in one
gb_fwi2d_run_instances call, whose waves mix solves of different geometry in
one launch per time step, when the cost model expects that to be faster than
their own plans; every other batch chooses how it holds its forward field
(full storage in waves, or sqrt(nt) checkpoints) from the cost model.  Admitted calls run
concurrently on a pool of CUDA streams.  Observed data stay resident per
inversion; each call's workspace lives only while it runs.

Every kernel is deterministic and a solve never reads another solve's memory,
so a request's result does not depend on what ran beside it (the tests check
this bit for bit).
"""
from __future__ import annotations

import ctypes
import math
import queue
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native
from .params import Params

# Cost model of one time step of a wave on GB300: t = LAUNCH_OVERHEAD_S +
# padded cells x (CELL_S + STRIP_CELL_S x f), f the fraction of the padded
# grid outside the interior (rim and absorbing strips: the step kernel's
# general rows, which cost ~2.5x an interior row).  Least-squares fit to the
# step kernel's measured rates on three grids with full storage of every step
# (f = 0.07: 1000x2000, 8 solves, 218 G cell-updates/s; f = 0.29: 200x400,
# 200 solves, 166 G; f = 0.91: 16x32, 4000 solves, 85 G), within 7 % of each;
# the fixed cost is the latency of one small launch (one 200x400 solve per
# step: ~22 us).
CELL_S = 3.78e-12
STRIP_CELL_S = 8.69e-12
LAUNCH_OVERHEAD_S = 20e-6


def step_seconds(p: Params, resident: int) -> float:
    """Estimated time of one time step of a wave of `resident` solves."""
    strip = 1.0 - (p.nx * p.nz) / p.ntp
    return LAUNCH_OVERHEAD_S + resident * p.ntp * (CELL_S + STRIP_CELL_S * strip)


def fused_seconds(batches: list, cap_bytes: int, lib=None) -> float:
    """Estimated time of one fused gb_fwi2d_run_instances call over
    `batches` [(Params, nsamples)] in cap_bytes: every step of every solve
    (full storage, 2 nt steps) at the step kernel's per-cell cost, plus the
    launches -- a wave's launch serves all its solves, so a pass costs about
    one launch per step of the longest time axis, and the waves are the
    stored fields over the workspace (each batch's nt weighted by its share)."""
    lib = lib or _native.load()
    work = wave_steps = 0.0
    longest = 0
    for p, n in batches:
        strip = 1.0 - (p.nx * p.nz) / p.ntp
        work += 2 * p.nt * n * p.ns * p.ntp * (CELL_S + STRIP_CELL_S * strip)
        wave_steps += p.nt * _ws(lib, p.c(), n, 0, 0) / cap_bytes
        longest = max(longest, p.nt)
    return work + 2 * max(wave_steps, longest) * LAUNCH_OVERHEAD_S


# A batch admitted beside running calls may be planned in the memory they
# leave; it is held back instead when that plan would take more than this
# factor of its time with the whole budget (tiny waves: every launch a
# handful of solves), since waiting for the running calls frees the memory.
SQUEEZE_LIMIT = 1.5


def worth_starting(now_seconds: float, best_seconds: float, others_running: bool) -> bool:
    """Start a batch planned in the memory free now (est. now_seconds), or
    wait for running calls to free more (best_seconds with the whole budget)?"""
    return not others_running or now_seconds <= SQUEEZE_LIMIT * best_seconds


@dataclass
class Plan:
    """How one batch runs: resident solves per wave, storage mode, bytes, cost."""
    resident: int
    checkpoint: bool
    nbytes: int
    est_seconds: float


def _ws(lib, cp, nsamples, resident, flags):
    return int(lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), nsamples, resident, flags))


def plan_batch(p: Params, nsamples: int, cap_bytes: int, lib=None) -> Plan | None:
    """Cheapest (storage mode, wave size) whose workspace fits in cap_bytes.

    Full storage runs 2*nt steps per wave; checkpointing 3*nt but needs
    ~sqrt(nt)/nt_save of the stored field, so more solves fit per wave.  A
    step launch costs step_seconds(p, resident)."""
    lib = lib or _native.load()
    cp = p.c()
    ninst = nsamples * p.ns
    best = None
    for ckpt in (False, True):
        flags = _native.FLAG_CHECKPOINT if ckpt else 0
        base = _ws(lib, cp, nsamples, 1, flags)
        if base == 0 or base > cap_bytes:
            continue
        per = _ws(lib, cp, nsamples, 2, flags) - base if ninst > 1 else 0
        r = ninst if per <= 0 else int(min(ninst, 1 + (cap_bytes - base) // per))
        waves = math.ceil(ninst / r)
        steps = (3 if ckpt else 2) * p.nt
        est = waves * steps * step_seconds(p, r)
        cand = Plan(resident=r, checkpoint=ckpt, nbytes=_ws(lib, cp, nsamples, r, flags), est_seconds=est)
        if best is None or cand.est_seconds < best.est_seconds:
            best = cand
    return best


class Arena:
    """First-fit sub-allocator over one device buffer (256-byte granules).

    The server's workspaces come from here instead of the framework's caching
    allocator, so admission can reason about one contiguous budget and
    requests of changing sizes do not fragment device memory."""

    ALIGN = 256

    def __init__(self, nbytes: int):
        self.size = nbytes // self.ALIGN * self.ALIGN
        self.free = [(0, self.size)]  # sorted (offset, length)

    def largest(self) -> int:
        return max((n for _, n in self.free), default=0)

    def alloc(self, nbytes: int) -> int | None:
        need = (nbytes + self.ALIGN - 1) // self.ALIGN * self.ALIGN
        for i, (off, n) in enumerate(self.free):
            if n >= need:
                if n == need:
                    self.free.pop(i)
                else:
                    self.free[i] = (off + need, n - need)
                return off
        return None

    def release(self, off: int, nbytes: int) -> None:
        need = (nbytes + self.ALIGN - 1) // self.ALIGN * self.ALIGN
        self.free.append((off, need))
        self.free.sort()
        merged = []
        for o, n in self.free:
            if merged and merged[-1][0] + merged[-1][1] == o:
                merged[-1] = (merged[-1][0], merged[-1][1] + n)
            else:
                merged.append((o, n))
        self.free = merged


@dataclass
class Request:
    inversion: str
    vel: torch.Tensor                  # (n, nz*nx) float32, host or device
    want_syn: bool = False
    together: bool = False             # came with others through submit_many
    future: Future = field(default_factory=Future)
    t_submit: float = 0.0
    t_start: float = 0.0
    t_done: float = 0.0

    @property
    def nsamples(self) -> int:
        return int(self.vel.shape[0])


@dataclass
class _Inversion:
    params: Params
    obs: torch.Tensor                  # device-resident observed data
    imaging: bool


@dataclass
class _Part:
    """One inversion's batch within a call: its requests and output tensors."""
    requests: list
    vel: torch.Tensor
    misfit: torch.Tensor
    grad: torch.Tensor
    syn: torch.Tensor | None


@dataclass
class _Running:
    parts: list
    stream: torch.cuda.Stream
    event: torch.cuda.Event
    work_off: int
    work_ptr: int
    plan: Plan
    keep: object = None  # what the enqueued call points at (instance array)

    @property
    def requests(self) -> list:
        return [r for p in self.parts for r in p.requests]


class FwiServer:
    """Dispatcher for misfit + gradient requests.

    hbm_budget: bytes of the one device arena the running batches' workspaces
        are carved from (allocated when the server starts; observed data and
        outputs are separate, small allocations).
    streams: batches that may run at once.
    max_group_samples: queued requests of one inversion merged up to this many
        samples per batch.
    Results are host tensors: misfit float64 (n,), gradient float32 (n, nz*nx)
    in the reference's scaling (the array fwi_2D accumulates), and the
    synthetic data (n, ns*nt*nr) when asked.
    """

    def __init__(self, device=None, hbm_budget: int = 150 << 30, streams: int = 4, max_group_samples: int = 64):
        self.device = torch.device(device if device is not None else "cuda")
        self.lib = _native.load()
        self.budget = int(hbm_budget)
        self.max_group_samples = max_group_samples
        self._streams = [torch.cuda.Stream(self.device) for _ in range(streams)]
        self._free_streams = list(self._streams)
        self._inv: dict[str, _Inversion] = {}
        self._queue: "queue.Queue[Request]" = queue.Queue()
        self._pending: list[Request] = []
        self._running: list[_Running] = []
        self._arena: Arena | None = None
        self._arena_mem: torch.Tensor | None = None
        self._stop = threading.Event()
        self._thread: threading.Thread | None = None
        self.completed: list[Request] = []
        self.busy_seconds = 0.0

    # ---- inversions ----
    def register(self, name: str, params: Params, obs, imaging: bool = False) -> None:
        """Upload an inversion's observed data (ns*nt*nr float32); it stays resident."""
        params.validate()
        obs = torch.as_tensor(np.ascontiguousarray(obs, dtype=np.float32) if not isinstance(obs, torch.Tensor) else obs)
        obs = obs.to(self.device, torch.float32).reshape(-1).contiguous()
        torch.cuda.synchronize(self.device)  # the batches read it from their own streams
        if obs.numel() != params.data_len:
            raise ValueError(f"observed data has {obs.numel()} values, expected {params.data_len}")
        self._inv[name] = _Inversion(params, obs, imaging)

    # ---- requests ----
    def submit(self, name: str, vel, want_syn: bool = False) -> Future:
        r = self._request(name, vel, want_syn)
        self._queue.put(r)
        return r.future

    def submit_many(self, items, want_syn: bool = False) -> list:
        """Submit [(name, vel), ...] at once: the dispatcher sees all of them together."""
        reqs = [self._request(name, vel, want_syn) for name, vel in items]
        for r in reqs:
            r.together = True
        self._queue.put(reqs)
        return [r.future for r in reqs]

    def _request(self, name: str, vel, want_syn: bool) -> Request:
        if name not in self._inv:
            raise KeyError(f"unknown inversion {name!r}")
        vel = vel if isinstance(vel, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(vel, dtype=np.float32))
        if vel.dim() == 1:
            vel = vel.unsqueeze(0)
        if vel.shape[1] != self._inv[name].params.ncell:
            raise ValueError("velocity models do not match the inversion's grid")
        if torch.isnan(vel).any():
            raise ValueError("NaN occured in sample!")
        r = Request(name, vel.to(torch.float32), want_syn)
        r.t_submit = time.perf_counter()
        return r

    def start(self) -> "FwiServer":
        if self._arena_mem is None:
            torch.cuda.empty_cache()
            self._arena_mem = torch.empty(self.budget, dtype=torch.uint8, device=self.device)
            self._arena = Arena(self.budget)
        self._stop.clear()
        self._thread = threading.Thread(target=self._loop, name="fwi-dispatch", daemon=True)
        self._thread.start()
        return self

    def stop(self) -> None:
        self._stop.set()
        if self._thread:
            self._thread.join()
            self._thread = None
        self._arena_mem = None
        self._arena = None

    def __enter__(self):
        return self.start()

    def __exit__(self, *exc):
        self.stop()

    def drain(self, timeout: float | None = None) -> None:
        """Wait until every submitted request finished."""
        t0 = time.perf_counter()
        while True:
            if self._queue.empty() and not self._pending and not self._running:
                return
            if timeout is not None and time.perf_counter() - t0 > timeout:
                raise TimeoutError("requests still running")
            time.sleep(0.002)

    # ---- dispatcher ----
    def _loop(self) -> None:
        torch.cuda.set_device(self.device)
        while not self._stop.is_set():
            try:
                progressed = self._reap()
                while True:
                    try:
                        item = self._queue.get_nowait()
                    except queue.Empty:
                        break
                    self._pending.extend(item if isinstance(item, list) else [item])
                progressed |= self._admit()
            except Exception as e:  # a failure fails the requests it touched, never the loop
                for r in self._pending:
                    if not r.future.done():
                        r.future.set_exception(e)
                self._pending.clear()
                progressed = False
            if not progressed:
                time.sleep(0.0005)
        # finish what runs, fail what never started
        while self._running:
            self._reap()
            time.sleep(0.001)
        for r in self._pending:
            r.future.set_exception(RuntimeError("server stopped before the request ran"))
        self._pending.clear()

    def _reap(self) -> bool:
        done = [g for g in self._running if g.event.query()]
        for g in done:
            self._running.remove(g)
            try:
                g.stream.synchronize()
                st = int(self.lib.gb_fwi2d_status(ctypes.c_void_p(g.work_ptr), ctypes.c_void_p(g.stream.cuda_stream)))
                now = time.perf_counter()
                for part in g.parts:
                    misfit = part.misfit.cpu()
                    grad = part.grad.cpu()
                    syn = part.syn.cpu() if part.syn is not None else None
                    i = 0
                    for r in part.requests:
                        n = r.nsamples
                        r.t_done = now
                        if st != _native.OK:
                            r.future.set_exception(_native.EngineError(st, "device status"))
                        else:
                            res = {"misfit": misfit[i:i + n], "grad": grad[i:i + n]}
                            if r.want_syn and syn is not None:
                                res["syn"] = syn[i:i + n]
                            r.future.set_result(res)
                        self.completed.append(r)
                        i += n
            except Exception as e:  # pragma: no cover - device errors surface here
                for r in g.requests:
                    if not r.future.done():
                        r.future.set_exception(e)
            finally:
                self._arena.release(g.work_off, g.plan.nbytes)
                self._free_streams.append(g.stream)
        return bool(done)

    def _groups(self) -> list:
        """Queued requests merged per inversion, in queue order: [(name, [requests], samples)]."""
        groups: dict = {}
        for r in self._pending:
            g = groups.setdefault(r.inversion, [r.inversion, [], 0])
            if g[2] + r.nsamples <= max(self.max_group_samples, g[1][0].nsamples if g[1] else r.nsamples):
                g[1].append(r)
                g[2] += r.nsamples
        return [tuple(g) for g in groups.values()]

    def _fused_call(self, groups: list, cap: int):
        """The groups (one imaging mode) that one gb_fwi2d_run_instances call
        runs in `cap` bytes, and its workspace size; None if fewer than two fit
        or if the cost model prefers the batches one by one (full storage only:
        where the stored fields dwarf the workspace, waves of a few solves
        cost more than the batches' own plans, which may checkpoint)."""
        imaging = self._inv[groups[0][0]].imaging
        groups = [g for g in groups if self._inv[g[0]].imaging == imaging]
        flags = _native.FLAG_IMAGING if imaging else 0
        while len(groups) > 1:
            insts = (_native.CInstance * len(groups))(*[
                _native.CInstance(self._inv[name].params.c(), n, 1, 1, None, 1, None) for name, _, n in groups])
            need = int(self.lib.gb_fwi2d_instances_workspace_bytes(insts, len(groups), 0, flags))
            if 0 < need <= cap:
                batches = [(self._inv[name].params, n) for name, _, n in groups]
                alone = [plan_batch(p, n, cap, self.lib) for p, n in batches]
                t = fused_seconds(batches, cap, self.lib)
                if self._running and not worth_starting(t, fused_seconds(batches, self.budget, self.lib), True):
                    return None
                if any(a is None for a in alone) or t <= sum(a.est_seconds for a in alone):
                    # room for every solve resident at once, capped by the arena
                    full = sum(_ws(self.lib, p.c(), n, 0, flags) for p, n in batches)
                    return groups, int(min(cap, full + (8 << 20)))
                return None
            groups = groups[:-1]
        return None

    def _admit(self) -> bool:
        admitted = False
        while self._pending and self._free_streams:
            groups = self._groups()
            free = self._arena.largest()
            # a call may take all of the free arena when it runs alone, half otherwise
            cap = free if not self._running else free // 2
            together = [g for g in groups if all(r.together for r in g[1])]
            fused = self._fused_call(together, cap) if len(together) > 1 else None
            if fused is not None:
                sel, nbytes = fused
                for _, reqs, _ in sel:
                    for r in reqs:
                        self._pending.remove(r)
                try:
                    self._launch_fused(sel, nbytes)
                except Exception as e:
                    for _, reqs, _ in sel:
                        for r in reqs:
                            if not r.future.done():
                                r.future.set_exception(e)
                admitted = True
                continue
            name, group, n = groups[0]
            inv = self._inv[name]
            plan = plan_batch(inv.params, n, cap, self.lib)
            if plan is not None and self._running:
                best = plan_batch(inv.params, n, self.budget, self.lib)
                if best is not None and not worth_starting(plan.est_seconds, best.est_seconds, True):
                    break  # squeezed into tiny waves: wait for memory to free up
            if plan is None:
                if not self._running:
                    for r in group:
                        self._pending.remove(r)
                        r.future.set_exception(_native.EngineError(_native.ENOMEM, "request exceeds the HBM budget"))
                    continue
                break  # wait for memory to free up
            for r in group:
                self._pending.remove(r)
            try:
                self._launch(group, inv, plan)
            except Exception as e:
                for r in group:
                    if not r.future.done():
                        r.future.set_exception(e)
            admitted = True
        return admitted

    def _part(self, group: list, inv: _Inversion) -> _Part:
        """Device inputs and outputs of one inversion's batch (on the current stream)."""
        p = inv.params
        n = sum(r.nsamples for r in group)
        want_syn = any(r.want_syn for r in group)
        vel = torch.cat([r.vel.to(self.device, non_blocking=True) for r in group]).contiguous()
        misfit = torch.empty(n, dtype=torch.float64, device=self.device)
        grad = torch.empty(n, p.ncell, dtype=torch.float32, device=self.device)
        syn = torch.empty(n, p.data_len, dtype=torch.float32, device=self.device) if want_syn else None
        return _Part(group, vel, misfit, grad, syn)

    def _launch(self, group: list, inv: _Inversion, plan: Plan) -> None:
        off = self._arena.alloc(plan.nbytes)
        if off is None:
            raise _native.EngineError(_native.ENOMEM, "arena")
        work_ptr = self._arena_mem.data_ptr() + off
        stream = self._free_streams.pop()
        p = inv.params
        now = time.perf_counter()
        for r in group:
            r.t_start = now
        with torch.cuda.stream(stream):
            part = self._part(group, inv)
            flags = (_native.FLAG_IMAGING if inv.imaging else 0) | (_native.FLAG_CHECKPOINT if plan.checkpoint else 0)
            cp = p.c()
            st = self.lib.gb_fwi2d_batch(ctypes.byref(cp), part.vel.shape[0], part.vel.data_ptr(),
                                         inv.obs.data_ptr(), part.syn.data_ptr() if part.syn is not None else None,
                                         part.grad.data_ptr(), part.misfit.data_ptr(), flags, plan.resident,
                                         work_ptr, plan.nbytes, ctypes.c_void_p(stream.cuda_stream))
            event = torch.cuda.Event()
            event.record(stream)
        if st != _native.OK:
            self._free_streams.append(stream)
            self._arena.release(off, plan.nbytes)
            for r in group:
                r.future.set_exception(_native.EngineError(st, "gb_fwi2d_batch"))
            return
        self._running.append(_Running([part], stream, event, off, work_ptr, plan))

    def _launch_fused(self, sel: list, nbytes: int) -> None:
        """One gb_fwi2d_run_instances call over several inversions' batches."""
        off = self._arena.alloc(nbytes)
        if off is None:
            raise _native.EngineError(_native.ENOMEM, "arena")
        work_ptr = self._arena_mem.data_ptr() + off
        stream = self._free_streams.pop()
        now = time.perf_counter()
        imaging = self._inv[sel[0][0]].imaging
        parts, insts = [], []
        with torch.cuda.stream(stream):
            for name, group, _ in sel:
                for r in group:
                    r.t_start = now
                inv = self._inv[name]
                part = self._part(group, inv)
                parts.append(part)
                insts.append(_native.CInstance(inv.params.c(), part.vel.shape[0], part.vel.data_ptr(),
                                               inv.obs.data_ptr(),
                                               part.syn.data_ptr() if part.syn is not None else None,
                                               part.grad.data_ptr(), part.misfit.data_ptr()))
            arr = (_native.CInstance * len(insts))(*insts)
            flags = _native.FLAG_IMAGING if imaging else 0
            st = self.lib.gb_fwi2d_run_instances(arr, len(insts), flags, 0, work_ptr, nbytes,
                                                 ctypes.c_void_p(stream.cuda_stream))
            event = torch.cuda.Event()
            event.record(stream)
        plan = Plan(resident=0, checkpoint=False, nbytes=nbytes, est_seconds=0.0)
        if st != _native.OK:
            self._free_streams.append(stream)
            self._arena.release(off, nbytes)
            for part in parts:
                for r in part.requests:
                    r.future.set_exception(_native.EngineError(st, "gb_fwi2d_run_instances"))
            return
        self._running.append(_Running(parts, stream, event, off, work_ptr, plan, keep=arr))


def latency_summary(requests: list) -> dict:
    """p50 / p99 / max latency (seconds) from submit to result."""
    lat = np.array([r.t_done - r.t_submit for r in requests if r.t_done > 0])
    if lat.size == 0:
        return {"count": 0}
    return {"count": int(lat.size), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "max_s": float(lat.max()), "mean_s": float(lat.mean())}

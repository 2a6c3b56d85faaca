"""Batched GPU solves through the C ABI, with torch for device memory and streams.

``Fwi2dEngine.run`` takes a batch of velocity models already on the GPU and
returns per-sample misfits and gradients (and optionally the synthetic data),
all as CUDA tensors.  It replaces the per-sample ``aco2d.fwi`` loop of
``Posterior.fwi`` (geopvi/forward/fwi2d/posterior.py:112-129) with one
enqueue of every (sample, shot) solve.  The workspace is allocated once per
batch shape and reused; with ``graph=True`` the whole step sequence is
captured once and replayed from a CUDA graph on later calls.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from . import _native
from .params import Params


@dataclass
class RunResult:
    misfit: torch.Tensor          # (n,) float64
    grad: torch.Tensor | None     # (n, nz*nx) float32
    syn: torch.Tensor | None      # (n, ns*nt*nr) float32
    launches: int                 # kernel launches enqueued by the call


def _require_cuda(t: torch.Tensor, name: str, dtype: torch.dtype) -> None:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


class Fwi2dEngine:
    """One solver configuration bound to one CUDA device.

    max_resident: (sample, shot) solves whose wavefield state is held at once;
        None sizes it from ``hbm_budget`` (bytes, default 80% of free memory), in waves of equal size.
    graph: capture the step sequence in a CUDA graph on first use and replay.
    plain: one solve per launch, shots in order -- the comparator form.
    checkpoint: keep the forward state every ~sqrt(nt) steps and recompute
        each segment in the adjoint (for solves whose stored field would not fit).
    """

    def __init__(self, params: Params, device=None, max_resident: int | None = None,
                 hbm_budget: int | None = None, graph: bool = True, plain: bool = False,
                 checkpoint: bool = False, variant: int | None = None):
        self.params = params
        self.lib = _native.load()
        self.device = torch.device(device if device is not None else "cuda")
        if self.device.type != "cuda":
            raise ValueError("the engine runs on CUDA devices only")
        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA device: the GB300 engine has no CPU path")
        params.validate()
        self.max_resident = max_resident
        self.hbm_budget = hbm_budget
        self.graph = graph
        self.plain = plain
        self.checkpoint = checkpoint
        self.variant = variant  # FD step kernel variant; None: the library's tuner picks
        self._cp = params.c()
        self._work: torch.Tensor | None = None
        self._work_key = None
        self._outs = {}

    # ---- sizing ----
    def workspace_bytes(self, nsamples: int, resident: int, flags: int = 0) -> int:
        return int(self.lib.gb_fwi2d_workspace_bytes(ctypes.byref(self._cp), nsamples, resident, flags))

    def per_solve_bytes(self) -> int:
        return self.workspace_bytes(1, 1) if self.params.ns == 1 else \
            self.workspace_bytes(1, 2) - self.workspace_bytes(1, 1)

    def resident_for(self, nsamples: int, flags: int = 0) -> int:
        ninst = nsamples * self.params.ns
        if self.max_resident:
            return max(1, min(self.max_resident, ninst))
        if flags & _native.FLAG_PLAIN:
            return 1
        budget = self.hbm_budget
        if budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            budget = int(free * 0.8)
        base = self.workspace_bytes(nsamples, 1, flags)
        per = max(1, self.workspace_bytes(nsamples, 2, flags) - base) if ninst > 1 else 1
        fit = int(max(1, min(ninst, 1 + max(0, (budget - base) // per))))
        # Equal waves: as many as the budget needs, each as full as the others
        # (a short last wave would run a launch's worth of steps half empty).
        waves = -(-ninst // fit)
        return -(-ninst // waves)

    def _workspace(self, nsamples: int, flags: int) -> tuple[torch.Tensor, int]:
        """One workspace is held at a time; it is sized once per batch shape
        (the resident count is not re-derived from free memory while the
        engine's own workspace occupies part of it)."""
        key = (nsamples, flags & (_native.FLAG_FORWARD_ONLY | _native.FLAG_CHECKPOINT | _native.FLAG_PLAIN |
                                  _native.FLAG_EXACT_GRADIENT))
        if self._work_key != key:
            self._work = None
            self._work_key = None
            if torch.cuda.is_initialized():
                torch.cuda.empty_cache()
            resident = self.resident_for(nsamples, flags)
            nbytes = self.workspace_bytes(nsamples, resident, flags)
            if nbytes == 0:
                raise _native.EngineError(_native.EINVAL, "gb_fwi2d_workspace_bytes")
            self._work = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._work_key = key
            self._resident = resident
        return self._work, self._resident

    # ---- solve ----
    def run(self, vel: torch.Tensor, obs: torch.Tensor, *, imaging: bool = False,
            want_grad: bool = True, want_syn: bool = False, forward_only: bool = False,
            profile: bool = False, exact: bool = False, out: dict | None = None) -> RunResult:
        """vel (n, nz*nx) float32 CUDA; obs (ns*nt*nr,) float32 CUDA.

        Returns misfit (n,) float64, grad (n, nz*nx) float32 in the reference's
        scaling (the array fwi_2D accumulates), syn (n, ns*nt*nr) if asked.
        ``exact=True`` returns instead grad = dJ/dv of the misfit J, the exact
        discrete adjoint of the scheme (no counterpart in the reference).
        Outputs are reused across calls of the same shape unless ``out`` is given.
        """
        p = self.params
        if vel.dim() == 1:
            vel = vel.unsqueeze(0)
        _require_cuda(vel, "vel", torch.float32)
        _require_cuda(obs, "obs", torch.float32)
        n = vel.shape[0]
        if vel.shape[1] != p.ncell:
            raise ValueError(f"vel has {vel.shape[1]} cells per model, expected nz*nx = {p.ncell}")
        if obs.numel() != p.data_len:
            raise ValueError(f"obs has {obs.numel()} values, expected ns*nt*nr = {p.data_len}")
        flags = 0
        if imaging:
            flags |= _native.FLAG_IMAGING
        if self.plain:
            flags |= _native.FLAG_PLAIN
        if self.checkpoint:
            flags |= _native.FLAG_CHECKPOINT
        if profile:
            flags |= _native.FLAG_PROFILE
        elif self.graph and not self.plain:
            flags |= _native.FLAG_GRAPH
        if exact:
            if imaging:
                raise ValueError("the exact gradient is defined for the FWI misfit, not for imaging")
            flags |= _native.FLAG_EXACT_GRADIENT
        if forward_only:
            flags |= _native.FLAG_FORWARD_ONLY
            want_grad = False
            want_syn = True
        if self.variant is not None:
            flags |= _native.flag_variant(self.variant)
        work, resident = self._workspace(n, flags)
        bufs = out if out is not None else self._outs.setdefault((n, want_grad, want_syn), {})
        if "misfit" not in bufs:
            bufs["misfit"] = torch.empty(n, dtype=torch.float64, device=self.device)
        if want_grad and "grad" not in bufs:
            bufs["grad"] = torch.empty(n, p.ncell, dtype=torch.float32, device=self.device)
        if want_syn and "syn" not in bufs:
            bufs["syn"] = torch.empty(n, p.data_len, dtype=torch.float32, device=self.device)
        misfit = bufs["misfit"]
        grad = bufs.get("grad") if want_grad else None
        syn = bufs.get("syn") if want_syn else None
        stream = torch.cuda.current_stream(self.device).cuda_stream
        with torch.cuda.device(self.device):
            st = self.lib.gb_fwi2d_batch(
                ctypes.byref(self._cp), n, vel.data_ptr(), obs.data_ptr(),
                syn.data_ptr() if syn is not None else None,
                grad.data_ptr() if grad is not None else None,
                misfit.data_ptr(), flags, resident, work.data_ptr(), work.numel(), stream)
        _native.check(st, "gb_fwi2d_batch")
        return RunResult(misfit=misfit, grad=grad, syn=syn,
                         launches=int(self.lib.gb_fwi2d_last_launch_count()))

    def tuned_variant(self, nsamples: int, *, imaging: bool = False, forward_only: bool = False,
                      exact: bool = False) -> int:
        """The FD step variant the tuner settled on for batches of ``nsamples``
        run with the given mode (-1 while variants remain untried)."""
        flags = (_native.FLAG_IMAGING if imaging else 0) | (_native.FLAG_PLAIN if self.plain else 0) | \
            (_native.FLAG_CHECKPOINT if self.checkpoint else 0) | \
            (_native.FLAG_FORWARD_ONLY if forward_only else 0) | (_native.FLAG_EXACT_GRADIENT if exact else 0)
        _, resident = self._workspace(nsamples, flags)
        with torch.cuda.device(self.device):
            return int(self.lib.gb_fwi2d_tuned_variant(ctypes.byref(self._cp), nsamples, resident, flags))

    def status(self) -> int:
        """Device status word of the current workspace after the queued work
        finishes: 0, or the C ABI's ETIMEOUT if a bounded wait gave up."""
        if self._work is None:
            return _native.OK
        stream = torch.cuda.current_stream(self.device).cuda_stream
        return int(self.lib.gb_fwi2d_status(ctypes.c_void_p(self._work.data_ptr()), ctypes.c_void_p(stream)))

    def step_profile(self) -> tuple[float, int]:
        """(device ms, launches) of the time-step kernels of every
        ``run(..., profile=True)`` on this thread since the previous read."""
        n = ctypes.c_longlong(0)
        ms = float(self.lib.gb_fwi2d_profile_step_ms(ctypes.byref(n)))
        if ms < 0:
            raise RuntimeError("no profiled run since the last read")
        return ms, int(n.value)

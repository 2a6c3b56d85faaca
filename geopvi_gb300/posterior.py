"""Drop-in for geopvi/forward/fwi2d/posterior.py on the GB300 engine.

``Posterior`` keeps the reference's constructor, attributes and methods
(posterior.py:71-166): ``solver``, ``fwi``, ``fwi_parallel`` and
``log_prob``, the water-layer ``mask`` / ``vel_fixed`` handling and the
``ForwardModel`` autograd Function whose backward scales the saved gradient by
the incoming per-sample gradient (posterior.py:8-24).  What changes is where
the work runs: ``fwi`` sends the whole batch of samples to the GPU in one
enqueue (every sample x shot solve together) instead of looping over
``aco2d.fwi``, observed data and workspace stay resident on the device, and
the misfit is summed in FP64.  ``fwi_parallel`` is the same batched call --
the process pool it replaced has nothing left to parallelise.

Returned values follow the reference: ``solver(vel) -> (loss, -grad[mask])``
and ``fwi(x) -> (loss (m,), grad (m, ndim))``, the gradient in the reference's
own scaling.  A CPU ``x`` gets numpy arrays back, as in the reference; a CUDA
``x`` gets CUDA tensors and nothing leaves the device.
"""
from __future__ import annotations

import numpy as np
import torch
from torch.autograd import Function

from .engine import Fwi2dEngine
from .params import Params, prepare_fwi_parameters


class ForwardModel(Function):
    """loss = func(x) with the gradient computed alongside (posterior.py:8-24)."""

    @staticmethod
    def forward(ctx, input, func):
        output, grad = func(input)
        output = torch.as_tensor(output)
        grad = torch.as_tensor(grad)
        if input.is_cuda:
            output = output.to(input.device)
            grad = grad.to(input.device)
        ctx.save_for_backward(input, grad.to(input.dtype))
        return output.to(input.dtype)

    @staticmethod
    def backward(ctx, grad_output):
        input, grad = ctx.saved_tensors
        return grad_output[..., None] * grad, None


class Posterior:
    def __init__(self, data, config, vel_fixed=1950, sigma=0.1, num_processes=1,
                 log_prior=None, mask=None, paramfile="input_params.txt", device=None,
                 max_resident=None, hbm_budget=None, graph=True, gradient="reference", checkpoint=False):
        """
        data: observed data with shape (ns*nt*nr,), float32
        config: configparser with the ``[FWI]`` section of the example's config.ini
        vel_fixed: velocity of the fixed (masked-out, e.g. water) cells
        sigma: data noise level; log_prob = -loss/sigma^2 + log_prior(x)
        num_processes: accepted for compatibility; the GPU batch replaces the pool
        log_prior: callable x -> log prior (torch)
        mask: boolean array (nz*nx,) -- cells with mask = False are fixed
        paramfile: the positional parameter file written from ``config``
        device / max_resident / hbm_budget / graph: engine placement and sizing
        gradient: "reference" -- the reference's gradient (backward_IO's
            imaging-condition approximation, in its scaling); "exact" -- dJ/dv
            of the misfit, the exact discrete adjoint of the scheme, which a
            finite difference of ``fwi``'s loss converges to
        checkpoint: keep the forward state every ~sqrt(nt) steps and recompute
            each segment in the adjoint instead of storing the whole forward
            field (1.5x the steps; results bit for bit those of full storage)
        """
        if gradient not in ("reference", "exact"):
            raise ValueError(f"gradient must be 'reference' or 'exact', not {gradient!r}")
        self.gradient = gradient
        self.data = data
        self.log_prior = log_prior
        self.num_processes = num_processes
        self.sigma = sigma
        self.vel_water = vel_fixed
        self.paramfile = paramfile
        if mask is None:
            nx = config.getint("FWI", "nx")
            nz = config.getint("FWI", "nz")
            mask = np.full((nx * nz), True)
        self.mask = np.asarray(mask, dtype=bool).reshape(-1)
        prepare_fwi_parameters(self.paramfile, config)
        self.params = Params.from_config(config)
        if self.mask.size != self.params.ncell:
            raise ValueError(f"mask has {self.mask.size} cells, the model has nz*nx = {self.params.ncell}")
        self.device = torch.device(device if device is not None else "cuda")
        self.engine = Fwi2dEngine(self.params, device=self.device, max_resident=max_resident,
                                  hbm_budget=hbm_budget, graph=graph, checkpoint=checkpoint)
        obs = np.ascontiguousarray(np.asarray(data, dtype=np.float32).reshape(-1))
        if obs.size != self.params.data_len:
            raise ValueError(f"data has {obs.size} values, expected ns*nt*nr = {self.params.data_len}")
        self._obs = torch.from_numpy(obs).to(self.device)
        self._mask_dev = torch.from_numpy(self.mask).to(self.device)
        self._last_syn = None

    # ---- per-sample form (posterior.py:101-110) ----
    def solver(self, vel):
        """vel: full model (nz*nx,) float64 -> (loss, -grad[mask])."""
        vel = torch.as_tensor(np.asarray(vel, dtype=np.float64)).to(self.device)
        loss, grad = self._run(vel.to(torch.float32).unsqueeze(0))
        return float(loss[0].item()), grad[0][self._mask_dev].double().cpu().numpy()

    def _full_models(self, x: torch.Tensor) -> torch.Tensor:
        m = x.shape[0]
        vel = torch.full((m, self.mask.size), float(self.vel_water), dtype=torch.float64, device=self.device)
        vel[:, self._mask_dev] = x.to(self.device, torch.float64)
        return vel.to(torch.float32)

    def _run(self, vel32: torch.Tensor):
        """(loss, d loss / d vel): the reference's -grad, or the exact dJ/dv."""
        exact = self.gradient == "exact"
        r = self.engine.run(vel32.contiguous(), self._obs, want_grad=True, exact=exact)
        return r.misfit, (r.grad if exact else -r.grad)

    # ---- batched form (posterior.py:112-149) ----
    def fwi(self, x):
        """x (m, ndim) -> (loss (m,), grad (m, ndim)); numpy for CPU input."""
        on_device = isinstance(x, torch.Tensor) and x.is_cuda
        xt = torch.as_tensor(x.detach() if isinstance(x, torch.Tensor) else np.asarray(x, dtype=np.float64))
        loss, grad = self._run(self._full_models(xt))
        g = grad[:, self._mask_dev].to(torch.float64)
        loss = loss.clone()
        if on_device:
            return loss, g
        return loss.cpu().numpy(), g.cpu().numpy()

    def fwi_parallel(self, x):
        return self.fwi(x)

    def log_prob(self, x):
        """Unnormalised log posterior per sample (posterior.py:151-166)."""
        if torch.isnan(x).any():
            raise ValueError("NaN occured in sample!")
        loss = ForwardModel.apply(x, self.fwi)
        logp = -loss / self.sigma ** 2
        if self.log_prior is not None:
            logp = logp + self.log_prior(x)
        return logp

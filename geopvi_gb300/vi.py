"""A device-resident variational-inversion step for the FWI posterior.

The reference's VI drivers (geopvi/nfvi/flows.py, models.py, geopvi/prior.py)
build some tensors on the CPU inside their forward passes (the structured
``Linear`` kernel's scatter buffer, ``create_lower_triangular``) and evaluate
the smoothing prior with scipy on the host, so one VI iteration crosses the
host twice besides the forward solver.  This module restates the pieces a
batched FWI iteration uses -- the ``Linear`` flow (ADVI / PSVI), the
constraint transforms, the flow-based distribution, the Uniform and Normal
priors with an optional smoothing matrix, and ``VariationalInversion.update``
-- with every tensor on the device of the model's parameters.  Together with
``geopvi_gb300.posterior.Posterior`` on CUDA tensors, an iteration (base
samples, flows, misfit and gradient of every sample x shot, prior, ELBO,
backward, optimizer step) runs without leaving the GPU.

Names, arguments and parameter layouts follow the reference
(flows.py:28-260, models.py:8-140, prior.py:64-170, utils.py:5-54), so a
driver switches by changing its imports.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sparse
import torch
from torch import nn


def _as_tensor(v, dim):
    if v is None:
        return None
    if np.isscalar(v):
        v = np.full((dim,), v)
    return torch.as_tensor(np.asarray(v))


class Real2Constr(nn.Module):
    """Real numbers -> the box (lower, upper): flows.py:28-78."""

    def __init__(self, dim, lower=None, upper=None):
        super().__init__()
        self.dim = dim
        self.register_buffer("lower", _as_tensor(lower, dim))
        self.register_buffer("upper", _as_tensor(upper, dim))

    def forward(self, x, train=True):
        lo, up = self.lower, self.upper
        if lo is None and up is None:
            return x, 0
        if up is None:
            return lo + torch.exp(x), x.sum(axis=-1)
        if lo is None:
            return up - torch.exp(x), x.sum(axis=-1)
        z = lo + (up - lo) / (1 + torch.exp(-x))
        log_det = (torch.log(up - lo) - x - 2 * torch.log(1 + torch.exp(-x))).sum(axis=-1)
        return z, log_det

    def inverse(self, z):
        lo, up = self.lower, self.upper
        if lo is None and up is None:
            return z, 0
        if up is None:
            return torch.log(z - lo), torch.log(1 / (z - lo)).sum(axis=-1)
        if lo is None:
            return torch.log(up - z), torch.log(1 / (up - z)).sum(axis=-1)
        x = torch.log(z - lo) - torch.log(up - z)
        return x, torch.log(1.0 / (z - lo) + 1.0 / (up - z)).sum(axis=-1)


class Constr2Real(Real2Constr):
    """The box (lower, upper) -> real numbers: flows.py:80-129 (Real2Constr reversed)."""

    def forward(self, x, train=True):
        return Real2Constr.inverse(self, x)

    def inverse(self, z):
        return Real2Constr.forward(self, z)


class Linear(nn.Module):
    """z = u + L x (flows.py:131-260).  L = diag(exp(diag)) plus, by kernel:
    'diagonal' nothing (mean-field ADVI); 'fullrank' the strict lower triangle
    (row-major order of np.tril_indices(dim, -1)); 'structured' (PSVI) bands:
    row i of ``mask`` holds the band's coefficients, its True entries taken in
    order land on rows offset_i, offset_i + 1, ... of z (offset_i = number of
    False entries), which for the masks psvi_mask_2D builds is the sub-diagonal
    at distance offset_i.  ``param`` = [u, exp(diag), off-diagonals] as in the
    reference (used to start a high-frequency inversion from a low-frequency
    one)."""

    def __init__(self, dim, kernel="diagonal", mask=None, param=None, trainable=True):
        super().__init__()
        self.dim = dim
        self.kernel = kernel
        self.u = nn.Parameter(torch.zeros(dim))
        self.diag = nn.Parameter(torch.zeros(dim))
        self.non_diag = None
        if kernel == "fullrank":
            self.non_diag = nn.Parameter(torch.zeros(dim * (dim - 1) // 2))
            rows, cols = np.tril_indices(dim, -1)
            self.register_buffer("_tril", torch.from_numpy(np.stack([rows, cols])))
        elif kernel == "structured":
            if mask is None:
                mask = np.ones([1, dim])
                mask[0, -1] = 0.0
            self.mask = np.asarray(mask)
            self.offset = (self.mask == 0).sum(axis=1)
            self.non_diag = nn.Parameter(torch.zeros(self.mask.shape))
            band, src = np.nonzero(self.mask)
            rank = np.concatenate([np.arange(n) for n in (self.mask != 0).sum(axis=1)])
            self.register_buffer("_band", torch.from_numpy(band))
            self.register_buffer("_src", torch.from_numpy(src))
            self.register_buffer("_dst", torch.from_numpy(self.offset[band] + rank))
        elif kernel != "diagonal":
            raise NotImplementedError(f"unknown kernel {kernel!r}")
        if param is not None:
            param = np.asarray(param)
            if param.size >= dim:
                self.u = nn.Parameter(torch.from_numpy(param[:dim].copy()))
            if param.size >= 2 * dim:
                self.diag = nn.Parameter(torch.from_numpy(np.log(param[dim:2 * dim])))
            if param.size > 2 * dim:
                rest = param[2 * dim:]
                if kernel == "fullrank" and rest.size == dim * (dim - 1) // 2:
                    self.non_diag = nn.Parameter(torch.from_numpy(rest.copy()))
                elif kernel == "structured":
                    if rest.size != self.mask.size:
                        raise ValueError("Shape of mask and parameter does not match!")
                    self.non_diag = nn.Parameter(torch.from_numpy(rest.reshape(self.mask.shape).copy()))
        if not trainable:
            for t in (self.u, self.diag, self.non_diag):
                if t is not None:
                    t.requires_grad = False

    def lower_matrix(self):
        d = torch.exp(self.diag)
        L = torch.diag(d)
        if self.kernel == "fullrank":
            L = L.index_put((self._tril[0], self._tril[1]), self.non_diag.to(L.dtype))
        return L

    def forward(self, x, train=True):
        d = torch.exp(self.diag)
        if self.kernel == "fullrank":
            z = self.u + torch.matmul(self.lower_matrix(), x.T).T
        elif self.kernel == "diagonal":
            z = self.u + d * x
        else:
            contrib = x[:, self._src] * self.non_diag[self._band, self._src]
            bands = torch.zeros(x.shape[0], self.dim, dtype=contrib.dtype, device=x.device)
            z = self.u + d * x + bands.index_add(1, self._dst, contrib)
        log_det = torch.log(d).sum().repeat(x.shape[0])
        return z, log_det

    def inverse(self, z):
        d = torch.exp(self.diag)
        if self.kernel == "fullrank":
            x = torch.linalg.solve_triangular(self.lower_matrix(), (z - self.u).T, upper=False).T
        elif self.kernel == "diagonal":
            x = (z - self.u) / d
        else:
            # Banded triangular solve; used to evaluate densities of given
            # samples, not inside the VI iteration -- solved on the host.
            import scipy.sparse.linalg as linalg
            w = self.non_diag.detach().cpu().numpy()
            rows = np.concatenate([np.arange(self.dim), self._dst.cpu().numpy()])
            cols = np.concatenate([np.arange(self.dim), self._src.cpu().numpy()])
            vals = np.concatenate([d.detach().cpu().numpy(), w[self._band.cpu().numpy(), self._src.cpu().numpy()]])
            L = sparse.csr_matrix((vals, (rows, cols)), shape=(self.dim, self.dim))
            rhs = (z - self.u).detach().cpu().numpy().T
            x = torch.from_numpy(linalg.spsolve_triangular(L, rhs, lower=True).T).to(z.device)
        log_det = -torch.log(d).sum().repeat(x.shape[0])
        return x, log_det


class FlowsBasedDistribution(nn.Module):
    """q(z): a base density pushed through the flows (models.py:8-66)."""

    def __init__(self, flows, base="Normal"):
        super().__init__()
        self.flows = nn.ModuleList(flows)
        if base not in ("Normal", "Uniform"):
            raise NotImplementedError("Base distribution provided not currently supported")
        self.base = base
        for flow in flows:
            if hasattr(flow, "dim"):
                self.dim = flow.dim
                break

    def _device(self):
        for p in self.parameters():
            return p.device
        for b in self.buffers():
            return b.device
        return torch.device("cpu")

    def _log_prob_base(self, x):
        if self.base == "Normal":
            return -0.5 * self.dim * math.log(2 * math.pi) - 0.5 * (x ** 2).sum(axis=1)
        return torch.zeros(x.shape[0], dtype=x.dtype, device=x.device)

    def sample_from_base(self, nsamples):
        dev = self._device()
        if self.base == "Normal":
            return torch.randn(nsamples, self.dim, device=dev)
        return torch.rand(nsamples, self.dim, device=dev)

    def forward(self, x):
        log_det = torch.zeros(x.shape[0], device=x.device)
        logq0 = self._log_prob_base(x)
        for flow in self.flows:
            x, ld = flow.forward(x)
            log_det = log_det + ld
        return x, logq0 - log_det

    def inverse(self, z):
        log_det = torch.zeros(z.shape[0], device=z.device)
        for flow in self.flows[::-1]:
            z, ld = flow.inverse(z)
            log_det = log_det + ld
        return z, self._log_prob_base(z) + log_det

    def sample_tensor(self, nsamples):
        """Samples of q on the model's device (no host copy)."""
        with torch.no_grad():
            x = self.sample_from_base(nsamples)
            for flow in self.flows:
                x, _ = flow.forward(x, train=False)
        return x

    def sample(self, nsamples):
        """As the reference: a numpy array."""
        return self.sample_tensor(nsamples).cpu().numpy()


def _to_torch_sparse(m, device=None):
    m = sparse.coo_matrix(m)
    idx = torch.from_numpy(np.vstack([m.row, m.col]).astype(np.int64))
    with torch.sparse.check_sparse_tensor_invariants(True):  # checked here, global setting untouched
        return torch.sparse_coo_tensor(idx, torch.from_numpy(m.data), m.shape, device=device).coalesce()


def _smooth_logp(x, S):
    """-0.5 ||S x||^2 per sample, S sparse on x's device (prior.py:37-60)."""
    if S.device != x.device:
        S = S.to(x.device)
    t = torch.sparse.mm(S.to(x.dtype), x.T)
    return -0.5 * (t ** 2).sum(axis=0)


class Uniform:
    """Uniform prior with optional smoothing (prior.py:64-93)."""

    def __init__(self, lower=np.array([0.0]), upper=np.array([1.0]), smooth_matrix=None, device=None):
        if np.isscalar(upper):
            upper = np.array([upper])
        if np.isscalar(lower):
            lower = np.array([lower])
        self.lower = torch.as_tensor(np.asarray(lower), device=device)
        self.upper = torch.as_tensor(np.asarray(upper), device=device)
        self.smooth_matrix = None if smooth_matrix is None else _to_torch_sparse(smooth_matrix, device)

    def log_prob(self, x):
        logp = -torch.log(self.upper - self.lower).sum(axis=-1).to(x.device)
        if self.smooth_matrix is not None:
            return logp + _smooth_logp(x, self.smooth_matrix)
        return logp


class Normal:
    """Gaussian prior by std, covariance, scale_tril or precision, with optional
    smoothing (prior.py:96-168)."""

    def __init__(self, loc=np.array([0.0]), std=np.array([1.0]), covariance=None, scale_tril=None, precision=None,
                 inverse=False, smooth_matrix=None, device=None):
        import scipy.linalg
        loc = np.asarray(loc)
        self.loc = torch.as_tensor(loc, device=device)
        self.dim = loc.size
        if (covariance is not None) + (scale_tril is not None) + (precision is not None) + (std is not None) != 1:
            raise ValueError("Exactly one of std, covariance or precision or scale_tril may be specified.")
        self.logdet_cov = None
        if std is not None:
            p2, kind = np.asarray(std), "std"
        elif covariance is not None:
            p2, kind = np.linalg.cholesky(covariance), "scale_tril"
        elif scale_tril is not None:
            p2, kind = np.asarray(scale_tril), "scale_tril"
        else:
            p2, kind = np.asarray(precision), "precision"
        if kind == "scale_tril" and inverse:
            self.logdet_cov = np.log(np.diagonal(p2)).sum() * 2
            inv = scipy.linalg.solve_triangular(p2, np.eye(self.dim), lower=True)
            p2, kind = inv.T @ inv, "precision"
        self.param2 = torch.as_tensor(p2, device=device)
        self.param2_type = kind
        self.smooth_matrix = None if smooth_matrix is None else _to_torch_sparse(smooth_matrix, device)

    def log_prob(self, x):
        d = x - self.loc.to(x.device)
        p2 = self.param2.to(x.device)
        c = 0.5 * self.dim * math.log(2 * math.pi)
        if self.param2_type == "std":
            logp = -0.5 * torch.sum((d / p2) ** 2, axis=1) - torch.log(p2).sum() - c
        elif self.param2_type == "precision":
            logp = -0.5 * (torch.tensordot(d, p2, dims=1) * d).sum(axis=-1) - 0.5 * self.logdet_cov - c
        else:
            eps = torch.linalg.solve_triangular(p2, d.T, upper=False).T
            logp = -0.5 * torch.sum(eps ** 2, axis=1) - torch.log(p2.diagonal()).sum() - c
        if self.smooth_matrix is not None:
            return logp + _smooth_logp(x, self.smooth_matrix)
        return logp


class VariationalInversion:
    """Maximise the ELBO of q against log_posterior (models.py:69-140).  The
    loss history stays on the device until update returns."""

    def __init__(self, variationalDistribution, log_posterior):
        self.log_posterior = log_posterior
        self.variationalDistribution = variationalDistribution

    def step(self, optim, nsample):
        """One iteration: base samples, flows, -mean(log p - log q), backward,
        optimizer step.  Returns the loss as a 0-d device tensor."""
        q = self.variationalDistribution
        x = q.sample_from_base(nsample)
        z, logq = q(x)
        logp = self.log_posterior(z)
        negative_elbo = -torch.mean(logp - logq)
        optim.zero_grad()
        negative_elbo.backward()
        optim.step()
        return negative_elbo.detach()

    def update(self, optimizer="torch.optim.Adam", lr=0.001, n_iter=1000, nsample=10, n_out=1, verbose=False,
               **kwargs):
        if isinstance(optimizer, str):
            optim = eval(optimizer)(self.variationalDistribution.parameters(), lr=lr)
        else:
            optim = optimizer
        interval = math.ceil(n_iter / n_out)
        losses = []
        for i in range(n_iter):
            losses.append(self.step(optim, nsample))
            if verbose and i % interval == 0:
                print(f"Iteration: {i:>5d},\tLoss: {float(losses[-1]):>10.2f}")
        return torch.stack(losses).cpu().numpy() if losses else np.zeros(0)


def delta(n):
    """Second-difference matrix with free ends (utils.py:5-10)."""
    d0 = np.full((n,), -2.0)
    d0[0] = d0[-1] = -1.0
    d1 = np.ones(n - 1)
    return sparse.diags([d0, d1, d1], [0, -1, 1]).tocsc()


def smooth_matrix_2D(nx, nz, smoothx, smoothz):
    """Stacked x and z smoothing operators on an [nz, nx] model (utils.py:12-22)."""
    sz = np.full((nz,), smoothz, dtype=float)
    Sx = sparse.kron(sparse.eye(nz) / smoothx, delta(nx))
    Sz = sparse.kron(delta(nz) / sz[:, None], sparse.eye(nx))
    return sparse.vstack([Sx, Sz])


def psvi_mask_2D(correlation, ndim, nx=1, nz=1):
    """Band mask of the structured kernel for a 2-D correlation stencil (utils.py:38-54)."""
    z, x = correlation.shape
    rank = (correlation != 0).sum() // 2
    cz, cx = correlation.size // 2 // x, correlation.size // 2 % x
    mask = np.ones((rank, ndim), dtype=bool)
    i = 0
    for iz in range(z):
        for ix in range(x):
            if correlation[iz, ix] == 0 or iz * x + ix >= correlation.size // 2:
                continue
            off = (cz - iz) * nx + (cx - ix)
            mask[i, -off:] = False
            i += 1
    return mask


def get_flow_param(flow):
    """[u, exp(diag), off-diagonals] of a Linear flow: the layout ``Linear(param=...)``
    reads, saved after one frequency band to start the next
    (examples/fwi3d/fwi3d.py:46-53 in the reference)."""
    mus = flow.u.detach().cpu().numpy()
    sigmas = np.exp(flow.diag.detach().cpu().numpy())
    if flow.non_diag is None:
        return np.hstack([mus, sigmas])
    return np.hstack([mus, sigmas, flow.non_diag.detach().cpu().numpy().ravel()])

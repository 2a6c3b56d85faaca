"""Golden vectors for geopvi_gb300.vi from the reference's own Python modules.

Run in a container that has the reference source tree (it is imported from
there, never at test time):

    python tests/golden/make_vi_golden.py /path/to/reference

Writes tests/golden/vi_golden.npz: Linear flow forward/inverse for the
diagonal, full-rank and structured (PSVI) kernels, the constraint
transforms, a flow-based distribution, the Uniform and Normal priors with a
smoothing matrix (values and gradients), and five Adam iterations of
VariationalInversion.update on a Gaussian target from a fixed seed.
"""
import os
import sys

import numpy as np
import torch

ref = sys.argv[1] if len(sys.argv) > 1 else None
if not ref or not os.path.isdir(os.path.join(ref, "geopvi")):
    sys.exit("usage: make_vi_golden.py <reference source tree>")
sys.path.insert(0, ref)
from geopvi.nfvi import flows as F  # noqa: E402
from geopvi.nfvi import models as M  # noqa: E402
from geopvi import prior as P  # noqa: E402
from geopvi import utils as U  # noqa: E402

torch.set_default_dtype(torch.float64)
rng = np.random.default_rng(7)
nz, nx = 5, 6
dim = nz * nx
n = 4
out = {}

x = rng.standard_normal((n, dim))
out["x"] = x
u = rng.standard_normal(dim)
d = np.exp(0.3 * rng.standard_normal(dim))

# diagonal
param = np.concatenate([u, d])
f = F.Linear(dim, kernel="diagonal", param=param)
z, ld = f.forward(torch.from_numpy(x))
out["diag_param"] = param
out["diag_z"], out["diag_ld"] = z.detach().numpy(), ld.detach().numpy()
xi, li = f.inverse(z)
out["diag_xi"], out["diag_li"] = xi.detach().numpy(), li.detach().numpy()

# full rank
nd = 0.1 * rng.standard_normal(dim * (dim - 1) // 2)
param = np.concatenate([u, d, nd])
f = F.Linear(dim, kernel="fullrank", param=param)
z, ld = f.forward(torch.from_numpy(x))
out["full_param"] = param
out["full_z"], out["full_ld"] = z.detach().numpy(), ld.detach().numpy()

# structured (PSVI) with the 2-D mask of a 3x3 correlation stencil
mask = U.psvi_mask_2D(np.ones((3, 3)), dim, nx=nx, nz=nz)
nd = 0.1 * rng.standard_normal(mask.shape)
param = np.concatenate([u, d, nd.ravel()])
f = F.Linear(dim, kernel="structured", mask=mask, param=param)
z, ld = f.forward(torch.from_numpy(x))
out["psvi_mask"] = mask
out["psvi_param"] = param
out["psvi_z"], out["psvi_ld"] = z.detach().numpy(), ld.detach().numpy()

# constraint transforms and a flow-based distribution
lower = 1500.0 + 100.0 * rng.random(dim)
upper = lower + 1000.0 + 500.0 * rng.random(dim)
out["lower"], out["upper"] = lower, upper
r2c = F.Real2Constr(dim, lower=lower, upper=upper)
zc, ldc = r2c.forward(torch.from_numpy(x))
out["r2c_z"], out["r2c_ld"] = zc.numpy(), ldc.numpy()
xc, lic = r2c.inverse(zc)
out["r2c_xi"], out["r2c_li"] = xc.numpy(), lic.numpy()
c2r = F.Constr2Real(dim, lower=0.0, upper=1.0)
ub = rng.random((n, dim))
out["ub"] = ub
zz, ll = c2r.forward(torch.from_numpy(ub))
out["c2r_z"], out["c2r_ld"] = zz.numpy(), ll.numpy()
q = M.FlowsBasedDistribution([F.Linear(dim, kernel="structured", mask=mask, param=param),
                              F.Real2Constr(dim, lower=lower, upper=upper)], base="Normal")
zq, lq = q(torch.from_numpy(x))
out["q_z"], out["q_logq"] = zq.detach().numpy(), lq.detach().numpy()

# priors with smoothing
S = U.smooth_matrix_2D(nx, nz, 2.0, 3.0)
xm = torch.from_numpy(0.5 * (lower + upper) + 50.0 * x).requires_grad_(True)
pu = P.Uniform(lower=lower, upper=upper, smooth_matrix=S)
lp = pu.log_prob(xm)
lp.sum().backward()
out["xm"] = xm.detach().numpy()
out["unif_logp"], out["unif_grad"] = lp.detach().numpy(), xm.grad.numpy().copy()
xm.grad = None
pn = P.Normal(loc=0.5 * (lower + upper), std=np.sqrt((upper - lower) ** 2 / 12), smooth_matrix=S)
lp = pn.log_prob(xm)
lp.sum().backward()
out["norm_logp"], out["norm_grad"] = lp.detach().numpy(), xm.grad.numpy().copy()

# five Adam iterations of the VI update on a Gaussian target
mu_t = rng.standard_normal(dim)
out["mu_t"] = mu_t


def log_post(zs):
    return -0.5 * ((zs - torch.from_numpy(mu_t)) ** 2).sum(axis=1) / 0.25


torch.manual_seed(123)
q = M.FlowsBasedDistribution([F.Linear(dim, kernel="diagonal")], base="Normal")
vi = M.VariationalInversion(q, log_post)
loss = vi.update(lr=0.05, n_iter=5, nsample=8)
out["vi_loss"] = np.asarray([float(v) for v in loss])
out["vi_u"] = q.flows[0].u.detach().numpy()
out["vi_diag"] = q.flows[0].diag.detach().numpy()

np.savez(os.path.join(os.path.dirname(os.path.abspath(__file__)), "vi_golden.npz"), **out)
print("wrote", len(out), "arrays")

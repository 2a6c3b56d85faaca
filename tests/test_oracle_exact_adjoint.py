"""The oracle's exact discrete adjoint against central finite differences (CPU).

``exact_grad_f64`` transposes the FD scheme step by step (stencil, boundary
blends, source, padding).  A central difference of the FP64 misfit with
h = 1e-2 m/s converges to it at O(h^2), so on 50 random cells plus the
corners and edges of the model (the cells whose gradient collects the
replicated padding) the two agree to ~1e-8 relative.  The reference's own
gradient (backward_IO, fdtd2D_modelling.c:941-978) is a continuous-adjoint
approximation: it points the same way to within a modest angle and is about
dt times smaller, which the last test records.
"""
import numpy as np
import pytest

import cases

H = 1e-2  # m/s


def oparams(O, p):
    return O.Params(**cases.params_to_dict(p))


def fd_cells(p, n_random, seed):
    rng = np.random.default_rng(seed)
    nz, nx = p.nz, p.nx
    edge = [(0, 0), (0, nx - 1), (nz - 1, 0), (nz - 1, nx - 1), (0, nx // 2), (nz // 2, 0),
            (nz - 1, nx // 3), (nz // 3, nx - 1)]
    cells = [iz * nx + ix for iz, ix in edge]
    cells += [int(c) for c in rng.choice(nz * nx, n_random, replace=False)]
    return sorted(set(cells))


@pytest.mark.parametrize("name,n_random", [("fwi_o8", 50), ("fwi_ragged", 50), ("fwi_pml1", 20),
                                           ("fwi_o12", 20)])
def test_exact_gradient_matches_central_difference(oracle, name, n_random):
    z = np.load(f"{cases.__file__.rsplit('/', 1)[0]}/{name}.npz")
    p = cases.params_from_npz(z)
    op = oparams(oracle, p)
    vel = z["start"].astype(np.float64)
    obs = z["obs"].astype(np.float64)
    J, g = oracle.exact_grad_f64(op, vel, obs)
    assert J == pytest.approx(oracle.misfit_f64(op, vel, obs), rel=1e-12)
    cells = fd_cells(p, n_random, seed=cases.SMALL[name]["seed"])
    fd = np.empty(len(cells))
    for i, c in enumerate(cells):
        vp = vel.copy()
        vp[c] += H
        vm = vel.copy()
        vm[c] -= H
        fd[i] = (oracle.misfit_f64(op, vp, obs) - oracle.misfit_f64(op, vm, obs)) / (2 * H)
    ge = g[cells]
    scale = np.max(np.abs(fd))
    assert np.max(np.abs(ge - fd)) <= 1e-6 * scale, (name, np.max(np.abs(ge - fd)) / scale)


def test_reference_gradient_is_a_scaled_approximation(oracle):
    """-grad_ref ~ dt * dJ/dv in direction (cosine > 0.8) on the 8th-order case."""
    z = np.load(f"{cases.__file__.rsplit('/', 1)[0]}/fwi_o8.npz")
    p = cases.params_from_npz(z)
    op = oparams(oracle, p)
    _, g = oracle.exact_grad_f64(op, z["start"].astype(np.float64), z["obs"].astype(np.float64))
    gref = -z["grad"].astype(np.float64)
    cos = float(g @ gref / (np.linalg.norm(g) * np.linalg.norm(gref)))
    scale = float(g @ gref / (gref @ gref))
    assert cos > 0.8
    assert 0.5 / p.dt < scale < 3.0 / p.dt

"""The 3-D oracle against a second restatement of the scheme, in numpy.

include/geopvi_fwi3d.h states the 3-D scheme step by step; oracle/fwi3d_oracle.cpp
(loops, C++) and the engine follow it.  This file restates it a third way --
whole-array numpy operations over the padded grid, the six absorbing passes
as slices, the adjoint and gradient from the same definitions -- and checks
the oracle against it on small grids.  numpy has no fused multiply-add, so
fma(a, b, c) is the FP64 value a*b + c (a*b exact) rounded to FP32; that can
differ from a single rounding by one ulp in rare cases, hence a tolerance
(1e-6 relative) instead of bit equality.  No GPU.
"""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import oracle3d as O

F = np.float32


def fma(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(F)


WEIGHTS = {
    3: [-49.0 / 18, 1.5, -3.0 / 20, 1.0 / 90],
    4: [-205.0 / 72, 8.0 / 5, -1.0 / 5, 8.0 / 315, -1.0 / 560],
    5: [-73766.0 / 25200, 42000.0 / 25200, -6000.0 / 25200, 1000.0 / 25200, -125.0 / 25200, 8.0 / 25200],
}


class Spec:
    def __init__(self, p):
        self.p = p
        self.L = p.Lc + 1
        self.pml = p.pml0 + self.L
        self.n = (p.nz + 2 * self.pml, p.ny + 2 * self.pml, p.nx + 2 * self.pml)  # (z, y, x)
        self.c = [F(w) for w in WEIGHTS[p.Lc]]
        d = (p.dz, p.dy, p.dx)  # axis order z, y, x
        self.id = [F(1.0 / float(v)) for v in d]
        self.id2 = [F(1.0 / (float(v) * float(v))) for v in d]
        self.idt2 = F(1.0 / (float(p.dt) * float(p.dt)))
        self.w = [F(1.0 - i / p.pml0) for i in range(p.pml0)]
        self.omw = [F(1.0 - float(w)) for w in self.w]

    def pad(self, vel):
        v = np.asarray(vel, F).reshape(self.p.ny, self.p.nx, self.p.nz).transpose(2, 0, 1)  # (z, y, x)
        return np.pad(v, self.pml, mode="edge")

    def step(self, vd, p0, p1):
        L, H = self.L, self.p.Lc
        nz, ny, nx = self.n
        q = np.zeros_like(p1)
        core = (slice(L, nz - L), slice(L, ny - L), slice(L, nx - L))

        def sh(a, axis, m):  # a shifted by m cells along axis, over the core
            sl = list(core)
            sl[axis] = slice(core[axis].start + m, core[axis].stop + m)
            return a[tuple(sl)]
        pc = p1[core]
        lap = [self.c[0] * pc for _ in range(3)]
        for m in range(1, H + 1):
            for a in range(3):
                lap[a] = fma(self.c[m], sh(p1, a, m) + sh(p1, a, -m), lap[a])
        t = lap[0] * self.id2[0]
        t = fma(lap[1], self.id2[1], t)
        t = fma(lap[2], self.id2[2], t)
        u = fma(F(2), pc, -p0[core])
        q[core] = fma(vd[core] * vd[core], t, u)
        # faces: z, y, x; min side then max side, each over the full other axes
        for a in range(3):
            for side in (0, 1):
                idx = range(L, self.pml) if side == 0 else range(self.n[a] - self.pml, self.n[a] - L)
                for i in idx:
                    wi = i - L if side == 0 else self.n[a] - L - 1 - i
                    d = 1 if side == 0 else -1

                    def plane(arr, off):
                        sl = [slice(None)] * 3
                        sl[a] = i + off * d
                        return arr[tuple(sl)]
                    s = plane(vd, 0) * self.id[a]
                    t11 = ((F(2) - s) * (F(1) - s)) * F(0.5)
                    t12 = s * (F(2) - s)
                    t13 = (s * (s - F(1))) * F(0.5)
                    k0, k1, k2 = F(2) * t11, F(2) * t12, F(2) * t13
                    k3, k4 = t11 * t11, k0 * t12
                    k5 = fma(t12, t12, k0 * t13)
                    k6, k7 = k1 * t13, t13 * t13
                    e = k0 * plane(p1, 0)
                    e = fma(k1, plane(p1, 1), e)
                    e = fma(k2, plane(p1, 2), e)
                    for kk, k in enumerate((k3, k4, k5, k6, k7)):
                        e = fma(-k, plane(p0, kk), e)
                    sl = [slice(None)] * 3
                    sl[a] = i
                    q[tuple(sl)] = fma(self.w[wi], e, self.omw[wi] * q[tuple(sl)])
        return q

    def run(self, src, rec, wav, vel, obs):
        p, pml = self.p, self.pml
        v = self.pad(vel)
        vd = v * F(p.dt)
        inner = (slice(pml, -pml), slice(pml, -pml), slice(pml, -pml))
        nti = p.nt_interval
        ns = len(src)
        syn = np.zeros((ns, p.nt, len(rec)), F)
        G = np.zeros((p.nz, p.ny, p.nx), np.float64)
        for s in range(ns):
            sx, sy, sz = src[s]
            vs = np.asarray(vel, F).reshape(p.ny, p.nx, p.nz)[sy, sx, sz]
            f = [np.zeros(self.n, F) for _ in range(3)]
            snaps = {}
            for it in range(p.nt):
                p0, p1 = f[0], f[1]
                p2 = self.step(vd, p0, p1)
                p2[sz + pml, sy + pml, sx + pml] += (((F(wav[it]) * F(p.dt)) * F(p.dt)) * vs) * vs
                if it % nti == 0:
                    snaps[it] = (p2[inner] - fma(F(2), p1[inner], -p0[inner])) * self.idt2
                for r, (rx, ry, rz) in enumerate(rec):
                    syn[s, it, r] = p2[rz + pml, ry + pml, rx + pml]
                f = [p1, p2, p0]
            lam = [np.zeros(self.n, F) for _ in range(3)]
            Gs = np.zeros((p.nz, p.ny, p.nx), F)
            for it in range(p.nt - 1, -1, -1):
                q0, q1 = lam[0], lam[1]
                q2 = self.step(vd, q0, q1)
                if it % nti == 0:
                    Gs = fma(snaps[it], q2[inner], Gs)
                for r, (rx, ry, rz) in enumerate(rec):
                    inj = syn[s, it, r] - F(obs[s, it, r])
                    q2[rz + pml, ry + pml, rx + pml] += inj
                    if it % nti == 0:
                        Gs[rz, ry, rx] = fma(snaps[it][rz, ry, rx], inj, Gs[rz, ry, rx])
                lam = [q1, q2, q0]
            G += Gs
        vm = np.asarray(vel, F).reshape(p.ny, p.nx, p.nz).astype(np.float64)
        grad = (2.0 * (nti * float(p.dt) * float(p.dt)) * G.transpose(1, 2, 0) / vm).astype(F)
        return syn, grad.ravel()


@pytest.mark.parametrize("Lc,nti,pml0", [(4, 1, 3), (3, 2, 2), (5, 3, 1)])
def test_oracle_matches_numpy_restatement(Lc, nti, pml0):
    p = SimpleNamespace(nx=6, ny=5, nz=7, pml0=pml0, Lc=Lc, ns=2, nr=5, nt=40, nt_interval=nti,
                        dx=10.0, dy=12.0, dz=9.0, dt=1e-3)
    rng = np.random.default_rng(Lc + 10 * nti)
    src = np.array([[1, 2, 0], [4, 3, 2]])
    rec = np.array([[0, 0, 0], [5, 4, 6], [2, 2, 3], [2, 2, 3], [3, 1, 1]])
    t = np.arange(p.nt) * p.dt - 1 / 30.0
    a = (np.pi * 30 * t) ** 2
    wav = ((1 - 2 * a) * np.exp(-a)).astype(F)
    truth = (1800 + 500 * rng.random(p.nx * p.ny * p.nz)).astype(F)
    vel = (truth + rng.uniform(-100, 100, truth.shape)).astype(F)
    obs = O.run(p, src, rec, wav, truth)[0]
    syn_o, grad_o, _ = O.run(p, src, rec, wav, vel, obs, grad=True)
    syn_s, grad_s = Spec(p).run(src, rec, wav, vel, obs)
    assert np.abs(syn_o).max() > 0 and np.abs(grad_o).max() > 0
    assert np.abs(syn_o - syn_s).max() <= 1e-6 * np.abs(syn_o).max()
    assert np.abs(grad_o - grad_s).max() <= 1e-5 * np.abs(grad_o).max()

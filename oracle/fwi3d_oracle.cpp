/*
 * fwi3d_oracle.cpp -- CPU restatement of the 3-D acoustic FWI scheme.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA 3-D engine
 * in geopvi_gb300/: only tests/ and bench.py's cpu_baseline leg load it.  The
 * product never links or calls it.
 *
 * The reference's 3-D posterior (geopvi/forward/fwi3d/posterior.py:44-77)
 * drives an external executable that it does not ship, so there is no
 * reference arithmetic to restate here; parity for the 3-D engine is parity
 * with this file, which spells out the scheme documented in
 * include/geopvi_fwi3d.h: the 2-D reference's algorithm
 * (geopvi/forward/fwi2d/fdtd2D_modelling.c) on three axes:
 *   fd_coefficient weights                fdtd2D_modelling.c:1272-1326
 *   get_velp edge padding                 fdtd2D_modelling.c:1187-1238
 *   absorbing weights w = 1 - i/pml0,
 *   s = v dt / d, t11, t12, t13           fdtd2D_modelling.c:220-240
 *   stencil step (fdtd_2d_calculate_p)    fdtd2D_modelling.c:756-780
 *   hybrid one-way boundary (abc_for_p)   fdtd2D_modelling.c:833-900
 *   source / receivers (forward_IO)       fdtd2D_modelling.c:902-939
 *   residual injection, imaging term
 *   (backward_IO, scaled as the discrete
 *   adjoint of the step)                  fdtd2D_modelling.c:941-978
 *   forward / adjoint time loops          fdtd2D_modelling.c:678-753
 *
 * Every operation is FP32 with fused multiply-adds written as fmaf; build
 * with -ffp-contract=off so the compiler adds none (the Makefile does).
 * Fields are [z][y][x] (x fastest) over the padded grid.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../include/geopvi_fwi3d.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { kOk = 0, kEinval = -22 };

/* fd_coefficient (fdtd2D_modelling.c:1292-1325) for Lc' = Lc + 1 = 4..7:
 * double literals rounded to float. */
void fd_weights(int L, float *c)
{
    switch (L) {
    case 4:
        c[0] = (float)(-49.0 / 18); c[1] = 1.5f; c[2] = (float)(-3.0 / 20); c[3] = (float)(1.0 / 90);
        break;
    case 5:
        c[0] = (float)(-205.0 / 72); c[1] = (float)(8.0 / 5); c[2] = (float)(-1.0 / 5);
        c[3] = (float)(8.0 / 315); c[4] = (float)(-1.0 / 560);
        break;
    case 6:
        c[0] = (float)(-73766.0 / 25200); c[1] = (float)(42000.0 / 25200); c[2] = (float)(-6000.0 / 25200);
        c[3] = (float)(1000.0 / 25200); c[4] = (float)(-125.0 / 25200); c[5] = (float)(8.0 / 25200);
        break;
    default: {
        const double den = 7.820582005659452e+44;
        c[0] = (float)(-2.332705821577166e+45 / den); c[1] = (float)(1.3406712009703548e+45 / den);
        c[2] = (float)(-2.0947987515168676e+44 / den); c[3] = (float)(4.13787407707198e+43 / den);
        c[4] = (float)(-6.982662505061379e+42 / den); c[5] = (float)(8.12528000589218e+41 / den);
        c[6] = (float)(-4.702129633040854e+40 / den);
        break;
    }
    }
}

struct Geo {
    int L, H, pml, pml0;
    int ntx, nty, ntz, nx, ny, nz;
    long long sy, sz, ntp;  /* strides of y and z, padded cells */
    float c[8];
    float id[3];            /* 1/dx, 1/dy, 1/dz (s = v dt / d along a face normal) */
    float id2[3];           /* 1/dx^2, 1/dy^2, 1/dz^2 */
    float idt2, dt;
    std::vector<float> w, omw;
};

int make_geo(const gb_fwi3d_params &p, Geo &g)
{
    if (p.nx < 1 || p.ny < 1 || p.nz < 1 || p.pml0 < 1 || p.Lc < 3 || p.Lc > 6 || p.ns < 1 || p.nr < 1 ||
        p.nt < 1 || p.nt_interval < 1 || !(p.dx > 0) || !(p.dy > 0) || !(p.dz > 0) || !(p.dt > 0))
        return kEinval;
    g.L = p.Lc + 1;
    g.H = p.Lc;
    g.pml0 = p.pml0;
    g.pml = p.pml0 + g.L;
    g.nx = p.nx; g.ny = p.ny; g.nz = p.nz;
    g.ntx = p.nx + 2 * g.pml; g.nty = p.ny + 2 * g.pml; g.ntz = p.nz + 2 * g.pml;
    g.sy = g.ntx;
    g.sz = (long long)g.ntx * g.nty;
    g.ntp = g.sz * g.ntz;
    fd_weights(g.L, g.c);
    const double d[3] = {p.dx, p.dy, p.dz};
    for (int a = 0; a < 3; ++a) {
        g.id[a] = (float)(1.0 / d[a]);
        g.id2[a] = (float)(1.0 / (d[a] * d[a]));
    }
    g.idt2 = (float)(1.0 / ((double)p.dt * (double)p.dt));
    g.dt = p.dt;
    g.w.resize(p.pml0);
    g.omw.resize(p.pml0);
    for (int i = 0; i < p.pml0; ++i) {
        g.w[i] = (float)(1.0 - (double)i / p.pml0);
        g.omw[i] = (float)(1.0 - (double)g.w[i]);
    }
    return kOk;
}

/* get_velp: the padded cell's velocity is the model value at the clamped
 * interior position; model order (ny, nx, nz), nz fastest. */
inline float vpad(const Geo &g, const float *vel, int x, int y, int z)
{
    const int jx = std::min(std::max(x - g.pml, 0), g.nx - 1);
    const int jy = std::min(std::max(y - g.pml, 0), g.ny - 1);
    const int jz = std::min(std::max(z - g.pml, 0), g.nz - 1);
    return vel[((long long)jy * g.nx + jx) * g.nz + jz];
}

/* The absorbing blend's eight coefficients from s = v dt / d:
 * 2 t11, 2 t12, 2 t13, t11^2, 2 t11 t12, t12^2 + 2 t11 t13, 2 t12 t13, t13^2. */
inline void abc_coef(float s, float *k)
{
    const float t11 = ((2.0f - s) * (1.0f - s)) * 0.5f;
    const float t12 = s * (2.0f - s);
    const float t13 = (s * (s - 1.0f)) * 0.5f;
    k[0] = 2.0f * t11;
    k[1] = 2.0f * t12;
    k[2] = 2.0f * t13;
    k[3] = t11 * t11;
    k[4] = k[0] * t12;
    k[5] = std::fma(t12, t12, k[0] * t13);
    k[6] = k[1] * t13;
    k[7] = t13 * t13;
}

/* One step of one solve: stencil over [L, n - L)^3 (zero elsewhere), then the
 * six absorbing passes in order. */
void step(const Geo &g, const float *vd, const float *p0, const float *p1, float *p2)
{
    const int L = g.L, H = g.H;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < g.ntz; ++z)
        for (int y = 0; y < g.nty; ++y)
            for (int x = 0; x < g.ntx; ++x) {
                const long long i = z * g.sz + y * g.sy + x;
                if (x < L || x >= g.ntx - L || y < L || y >= g.nty - L || z < L || z >= g.ntz - L) {
                    p2[i] = 0.0f;
                    continue;
                }
                const float pc = p1[i];
                float lx = g.c[0] * pc, ly = lx, lz = lx;
                for (int m = 1; m <= H; ++m) {
                    lx = std::fma(g.c[m], p1[i + m] + p1[i - m], lx);
                    ly = std::fma(g.c[m], p1[i + m * g.sy] + p1[i - m * g.sy], ly);
                    lz = std::fma(g.c[m], p1[i + m * g.sz] + p1[i - m * g.sz], lz);
                }
                float t = lz * g.id2[2];
                t = std::fma(ly, g.id2[1], t);
                t = std::fma(lx, g.id2[0], t);
                const float u = std::fma(2.0f, pc, -p0[i]);
                const float v2 = vd[i] * vd[i];
                p2[i] = std::fma(v2, t, u);
            }
    /* faces: axis 2 (z), 1 (y), 0 (x); min side then max side */
    const int n[3] = {g.ntx, g.nty, g.ntz};
    const long long st[3] = {1, g.sy, g.sz};
    for (int a = 2; a >= 0; --a)
        for (int side = 0; side < 2; ++side) {
            const int lo = side == 0 ? L : n[a] - g.pml, hi = side == 0 ? g.pml : n[a] - L;
            const long long d = side == 0 ? st[a] : -st[a];
#pragma omp parallel for schedule(static)
            for (int z = 0; z < g.ntz; ++z)
                for (int y = 0; y < g.nty; ++y)
                    for (int x = 0; x < g.ntx; ++x) {
                        const int ia = a == 0 ? x : a == 1 ? y : z;
                        if (ia < lo || ia >= hi) continue;
                        const long long i = z * g.sz + y * g.sy + x;
                        const int wi = side == 0 ? ia - L : n[a] - L - 1 - ia;
                        float k[8];
                        abc_coef(vd[i] * g.id[a], k);
                        float e = k[0] * p1[i];
                        e = std::fma(k[1], p1[i + d], e);
                        e = std::fma(k[2], p1[i + 2 * d], e);
                        e = std::fma(-k[3], p0[i], e);
                        e = std::fma(-k[4], p0[i + d], e);
                        e = std::fma(-k[5], p0[i + 2 * d], e);
                        e = std::fma(-k[6], p0[i + 3 * d], e);
                        e = std::fma(-k[7], p0[i + 4 * d], e);
                        p2[i] = std::fma(g.w[wi], e, g.omw[wi] * p2[i]);
                    }
        }
}

inline long long cell(const Geo &g, const int *xyz)
{
    return (long long)(xyz[2] + g.pml) * g.sz + (long long)(xyz[1] + g.pml) * g.sy + (xyz[0] + g.pml);
}

inline long long interior(const Geo &g, long long i)
{
    const int z = (int)(i / g.sz), y = (int)((i % g.sz) / g.sy), x = (int)(i % g.sy);
    return ((long long)(z - g.pml) * g.ny + (y - g.pml)) * g.nx + (x - g.pml);
}

/* ((a * dt) * dt * v) * v: the injection factor of forward_IO / backward_IO. */
inline float inject(float a, float dt, float v) { return (((a * dt) * dt) * v) * v; }

int check_acq(const gb_fwi3d_params &p, const gb_fwi3d_acq &a)
{
    if (!a.src || !a.rec || !a.wavelet) return kEinval;
    for (int s = 0; s < p.ns; ++s)
        if (a.src[3 * s] < 0 || a.src[3 * s] >= p.nx || a.src[3 * s + 1] < 0 || a.src[3 * s + 1] >= p.ny ||
            a.src[3 * s + 2] < 0 || a.src[3 * s + 2] >= p.nz)
            return kEinval;
    for (int r = 0; r < p.nr; ++r)
        if (a.rec[3 * r] < 0 || a.rec[3 * r] >= p.nx || a.rec[3 * r + 1] < 0 || a.rec[3 * r + 1] >= p.ny ||
            a.rec[3 * r + 2] < 0 || a.rec[3 * r + 2] >= p.nz)
            return kEinval;
    return kOk;
}

}  // namespace

extern "C" {

/* One sample: data syn [ns][nt][nr]; with obs, the misfit and (grad != NULL)
 * the gradient [ny][nx][nz] in model order. */
int oracle3d_run(const gb_fwi3d_params *pp, const gb_fwi3d_acq *ap, const float *vel, const float *obs,
                 float *syn, float *grad, double *misfit)
{
    if (!pp || !ap || !vel || !syn || (grad && !obs)) return kEinval;
    const gb_fwi3d_params &p = *pp;
    Geo g;
    if (make_geo(p, g) != kOk || check_acq(p, *ap) != kOk) return kEinval;
    const gb_fwi3d_acq &a = *ap;
    const long long ntp = g.ntp, nin = (long long)g.nx * g.ny * g.nz;
    const int nti = p.nt_interval, nsave = (p.nt + nti - 1) / nti;
    std::vector<float> vd(ntp);
    for (int z = 0; z < g.ntz; ++z)
        for (int y = 0; y < g.nty; ++y)
            for (int x = 0; x < g.ntx; ++x) vd[z * g.sz + y * g.sy + x] = vpad(g, vel, x, y, z) * p.dt;
    std::vector<std::vector<double>> gsum;  // per-sample sum over shots, interior order
    std::vector<double> acc;
    if (grad) acc.assign(nin, 0.0);
    double mis = 0.0;
    std::vector<float> f0(ntp), f1(ntp), f2(ntp), snap, G;
    if (grad) {
        snap.assign((size_t)nsave * nin, 0.0f);
        G.assign(nin, 0.0f);
    }
    for (int s = 0; s < p.ns; ++s) {
        float *sy = syn + (long long)s * p.nt * p.nr;
        const long long is = cell(g, a.src + 3 * s);
        const float vs = vel[((long long)a.src[3 * s + 1] * g.nx + a.src[3 * s]) * g.nz + a.src[3 * s + 2]];
        std::fill(f0.begin(), f0.end(), 0.0f);
        std::fill(f1.begin(), f1.end(), 0.0f);
        std::fill(f2.begin(), f2.end(), 0.0f);
        float *q0 = f0.data(), *q1 = f1.data(), *q2 = f2.data();
        for (int it = 0; it < p.nt; ++it) {
            step(g, vd.data(), q0, q1, q2);
            q2[is] = q2[is] + inject(a.wavelet[it], p.dt, vs);
            if (grad && it % nti == 0) {
                float *sv = snap.data() + (long long)(it / nti) * nin;
#pragma omp parallel for schedule(static)
                for (int z = g.pml; z < g.ntz - g.pml; ++z)
                    for (int y = g.pml; y < g.nty - g.pml; ++y)
                        for (int x = g.pml; x < g.ntx - g.pml; ++x) {
                            const long long i = z * g.sz + y * g.sy + x;
                            const float u = std::fma(2.0f, q1[i], -q0[i]);
                            sv[((long long)(z - g.pml) * g.ny + (y - g.pml)) * g.nx + (x - g.pml)] =
                                (q2[i] - u) * g.idt2;
                        }
            }
            for (int r = 0; r < p.nr; ++r) sy[(long long)it * p.nr + r] = q2[cell(g, a.rec + 3 * r)];
            float *t = q0; q0 = q1; q1 = q2; q2 = t;
        }
        if (obs) {
            const float *ob = obs + (long long)s * p.nt * p.nr;
            for (long long k = 0; k < (long long)p.nt * p.nr; ++k) {
                const double r = (double)sy[k] - (double)ob[k];
                mis += r * r;
            }
        }
        if (!grad) continue;
        /* adjoint: same operator, residual injection, imaging every nti-th step */
        std::fill(f0.begin(), f0.end(), 0.0f);
        std::fill(f1.begin(), f1.end(), 0.0f);
        std::fill(f2.begin(), f2.end(), 0.0f);
        std::fill(G.begin(), G.end(), 0.0f);
        q0 = f0.data(); q1 = f1.data(); q2 = f2.data();
        const float *ob = obs + (long long)s * p.nt * p.nr;
        for (int it = p.nt - 1; it >= 0; --it) {
            step(g, vd.data(), q0, q1, q2);
            const bool stored = it % nti == 0;
            const float *sv = snap.data() + (long long)(it / nti) * nin;
            if (stored) {
#pragma omp parallel for schedule(static)
                for (int z = g.pml; z < g.ntz - g.pml; ++z)
                    for (int y = g.pml; y < g.nty - g.pml; ++y)
                        for (int x = g.pml; x < g.ntx - g.pml; ++x) {
                            const long long i = z * g.sz + y * g.sy + x;
                            const long long j = ((long long)(z - g.pml) * g.ny + (y - g.pml)) * g.nx + (x - g.pml);
                            G[j] = std::fma(sv[j], q2[i], G[j]);
                        }
            }
            for (int r = 0; r < p.nr; ++r) {
                const int *rc = a.rec + 3 * r;
                const long long ir = cell(g, rc);
                const float inj = sy[(long long)it * p.nr + r] - ob[(long long)it * p.nr + r];
                q2[ir] = q2[ir] + inj;
                if (stored) {
                    const long long j = interior(g, ir);
                    G[j] = std::fma(sv[j], inj, G[j]);
                }
            }
            float *t = q0; q0 = q1; q1 = q2; q2 = t;
        }
        for (long long j = 0; j < nin; ++j) acc[j] += (double)G[j];
    }
    if (misfit) *misfit = 0.5 * mis;
    if (grad) {
        const double coef = 2.0 * ((double)nti * (double)p.dt * (double)p.dt);
        for (int iy = 0; iy < g.ny; ++iy)
            for (int ix = 0; ix < g.nx; ++ix)
                for (int iz = 0; iz < g.nz; ++iz) {
                    const long long m = ((long long)iy * g.nx + ix) * g.nz + iz;
                    const long long j = ((long long)iz * g.ny + iy) * g.nx + ix;
                    const double v = vel[m];
                    grad[m] = (float)(coef * acc[j] / v);
                }
    }
    return kOk;
}

}  // extern "C"

/*
 * fwi2d_oracle.cpp -- CPU restatement of GeoPVI's 2-D acoustic FWI solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA engine in
 * geopvi_gb300/: only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference legs of bench.py load it.  The product never links or calls it.
 *
 * It restates, in the same floating-point operation order, the finite
 * difference path of geopvi/forward/fwi2d/fdtd2D_modelling.c:
 *   read_parameters / read_*_value       fdtd2D_modelling.c:1328-1379
 *   fd_coefficient                       fdtd2D_modelling.c:1272-1326
 *   getrik (Ricker wavelet)              fdtd2D_modelling.c:1084-1093
 *   get_velp (edge padding)              fdtd2D_modelling.c:1187-1238
 *   absorbing-boundary tables w, t11..13 fdtd2D_modelling.c:220-240
 *   source / receiver geometry           fdtd2D_modelling.c:118-154
 *   fdtd_2d_calculate_p (stencil)        fdtd2D_modelling.c:756-780
 *   abc_for_p (hybrid one-way boundary)  fdtd2D_modelling.c:833-900
 *   forward_IO / backward_IO             fdtd2D_modelling.c:902-978
 *   updata_p / wavefield_initialization  fdtd2D_modelling.c:1053-1081
 *   forward_aco_2D / backward_aco_2D     fdtd2D_modelling.c:678-753
 *   fwi_2D / forward_2D drivers          fdtd2D_modelling.c:18-353, 356-675
 *
 * Two arithmetic modes share one template:
 *   Real = float  : the reference's own mixed float/double arithmetic
 *                   (expected to be bitwise identical to the reference built
 *                   with -O2 and no FMA contraction);
 *   Real = double : the same discretisation carried out in double precision,
 *                   used to report every result's error against FP64.
 * Build with -ffp-contract=off (the Makefile does): contraction into FMA
 * changes the FP32 result at the 1e-4 level.
 *
 * Differences from the reference that do not change results:
 *   - the forward wavefield store keeps only the interior nz*nx cells that the
 *     gradient reads (the reference stores the padded grid);
 *   - loops run row-major (iz outer, ix inner) with OpenMP over rows;
 *   - errors are returned as negative status codes instead of exit().
 */
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

/* Field order and types follow read_parameters (fdtd2D_modelling.c:1328-1356). */
typedef struct {
    int nx, nz, pml0, Lc, laplace_solver, ns, nt, ds, ns0, depths, depthr, nr, dr, nr0,
        nt_interval;
    float dx, dz, dt, f0;
} oracle_params;

enum { ORACLE_OK = 0, ORACLE_EINVAL = -22, ORACLE_ENOENT = -2, ORACLE_ENOMEM = -12 };

}  // extern "C"

namespace {

/* The reference defines pi as this literal (fdtd2D_modelling.c:15). */
const double kPi = 3.1415926;

/* One "--comment" line followed by a number, as read_int_value / read_float_value do. */
bool read_value_line(FILE *fp, const char *fmt, void *dst)
{
    char line[256];
    if (!std::fgets(line, sizeof line, fp)) return false;
    if (std::fscanf(fp, "\n") < 0) { /* whitespace skip only */ }
    if (std::fscanf(fp, fmt, dst) != 1) return false;
    if (std::fscanf(fp, "\n") < 0) { /* end of file after the last value is fine */ }
    return true;
}

struct Geometry {
    int Lc;     /* stencil half-width + 1 (the reference's Lc after Lc += 1) */
    int pml;    /* pml0 + Lc */
    int ntz, ntx, ntp;
    int nt_save;
    int s_iz, r_iz;
    std::vector<int> s_ix, r_ix;
};

int make_geometry(const oracle_params &p, Geometry &g)
{
    if (p.nx <= 0 || p.nz <= 0 || p.pml0 <= 0 || p.ns <= 0 || p.nt <= 0 || p.nr <= 0 ||
        p.nt_interval <= 0)
        return ORACLE_EINVAL;
    if (p.laplace_solver != 0 && p.laplace_solver != 1) return ORACLE_EINVAL;
    if (p.Lc < 3 || p.Lc > 6) return ORACLE_EINVAL;  /* fd_coefficient knows Lc+1 = 4..7 */
    /* The pseudo-spectral Laplacian has no stencil halo: the reference sets
     * Lc = 0 before pml = pml0 + Lc (fdtd2D_modelling.c:75-78, 85), so its
     * absorbing strips start at the grid's edge. */
    g.Lc = p.laplace_solver == 1 ? 0 : p.Lc + 1;
    g.pml = p.pml0 + g.Lc;
    g.ntz = p.nz + 2 * g.pml;
    g.ntx = p.nx + 2 * g.pml;
    g.ntp = g.ntz * g.ntx;
    g.nt_save = p.nt / p.nt_interval + ((p.nt % p.nt_interval) ? 1 : 0);
    g.s_iz = g.pml + p.depths;
    g.r_iz = g.pml + p.depthr;
    if (g.s_iz < 0 || g.s_iz >= g.ntz || g.r_iz < 0 || g.r_iz >= g.ntz) return ORACLE_EINVAL;
    g.s_ix.resize(p.ns);
    g.r_ix.resize(p.nr);
    for (int is = 0; is < p.ns; ++is) {
        g.s_ix[is] = is * p.ds + g.pml + p.ns0;
        if (g.s_ix[is] < 0 || g.s_ix[is] >= g.ntx) return ORACLE_EINVAL;
    }
    for (int ir = 0; ir < p.nr; ++ir) {
        g.r_ix[ir] = g.pml + ir * p.dr + p.nr0;
        if (g.r_ix[ir] < 0 || g.r_ix[ir] >= g.ntx) return ORACLE_EINVAL;
    }
    return ORACLE_OK;
}

/* fd_coefficient (fdtd2D_modelling.c:1272-1326): the second-derivative weights,
 * evaluated in double and stored as float. */
template <typename Real>
void fd_weights(int Lc, Real *fd)
{
    switch (Lc) {
    case 4:
        fd[3] = 1.0 / 90; fd[2] = -3.0 / 20; fd[1] = 1.5; fd[0] = -49.0 / 18;
        break;
    case 5:
        fd[4] = -1.0 / 560; fd[3] = 8.0 / 315; fd[2] = -1.0 / 5; fd[1] = 8.0 / 5;
        fd[0] = -205.0 / 72;
        break;
    case 6:
        fd[5] = 8.0 / 25200; fd[4] = -125.0 / 25200; fd[3] = 1000.0 / 25200;
        fd[2] = -6000.0 / 25200; fd[1] = 42000.0 / 25200; fd[0] = -73766.0 / 25200;
        break;
    case 7: {
        const double den = 7.820582005659452e+44;
        fd[6] = -4.702129633040854e+40 / den; fd[5] = 8.12528000589218e+41 / den;
        fd[4] = -6.982662505061379e+42 / den; fd[3] = 4.13787407707198e+43 / den;
        fd[2] = -2.0947987515168676e+44 / den; fd[1] = 1.3406712009703548e+45 / den;
        fd[0] = -2.332705821577166e+45 / den;
        break;
    }
    default:
        break;
    }
}

/* getrik (fdtd2D_modelling.c:1084-1093).  The reference keeps the squared
 * phase in a float and evaluates the wavelet in double. */
template <typename Real>
void ricker(int nt, Real dt, Real f0, Real *rik)
{
    for (int it = 0; it < nt; ++it) {
        Real phase = (Real)it * dt - (Real)1 / f0;
        double arg = kPi * f0 * (double)phase;
        Real a = (Real)(arg * arg);
        rik[it] = (Real)((1.0 - 2.0 * a) * std::exp((double)(-a)));
    }
}

/* wavenumber (fdtd2D_modelling.c:1127-1184): |k|^2 of the padded grid's DFT
 * bins, kx = 2 pi dkx min(ix, ntx - ix) with the upper half starting at
 * ceil(ntx/2), dkx = 1/ntx/dx stored as float, each |k| component stored as
 * float, the squares summed in double and stored as float. */
void wavenumber(int ntx, int ntz, float dx, float dz, std::vector<float> &k)
{
    const float dkz = (float)(1.0 / ntz / dz), dkx = (float)(1.0 / ntx / dx);
    const int ax = ntx / 2 * 2 < ntx ? ntx / 2 + 1 : ntx / 2;
    const int az = ntz / 2 * 2 < ntz ? ntz / 2 + 1 : ntz / 2;
    k.assign((size_t)ntx * ntz, 0.0f);
    for (int iz = 0; iz < ntz; ++iz)
        for (int ix = 0; ix < ntx; ++ix) {
            const float kz = (float)(2 * kPi * dkz * (iz < az ? iz : ntz - iz));
            const float kx = (float)(2 * kPi * dkx * (ix < ax ? ix : ntx - ix));
            k[(size_t)iz * ntx + ix] = (float)(std::pow((double)kx, 2.0) + std::pow((double)kz, 2.0));
        }
}

/* Unnormalised 2-D DFT of a [ntz][ntx] complex array in place, sign -1
 * (forward) or +1 (inverse) as FFTW_FORWARD / FFTW_BACKWARD: rows, then
 * columns, each a direct O(n^2) sum with twiddles from one cos/sin table.
 * The reference uses FFTW (absent here); any DFT agrees with it to double
 * round-off. */
void dft2(std::vector<std::complex<double>> &a, int ntz, int ntx, int sign)
{
    auto pass = [&](int n, int count, long long stride, long long step) {
        std::vector<std::complex<double>> tw(n);
        for (int j = 0; j < n; ++j) {
            const double ang = 2.0 * 3.14159265358979323846 * j / n;
            tw[j] = std::complex<double>(std::cos(ang), sign * std::sin(ang));
        }
#pragma omp parallel for schedule(static)
        for (int line = 0; line < count; ++line) {
            std::vector<std::complex<double>> in(n), out(n);
            for (int j = 0; j < n; ++j) in[j] = a[line * step + j * stride];
            for (int k = 0; k < n; ++k) {
                std::complex<double> acc = 0.0;
                for (int j = 0; j < n; ++j) acc += in[j] * tw[(long long)k * j % n];
                out[k] = acc;
            }
            for (int j = 0; j < n; ++j) a[line * step + j * stride] = out[j];
        }
    };
    pass(ntx, ntz, 1, ntx);  // along x for every row
    pass(ntz, ntx, ntx, 1);  // along z for every column
}

inline float cube(float v) { return powf(v, 3); }
inline double cube(double v) { return std::pow(v, 3); }

template <typename Real>
struct Engine {
    const oracle_params &p;
    const Geometry &g;
    Real dx, dz, dt;
    Real fd[8];
    std::vector<Real> rik, velp, vdt2, t11, t12, t13, w;
    std::vector<Real> p0, p1, p2;
    std::vector<Real> psave; /* [nt_save][nz*nx], interior only */
    std::vector<Real> record;
    std::vector<float> kk;                     /* pseudo-spectral |k|^2 */
    std::vector<std::complex<double>> spec;    /* pseudo-spectral work array */

    Engine(const oracle_params &pp, const Geometry &gg) : p(pp), g(gg)
    {
        if (p.laplace_solver == 1) {
            wavenumber(g.ntx, g.ntz, p.dx, p.dz, kk);
            spec.resize(g.ntp);
        }
        dx = (Real)p.dx; dz = (Real)p.dz; dt = (Real)p.dt;
        fd_weights<Real>(g.Lc, fd);
        rik.resize(p.nt);
        ricker<Real>(p.nt, dt, (Real)p.f0, rik.data());
        velp.resize(g.ntp); vdt2.resize(g.ntp);
        t11.resize(g.ntp); t12.resize(g.ntp); t13.resize(g.ntp);
        w.resize(p.pml0);
        p0.resize(g.ntp); p1.resize(g.ntp); p2.resize(g.ntp);
        psave.resize((size_t)g.nt_save * p.nz * p.nx);
        record.resize((size_t)p.nt * p.nr);
    }

    /* get_velp (fdtd2D_modelling.c:1187-1238): interior copy, top and bottom
     * rows over the interior columns, then left and right over full height
     * (which fills the corners from the already padded rows). */
    void pad_velocity(const Real *vel_inner)
    {
        const int pml = g.pml, ntx = g.ntx, ntz = g.ntz;
        for (int iz = pml; iz < ntz - pml; ++iz)
            for (int ix = pml; ix < ntx - pml; ++ix)
                velp[iz * ntx + ix] = vel_inner[(iz - pml) * p.nx + (ix - pml)];
        for (int iz = 0; iz < pml; ++iz)
            for (int ix = pml; ix < ntx - pml; ++ix) velp[iz * ntx + ix] = velp[pml * ntx + ix];
        for (int iz = ntz - pml; iz < ntz; ++iz)
            for (int ix = pml; ix < ntx - pml; ++ix)
                velp[iz * ntx + ix] = velp[(ntz - pml - 1) * ntx + ix];
        for (int iz = 0; iz < ntz; ++iz) {
            for (int ix = 0; ix < pml; ++ix) velp[iz * ntx + ix] = velp[iz * ntx + pml];
            for (int ix = ntx - pml; ix < ntx; ++ix)
                velp[iz * ntx + ix] = velp[iz * ntx + (ntx - pml - 1)];
        }
        /* powf(v*dt, 2) in the stencil: an exact square rounded once. */
        for (int i = 0; i < g.ntp; ++i) {
            Real vd = velp[i] * dt;
            vdt2[i] = vd * vd;
        }
        /* Absorbing-boundary tables (fdtd2D_modelling.c:220-240). */
        for (int i = 0; i < p.pml0; ++i) w[i] = (Real)(1.0 - 1.0 * i / p.pml0);
        const Real alpha = 1;
        for (int i = 0; i < g.ntp; ++i) {
            Real s = alpha * velp[i] * dt / dx;
            t11[i] = (2 - s) * (1 - s) / 2;
            t12[i] = s * (2 - s);
            t13[i] = s * (s - 1) / 2;
        }
    }

    void zero_fields()
    {
        std::fill(p0.begin(), p0.end(), (Real)0);
        std::fill(p1.begin(), p1.end(), (Real)0);
        std::fill(p2.begin(), p2.end(), (Real)0);
    }

    /* fdtd_2d_calculate_p (fdtd2D_modelling.c:756-780). */
    void stencil()
    {
        const int Lc = g.Lc, ntx = g.ntx, ntz = g.ntz;
#pragma omp parallel for schedule(static)
        for (int iz = Lc; iz < ntz - Lc; ++iz) {
            for (int ix = Lc; ix < ntx - Lc; ++ix) {
                const int c = iz * ntx + ix;
                Real lx = fd[0] * p1[c];
                for (int k = 1; k < Lc; ++k) lx += fd[k] * (p1[c + k] + p1[c - k]);
                Real lz = fd[0] * p1[c];
                for (int k = 1; k < Lc; ++k) lz += fd[k] * (p1[c + k * ntx] + p1[c - k * ntx]);
                p2[c] = 2 * p1[c] - p0[c] + vdt2[c] * (lx / dx / dx + lz / dz / dz);
            }
        }
    }

    /* One blend of abc_for_p at cell c; `step` is the offset that points
     * from the boundary towards the interior (+ntx top, -ntx bottom, +1 left,
     * -1 right).  The weighted extrapolation is float, the blend with the
     * current value is double, as in the reference. */
    inline Real blend(int c, int step, Real wk) const
    {
        const Real a = t11[c], b = t12[c], e = t13[c];
        Real ext = 2 * a * p1[c] + 2 * b * p1[c + step] + 2 * e * p1[c + 2 * step] -
                   a * a * p0[c] - 2 * a * b * p0[c + step] -
                   (b * b + 2 * a * e) * p0[c + 2 * step] - 2 * b * e * p0[c + 3 * step] -
                   e * e * p0[c + 4 * step];
        return (Real)((double)(wk * ext) + (1.0 - (double)wk) * (double)p2[c]);
    }

    /* abc_for_p (fdtd2D_modelling.c:833-900): top, bottom, left, right, in
     * that order; the corner cells take two blends. */
    /* pstd_2d_calculate_p (fdtd2D_modelling.c:783-830): p1 through a double
     * 2-D DFT, times -|k|^2, back, and p2 = 2 p1 - p0 + (v dt)^2 re / (ntx ntz)
     * over every cell, the float part evaluated in float and the sum in double
     * as the C expression promotes it. */
    void pstd()
    {
        const int ntp = g.ntp;
        for (int i = 0; i < ntp; ++i) spec[i] = std::complex<double>((double)p1[i], 0.0);
        dft2(spec, g.ntz, g.ntx, -1);
        for (int i = 0; i < ntp; ++i) spec[i] *= -(double)kk[i];
        dft2(spec, g.ntz, g.ntx, +1);
        const double n = (double)g.ntx * g.ntz;
        for (int i = 0; i < ntp; ++i) {
            const Real a = 2 * p1[i] - p0[i];
            p2[i] = (Real)((double)a + (double)vdt2[i] * spec[i].real() / n);
        }
    }

    /* The Laplacian update of laplace_solver (forward_aco_2D :692-695). */
    void laplacian()
    {
        if (p.laplace_solver == 1)
            pstd();
        else
            stencil();
    }

    void boundary()
    {
        const int Lc = g.Lc, pml = g.pml, ntx = g.ntx, ntz = g.ntz;
#pragma omp parallel for schedule(static)
        for (int iz = Lc; iz < pml; ++iz)
            for (int ix = 0; ix < ntx; ++ix) p2[iz * ntx + ix] = blend(iz * ntx + ix, ntx, w[iz - Lc]);
#pragma omp parallel for schedule(static)
        for (int iz = ntz - pml; iz < ntz - Lc; ++iz)
            for (int ix = 0; ix < ntx; ++ix)
                p2[iz * ntx + ix] = blend(iz * ntx + ix, -ntx, w[ntz - Lc - iz - 1]);
#pragma omp parallel for schedule(static)
        for (int iz = 0; iz < ntz; ++iz) {
            for (int ix = Lc; ix < pml; ++ix) p2[iz * ntx + ix] = blend(iz * ntx + ix, 1, w[ix - Lc]);
            for (int ix = ntx - pml; ix < ntx - Lc; ++ix)
                p2[iz * ntx + ix] = blend(iz * ntx + ix, -1, w[ntx - Lc - ix - 1]);
        }
    }

    /* updata_p (fdtd2D_modelling.c:1053-1066): p2 keeps its values, so cells
     * the stencil skips enter the next boundary pass equal to p1. */
    void rotate()
    {
        std::memcpy(p0.data(), p1.data(), sizeof(Real) * g.ntp);
        std::memcpy(p1.data(), p2.data(), sizeof(Real) * g.ntp);
    }

    /* forward_aco_2D (fdtd2D_modelling.c:678-714) with forward_IO (:902-939). */
    void forward_shot(int is, int run_fwi)
    {
        const int ntx = g.ntx, pml = g.pml, nx = p.nx, nz = p.nz;
        const int src = g.s_iz * ntx + g.s_ix[is];
        zero_fields();
        for (int it = 0; it < p.nt; ++it) {
            laplacian();
            boundary();
            p2[src] += rik[it] * dt * dt * velp[src] * velp[src];
            if (it % p.nt_interval == 0) {
                Real *ps = psave.data() + (size_t)(it / p.nt_interval) * nz * nx;
#pragma omp parallel for schedule(static)
                for (int iz = 0; iz < nz; ++iz)
                    for (int ix = 0; ix < nx; ++ix) {
                        const int c = (iz + pml) * ntx + ix + pml;
                        ps[iz * nx + ix] = run_fwi ? (p2[c] - 2 * p1[c] + p0[c]) / dt / dt : p2[c];
                    }
            }
            for (int ir = 0; ir < p.nr; ++ir) record[(size_t)it * p.nr + ir] = p2[g.r_iz * ntx + g.r_ix[ir]];
            rotate();
        }
    }

    /* backward_aco_2D (fdtd2D_modelling.c:717-753) with backward_IO (:941-978). */
    void backward_shot(int run_fwi, Real *grad)
    {
        const int ntx = g.ntx, pml = g.pml, nx = p.nx, nz = p.nz;
        zero_fields();
        for (int it = p.nt - 1; it >= 0; --it) {
            laplacian();
            boundary();
            for (int ir = 0; ir < p.nr; ++ir) {
                const int c = g.r_iz * ntx + g.r_ix[ir];
                p2[c] += record[(size_t)it * p.nr + ir] * dt * dt * velp[c] * velp[c];
            }
            if (it % p.nt_interval == 0) {
                const Real *ps = psave.data() + (size_t)(it / p.nt_interval) * nz * nx;
#pragma omp parallel for schedule(static)
                for (int iz = 0; iz < nz; ++iz)
                    for (int ix = 0; ix < nx; ++ix) {
                        const int c = (iz + pml) * ntx + ix + pml;
                        const int k = iz * nx + ix;
                        if (run_fwi)
                            grad[k] = (Real)((double)grad[k] + -2.0 / (double)cube(velp[c]) *
                                                                   (double)ps[k] * (double)p2[c] *
                                                                   (double)p.nt_interval * (double)dt);
                        else
                            grad[k] += ps[k] * p2[c] * p.nt_interval * dt;
                    }
            }
            rotate();
        }
    }
};

template <typename Real>
int run_fwi_impl(const oracle_params *pp, const Real *vel_inner, const Real *record_obs,
                 Real *record_syn, Real *grad, int run_fwi)
{
    Geometry g;
    int st = make_geometry(*pp, g);
    if (st) return st;
    Engine<Real> e(*pp, g);
    e.pad_velocity(vel_inner);
    const size_t shot_len = (size_t)pp->nt * pp->nr;
    for (int is = 0; is < pp->ns; ++is) {
        e.forward_shot(is, run_fwi);
        /* residual (fdtd2D_modelling.c:269-278) */
        for (size_t i = 0; i < shot_len; ++i) {
            record_syn[is * shot_len + i] = e.record[i];
            if (run_fwi)
                e.record[i] -= record_obs[is * shot_len + i];
            else
                e.record[i] = record_obs[is * shot_len + i];
        }
        e.backward_shot(run_fwi, grad);
    }
    return ORACLE_OK;
}

template <typename Real>
int run_forward_impl(const oracle_params *pp, const Real *vel_inner, Real *record_syn)
{
    Geometry g;
    int st = make_geometry(*pp, g);
    if (st) return st;
    Engine<Real> e(*pp, g);
    e.pad_velocity(vel_inner);
    const size_t shot_len = (size_t)pp->nt * pp->nr;
    for (int is = 0; is < pp->ns; ++is) {
        e.forward_shot(is, 1);
        std::memcpy(record_syn + is * shot_len, e.record.data(), sizeof(Real) * shot_len);
    }
    return ORACLE_OK;
}


/* ------------------------------------------------------------------------
 * Exact discrete adjoint (double precision).
 *
 * One step of the scheme maps the two previous levels to the next one
 * linearly: p2 = A1 p1 + A0 p0 + f_it, where for each cell c
 *   p2_c = beta_c * S_c + sum_b gamma_{c,b} * E_{c,b}
 * with S_c the stencil value 2 p1 - p0 + a_c (Dxx + Dzz) p1 (a_c = (v dt)^2)
 * inside the stencil region and the copied p1_c outside it, E_{c,b} the
 * one-way extrapolation of blend b (top/bottom, then left/right) with
 * weights w_b: beta = prod (1 - w_b), gamma_1 = w_1 (1 - w_2), gamma_2 = w_2.
 * With lambda^k = dJ/dP^k for J = 1/2 sum_t |R P^{t+1} - obs_t|^2:
 *   lambda^k = R^T r_{k-1} + A1^T lambda^{k+1} + A0^T lambda^{k+2},
 *   dJ/dv_c  = sum_t lambda^{t+1}_c d(p2_c)/d(v_c) |_{step t},
 * and the padded-grid derivative is summed back onto the interior cells the
 * padding replicates (get_velp is a clamp).  This is the gradient a central
 * finite difference of the scheme converges to; the reference's own
 * gradient (backward_IO) is a continuous-adjoint approximation of it.
 * ------------------------------------------------------------------------ */
struct CellOp {
    bool sten;
    double beta;
    int nb;
    int step[2];
    double gam[2];
};

static void cell_ops(const Geometry &g, const std::vector<double> &w, std::vector<CellOp> &ops)
{
    const int ntx = g.ntx, ntz = g.ntz, Lc = g.Lc, pml = g.pml;
    ops.assign((size_t)g.ntp, CellOp{});
    for (int iz = 0; iz < ntz; ++iz)
        for (int ix = 0; ix < ntx; ++ix) {
            CellOp &o = ops[(size_t)iz * ntx + ix];
            o.sten = iz >= Lc && iz < ntz - Lc && ix >= Lc && ix < ntx - Lc;
            double wv[2];
            o.nb = 0;
            if (iz >= Lc && iz < pml) { o.step[o.nb] = ntx; wv[o.nb++] = w[iz - Lc]; }
            else if (iz >= ntz - pml && iz < ntz - Lc) { o.step[o.nb] = -ntx; wv[o.nb++] = w[ntz - Lc - iz - 1]; }
            if (ix >= Lc && ix < pml) { o.step[o.nb] = 1; wv[o.nb++] = w[ix - Lc]; }
            else if (ix >= ntx - pml && ix < ntx - Lc) { o.step[o.nb] = -1; wv[o.nb++] = w[ntx - Lc - ix - 1]; }
            if (o.nb == 0) o.beta = 1.0;
            else if (o.nb == 1) { o.beta = 1.0 - wv[0]; o.gam[0] = wv[0]; }
            else { o.beta = (1.0 - wv[0]) * (1.0 - wv[1]); o.gam[0] = wv[0] * (1.0 - wv[1]); o.gam[1] = wv[1]; }
        }
}

struct ExactShot {
    const oracle_params &p;
    const Geometry &g;
    Engine<double> &e;
    std::vector<CellOp> ops;

    ExactShot(const oracle_params &pp, const Geometry &gg, Engine<double> &ee) : p(pp), g(gg), e(ee)
    {
        std::vector<double> w(e.w.begin(), e.w.end());
        cell_ops(g, w, ops);
    }

    // out += A1^T lam (p1 coefficients) or A0^T lam (p0 coefficients).
    void scatter(const double *lam, double *out, bool p1op) const
    {
        const int ntx = g.ntx;
        const int H = g.Lc - 1;
        const double rdx2 = 1.0 / ((double)e.dx * e.dx), rdz2 = 1.0 / ((double)e.dz * e.dz);
        for (int c = 0; c < g.ntp; ++c) {
            const double l = lam[c];
            if (l == 0.0) continue;
            const CellOp &o = ops[c];
            const double bl = o.beta * l;
            if (o.sten) {
                if (p1op) {
                    const double a = e.vdt2[c];
                    out[c] += 2.0 * bl + bl * a * e.fd[0] * (rdx2 + rdz2);
                    for (int m = 1; m <= H; ++m) {
                        const double kx = bl * a * e.fd[m] * rdx2, kz = bl * a * e.fd[m] * rdz2;
                        out[c + m] += kx;
                        out[c - m] += kx;
                        out[c + m * ntx] += kz;
                        out[c - m * ntx] += kz;
                    }
                } else {
                    out[c] -= bl;
                }
            } else if (p1op) {
                out[c] += bl;  // the copied previous level
            }
            for (int b = 0; b < o.nb; ++b) {
                const double gl = o.gam[b] * l;
                const int st = o.step[b];
                const double t11 = e.t11[c], t12 = e.t12[c], t13 = e.t13[c];
                if (p1op) {
                    out[c] += gl * 2 * t11;
                    out[c + st] += gl * 2 * t12;
                    out[c + 2 * st] += gl * 2 * t13;
                } else {
                    out[c] -= gl * t11 * t11;
                    out[c + st] -= gl * 2 * t11 * t12;
                    out[c + 2 * st] -= gl * (t12 * t12 + 2 * t11 * t13);
                    out[c + 3 * st] -= gl * 2 * t12 * t13;
                    out[c + 4 * st] -= gl * t13 * t13;
                }
            }
        }
    }

    // d(p2_c)/d(v_c) at one step, from the step's p1, p0 and source value.
    double dp2_dv(int c, const double *p1, const double *p0, double rik_it, int src) const
    {
        const CellOp &o = ops[c];
        const int ntx = g.ntx, H = g.Lc - 1;
        const double v = e.velp[c], dt = e.dt, dx = e.dx, dz = e.dz;
        double d = 0.0;
        if (o.sten) {
            double lx = e.fd[0] * p1[c], lz = e.fd[0] * p1[c];
            for (int m = 1; m <= H; ++m) {
                lx += e.fd[m] * (p1[c + m] + p1[c - m]);
                lz += e.fd[m] * (p1[c + m * ntx] + p1[c - m * ntx]);
            }
            d += o.beta * 2.0 * v * dt * dt * (lx / (dx * dx) + lz / (dz * dz));
        }
        if (o.nb) {
            const double s = v * dt / dx;
            const double t11 = (2 - s) * (1 - s) / 2, t12 = s * (2 - s), t13 = s * (s - 1) / 2;
            const double u11 = (2 * s - 3) / 2, u12 = 2 - 2 * s, u13 = (2 * s - 1) / 2;  // d t / d s
            for (int b = 0; b < o.nb; ++b) {
                const int st = o.step[b];
                const double dE = 2 * u11 * p1[c] + 2 * u12 * p1[c + st] + 2 * u13 * p1[c + 2 * st] -
                                  2 * t11 * u11 * p0[c] - 2 * (u11 * t12 + t11 * u12) * p0[c + st] -
                                  (2 * t12 * u12 + 2 * u11 * t13 + 2 * t11 * u13) * p0[c + 2 * st] -
                                  2 * (u12 * t13 + t12 * u13) * p0[c + 3 * st] - 2 * t13 * u13 * p0[c + 4 * st];
                d += o.gam[b] * dE * dt / dx;
            }
        }
        if (c == src) d += 2.0 * rik_it * dt * dt * v;
        return d;
    }

    // Misfit of the shot and its exact gradient on the padded grid (added to gpad).
    double run(int is, const double *obs, double *gpad)
    {
        const int ntp = g.ntp, nt = p.nt, nr = p.nr;
        const int src = g.s_iz * g.ntx + g.s_ix[is];
        std::vector<double> P((size_t)(nt + 2) * ntp, 0.0);  // level k at (k + 1) * ntp, k = -1..nt
        auto lev = [&](int k) { return P.data() + (size_t)(k + 1) * ntp; };
        std::vector<double> resid((size_t)nt * nr);
        e.zero_fields();
        double J = 0.0;
        for (int it = 0; it < nt; ++it) {
            e.stencil();
            e.boundary();
            e.p2[src] += e.rik[it] * e.dt * e.dt * e.velp[src] * e.velp[src];
            std::copy(e.p2.begin(), e.p2.end(), lev(it + 1));
            for (int ir = 0; ir < nr; ++ir) {
                const double r = e.p2[g.r_iz * g.ntx + g.r_ix[ir]] - obs[(size_t)it * nr + ir];
                resid[(size_t)it * nr + ir] = r;
                J += 0.5 * r * r;
            }
            e.rotate();
        }
        std::vector<double> l0(ntp, 0.0), l1(ntp, 0.0), l2(ntp, 0.0);  // lambda^k, ^k+1, ^k+2
        for (int k = nt; k >= 1; --k) {
            std::fill(l0.begin(), l0.end(), 0.0);
            for (int ir = 0; ir < nr; ++ir) l0[g.r_iz * g.ntx + g.r_ix[ir]] += resid[(size_t)(k - 1) * nr + ir];
            scatter(l1.data(), l0.data(), true);
            scatter(l2.data(), l0.data(), false);
            const int it = k - 1;  // the step whose p2 is level k
            const double *p1 = lev(it), *p0 = lev(it - 1);
            for (int c = 0; c < ntp; ++c)
                if (l0[c] != 0.0) gpad[c] += l0[c] * dp2_dv(c, p1, p0, e.rik[it], src);
            std::swap(l2, l1);
            std::swap(l1, l0);
        }
        return J;
    }
};

}  // namespace

extern "C" {

int oracle_read_params(const char *path, oracle_params *p)
{
    FILE *fp = std::fopen(path, "r");
    if (!fp) return ORACLE_ENOENT;
    int *ints[] = {&p->nx, &p->nz, &p->pml0, &p->Lc, &p->laplace_solver, &p->ns, &p->nt, &p->ds,
                   &p->ns0, &p->depths, &p->depthr, &p->nr, &p->dr, &p->nr0, &p->nt_interval};
    float *floats[] = {&p->dx, &p->dz, &p->dt, &p->f0};
    bool ok = true;
    for (int *v : ints) ok = ok && read_value_line(fp, "%d", v);
    for (float *v : floats) ok = ok && read_value_line(fp, "%f", v);
    std::fclose(fp);
    return ok ? ORACLE_OK : ORACLE_EINVAL;
}

/* fwi_2D: grad is accumulated (+=) like the reference; zero it first. */
int oracle_fwi2d_f32(const oracle_params *p, const float *vel, const float *obs, float *syn,
                     float *grad, int run_fwi)
{
    return run_fwi_impl<float>(p, vel, obs, syn, grad, run_fwi);
}

int oracle_fwi2d_f64(const oracle_params *p, const double *vel, const double *obs, double *syn,
                     double *grad, int run_fwi)
{
    return run_fwi_impl<double>(p, vel, obs, syn, grad, run_fwi);
}

int oracle_forward2d_f32(const oracle_params *p, const float *vel, float *syn)
{
    return run_forward_impl<float>(p, vel, syn);
}

int oracle_forward2d_f64(const oracle_params *p, const double *vel, double *syn)
{
    return run_forward_impl<double>(p, vel, syn);
}

/* Exact discrete gradient dJ/dv of J = 1/2 sum (syn - obs)^2 over all shots,
 * in double precision (see ExactShot); returns J. */
int oracle_exact_grad_f64(const oracle_params *pp, const double *vel, const double *obs, double *grad,
                          double *misfit)
{
    Geometry g;
    int st = make_geometry(*pp, g);
    if (st) return st;
    if (pp->laplace_solver != 0) return ORACLE_EINVAL;  // the exact adjoint transposes the FD stencil
    Engine<double> e(*pp, g);
    e.pad_velocity(vel);
    ExactShot x(*pp, g, e);
    std::vector<double> gpad((size_t)g.ntp, 0.0);
    double J = 0.0;
    const size_t shot_len = (size_t)pp->nt * pp->nr;
    for (int is = 0; is < pp->ns; ++is) J += x.run(is, obs + is * shot_len, gpad.data());
    for (int i = 0; i < pp->nz * pp->nx; ++i) grad[i] = 0.0;
    for (int iz = 0; iz < g.ntz; ++iz)
        for (int ix = 0; ix < g.ntx; ++ix) {
            const int jz = std::min(std::max(iz - g.pml, 0), pp->nz - 1);
            const int jx = std::min(std::max(ix - g.pml, 0), pp->nx - 1);
            grad[jz * pp->nx + jx] += gpad[(size_t)iz * g.ntx + ix];
        }
    if (misfit) *misfit = J;
    return ORACLE_OK;
}

/* The pseudo-spectral Laplacian of one [ntz][ntx] field (pstd_2d_calculate_p's
 * DFT / -|k|^2 / inverse DFT part), out = re / (ntx ntz), for checks against
 * known transforms. */
int oracle_pstd_laplacian(int ntz, int ntx, float dx, float dz, const double *in, double *out)
{
    if (ntz <= 0 || ntx <= 0) return ORACLE_EINVAL;
    std::vector<float> k;
    wavenumber(ntx, ntz, dx, dz, k);
    std::vector<std::complex<double>> a((size_t)ntz * ntx);
    for (size_t i = 0; i < a.size(); ++i) a[i] = in[i];
    dft2(a, ntz, ntx, -1);
    for (size_t i = 0; i < a.size(); ++i) a[i] *= -(double)k[i];
    dft2(a, ntz, ntx, +1);
    for (size_t i = 0; i < a.size(); ++i) out[i] = a[i].real() / ((double)ntx * ntz);
    return ORACLE_OK;
}

/* Ricker table as the float solver sees it (getrik, fdtd2D_modelling.c:1084). */
void oracle_ricker_f32(int nt, float dt, float f0, float *rik) { ricker<float>(nt, dt, f0, rik); }

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"

/* FFTW3 stand-ins for the reference build (test infrastructure only).
 *
 * The reference's pseudo-spectral Laplacian (pstd_2d_calculate_p,
 * geopvi/forward/fwi2d/fdtd2D_modelling.c:783-830) uses seven FFTW calls:
 * fftw_init_threads, fftw_plan_with_nthreads, fftw_malloc, fftw_free,
 * fftw_plan_dft_2d, fftw_execute, fftw_destroy_plan.  FFTW is not installed
 * here, so these definitions let the reference's own code run.
 *
 * fftw_execute computes FFTW's documented (unnormalised) 2-D transform of
 * an n0 x n1 row-major complex array,
 *     out[k0][k1] = sum_{j0,j1} in[j0][j1] exp(s 2 pi i (j0 k0 / n0 + j1 k1 / n1)),
 * s = -1 (FFTW_FORWARD) or +1 (FFTW_BACKWARD), by the direct separable
 * method: the 1-D transform of every row, then of every column.  Twiddle
 * factors exp(s 2 pi i m / n) are tabulated once per plan for m = 0..n-1
 * from cosl / sinl, the index m = (j k) mod n is exact, and every sum is
 * accumulated in long double, then rounded to double.  That is the
 * transform's definition evaluated directly, not FFTW's algorithm: the
 * spectra agree with FFTW's to within a few units in the last place of a
 * double, which the reference then rounds to float.  In-place plans
 * (in == out) are supported, as the reference uses them. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

struct oracle_fftw_plan_s {
    int n0, n1, sign;
    fftw_complex *in, *out;
    long double *c0, *s0, *c1, *s1; /* twiddles of the column and row transforms */
};

int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { (void)n; }
void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }

static int twiddles(int n, int sign, long double **c, long double **s)
{
    *c = (long double *)malloc(sizeof(long double) * (size_t)n);
    *s = (long double *)malloc(sizeof(long double) * (size_t)n);
    if (!*c || !*s) return 0;
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (int m = 0; m < n; ++m) {
        const long double a = two_pi * (long double)m / (long double)n;
        (*c)[m] = cosl(a);
        (*s)[m] = (long double)sign * sinl(a);
    }
    return 1;
}

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags)
{
    (void)flags;
    fftw_plan p = (fftw_plan)calloc(1, sizeof *p);
    if (!p) return NULL;
    p->n0 = n0;
    p->n1 = n1;
    p->sign = sign;
    p->in = in;
    p->out = out;
    if (!twiddles(n0, sign, &p->c0, &p->s0) || !twiddles(n1, sign, &p->c1, &p->s1)) {
        fftw_destroy_plan(p);
        return NULL;
    }
    return p;
}

void fftw_execute(const fftw_plan p)
{
    const int n0 = p->n0, n1 = p->n1;
    const size_t n = (size_t)n0 * n1;
    long double *re = (long double *)malloc(sizeof(long double) * n);
    long double *im = (long double *)malloc(sizeof(long double) * n);
    if (!re || !im) abort();
    /* rows: re/im[j0][k1] = sum_j1 in[j0][j1] w1^(j1 k1) */
    for (int j0 = 0; j0 < n0; ++j0) {
        const fftw_complex *row = p->in + (size_t)j0 * n1;
        for (int k1 = 0; k1 < n1; ++k1) {
            long double sr = 0.0L, si = 0.0L;
            int m = 0;
            for (int j1 = 0; j1 < n1; ++j1) {
                const long double xr = row[j1][0], xi = row[j1][1];
                sr += xr * p->c1[m] - xi * p->s1[m];
                si += xr * p->s1[m] + xi * p->c1[m];
                m += k1;
                if (m >= n1) m -= n1;
            }
            re[(size_t)j0 * n1 + k1] = sr;
            im[(size_t)j0 * n1 + k1] = si;
        }
    }
    /* columns: out[k0][k1] = sum_j0 (re, im)[j0][k1] w0^(j0 k0) */
    long double *cr = (long double *)malloc(sizeof(long double) * (size_t)n0);
    long double *ci = (long double *)malloc(sizeof(long double) * (size_t)n0);
    if (!cr || !ci) abort();
    for (int k1 = 0; k1 < n1; ++k1) {
        for (int k0 = 0; k0 < n0; ++k0) {
            long double sr = 0.0L, si = 0.0L;
            int m = 0;
            for (int j0 = 0; j0 < n0; ++j0) {
                const long double xr = re[(size_t)j0 * n1 + k1], xi = im[(size_t)j0 * n1 + k1];
                sr += xr * p->c0[m] - xi * p->s0[m];
                si += xr * p->s0[m] + xi * p->c0[m];
                m += k0;
                if (m >= n0) m -= n0;
            }
            cr[k0] = sr;
            ci[k0] = si;
        }
        for (int k0 = 0; k0 < n0; ++k0) {
            p->out[(size_t)k0 * n1 + k1][0] = (double)cr[k0];
            p->out[(size_t)k0 * n1 + k1][1] = (double)ci[k0];
        }
    }
    free(cr);
    free(ci);
    free(re);
    free(im);
}

void fftw_destroy_plan(fftw_plan p)
{
    if (!p) return;
    free(p->c0);
    free(p->s0);
    free(p->c1);
    free(p->s1);
    free(p);
}

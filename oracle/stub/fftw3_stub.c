/* Aborting FFTW3 stand-ins for the reference build (test infrastructure only).
 * The oracle never selects the pseudo-spectral Laplacian, so none of these
 * should run; if one does, the process stops with a message. */
#include <stdio.h>
#include <stdlib.h>
#include "fftw3.h"

static void oracle_fftw_unavailable(const char *fn)
{
    fprintf(stderr, "oracle: %s called, but the pseudo-spectral path is not built\n", fn);
    abort();
}
int fftw_init_threads(void) { oracle_fftw_unavailable("fftw_init_threads"); return 0; }
void fftw_plan_with_nthreads(int n) { (void)n; oracle_fftw_unavailable("fftw_plan_with_nthreads"); }
void *fftw_malloc(size_t n) { (void)n; oracle_fftw_unavailable("fftw_malloc"); return NULL; }
void fftw_free(void *p) { (void)p; oracle_fftw_unavailable("fftw_free"); }
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int s, unsigned f)
{
    (void)n0; (void)n1; (void)in; (void)out; (void)s; (void)f;
    oracle_fftw_unavailable("fftw_plan_dft_2d");
    return NULL;
}
void fftw_execute(const fftw_plan p) { (void)p; oracle_fftw_unavailable("fftw_execute"); }
void fftw_destroy_plan(fftw_plan p) { (void)p; oracle_fftw_unavailable("fftw_destroy_plan"); }

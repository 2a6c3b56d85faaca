/* Minimal FFTW3 declarations so the reference acoustic solver
 * (geopvi/forward/fwi2d/fdtd2D_modelling.c) compiles without FFTW.
 * Only the pseudo-spectral Laplacian (laplace_solver == 1,
 * fdtd2D_modelling.c:75-81 and :783-830) calls FFTW.  fftw3_stub.c defines
 * the seven calls it makes; its transform evaluates FFTW's definition of the
 * unnormalised 2-D DFT directly.  Test infrastructure only. */
#ifndef ORACLE_STUB_FFTW3_H
#define ORACLE_STUB_FFTW3_H
#include <stddef.h>
typedef double fftw_complex[2];
typedef struct oracle_fftw_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);
#endif

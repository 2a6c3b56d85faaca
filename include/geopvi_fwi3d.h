/*
 * geopvi_fwi3d.h -- C ABI of the GB300 3-D acoustic FWI engine.
 *
 * Boundary being replaced: GeoPVI's 3-D FWI posterior
 * (geopvi/forward/fwi3d/posterior.py:44-77, run_fwi_i) calls an external
 * 3-D FWI executable once per sample through a file interface: the model
 * `particles_<i>.npy` (prepare_samples, :13-19; values in (ny, nx, nz)
 * order, nz fastest), the shot subset `batch_src.npy` and its data
 * `batch_data.npy` (prepare_batch, :21-33), a wavelet file and a receiver
 * file; it reads back `gradout_<i>.npy` (dJ/dv of the model) and
 * `pred_data_<i>.npy`, and forms J = sum((pred - data)^2) itself (cal_loss,
 * :35-41).  The reference ships no such executable, so the engine defines
 * the 3-D scheme as the 2-D reference solver's algorithm
 * (geopvi/forward/fwi2d/fdtd2D_modelling.c) carried to three axes:
 *
 *   grid      padded by pml = pml0 + Lc + 1 cells per side, velocity edge-
 *             replicated (get_velp, :1187-1238); rim cells within Lc + 1 of a
 *             face are never updated (they stay zero).
 *   step      p2 = 2 p1 - p0 + (v dt)^2 (Lxx/dx^2 + Lyy/dy^2 + Lzz/dz^2) with
 *             the 2*Lc-order second-derivative weights of fd_coefficient
 *             (:1272-1326) along each axis (fdtd_2d_calculate_p, :756-780).
 *   boundary  the hybrid one-way absorbing blend of abc_for_p (:833-900) on
 *             the six faces in the order z-min, z-max, y-min, y-max, x-min,
 *             x-max, each over the full extent of the other two axes, with
 *             s = v dt / d along the face normal.
 *   source    p2[src] += w(it) dt dt v v after the step; receivers sample p2
 *             afterwards (forward_IO, :902-939); w is the caller's wavelet.
 *   gradient  the adjoint field runs the same step operator backwards in time
 *             from the residuals syn - obs added at the receivers (the
 *             transpose of sampling; backward_IO, :941-978, adds them scaled by
 *             dt^2 v^2); every nt_interval-th step adds the stored d2p/dt2
 *             times the adjoint field, and
 *             grad = 2 dt^2 nt_interval / v * (sum over shots).
 *             As P^{k+1} = 2P^k - P^{k-1} + v^2 dt^2 (lap P^k + f) gives
 *             dP^{k+1}/dv = (2/v)(P^{k+1} - 2P^k + P^{k-1}), this is dJ/dv of
 *             J = 0.5 * sum((syn - obs)^2) -- the `gradout` the reference's
 *             posterior expects -- up to the absorbing strips (the adjoint
 *             reuses the forward blend) and the velocity replicated into the
 *             padding (its share of an edge cell's derivative is not added).
 *             (The 2-D reference's grad, -2/v^3 dt sum psave p_adj with the
 *             scaled injection, is about -dt (v_rec/v)^2 times dJ/dv.)
 *
 * Arithmetic is FP32 with every fused multiply-add written out (no
 * contraction by the compiler), in an order the CPU oracle follows
 * operation by operation, so data and gradient are bit-identical to it; the
 * misfit 0.5 * sum((syn - obs)^2) is summed in FP64.
 *
 * Plain pointers and sizes only; `stream` is a cudaStream_t passed as void*.
 * Status codes are those of geopvi_fwi2d.h.
 */
#ifndef GEOPVI_FWI3D_H
#define GEOPVI_FWI3D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_fwi3d_params {
    int nx, ny, nz;     /* model cells */
    int pml0;           /* absorbing strip width in cells (>= 1) */
    int Lc;             /* finite-difference half order as in the 2-D parameter file: 3..6 */
    int ns;             /* shots of the batch */
    int nr;             /* receivers, common to every shot */
    int nt;             /* time steps */
    int nt_interval;    /* the gradient images every nt_interval-th step */
    float dx, dy, dz;   /* grid spacing */
    float dt;           /* time step */
} gb_fwi3d_params;

/* Acquisition, host memory: positions are model cells (0-based ix, iy, iz). */
typedef struct gb_fwi3d_acq {
    const int *src;       /* [ns][3] */
    const int *rec;       /* [nr][3] */
    const float *wavelet; /* [nt] source time function */
} gb_fwi3d_acq;

#define GB_FWI3D_FORWARD_ONLY 0x1u /* data (and misfit) only: no stored field, no adjoint */
#define GB_FWI3D_CHECKPOINT 0x2u   /* store ceil(sqrt(nt))-step segments and recompute them in the
                                      adjoint instead of the whole forward field */

/* Checks sizes, positions and the wavelet; GB_FWI2D_EINVAL codes on failure. */
int gb_fwi3d_validate(const gb_fwi3d_params *p, const gb_fwi3d_acq *a);

/* Device workspace for `nsamples` models with at most `max_resident`
 * (sample, shot) solves in flight (<= 0: all of them). */
int gb_fwi3d_workspace_size(const gb_fwi3d_params *p, const gb_fwi3d_acq *a, int nsamples,
                            int max_resident, unsigned flags, size_t *bytes);

/* Largest resident count whose workspace fits in `budget` bytes (0 if none). */
int gb_fwi3d_max_resident(const gb_fwi3d_params *p, const gb_fwi3d_acq *a, int nsamples,
                          unsigned flags, size_t budget);

/* One batch, stream-ordered, device buffers:
 *   vel    [nsamples][ny*nx*nz]  velocity, (ny, nx, nz) order, nz fastest
 *   obs    [ns][nt][nr]          observed data (ignored with FORWARD_ONLY unless misfit)
 *   syn    [nsamples][ns][nt][nr] synthetic data out (may be NULL)
 *   grad   [nsamples][ny*nx*nz]  dJ/dv out, model order (NULL with FORWARD_ONLY)
 *   misfit [nsamples]            0.5 * sum((syn - obs)^2) in FP64 out (may be NULL)
 * `work` is a device buffer of gb_fwi3d_workspace_size bytes. */
int gb_fwi3d_run(const gb_fwi3d_params *p, const gb_fwi3d_acq *a, int nsamples, const float *vel,
                 const float *obs, float *syn, float *grad, double *misfit, void *work, size_t work_bytes,
                 int max_resident, unsigned flags, void *stream);

/* Kernel launches of the calling thread's last gb_fwi3d_run. */
long long gb_fwi3d_last_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* GEOPVI_FWI3D_H */

/*
 * geopvi_fwi2d.h -- C ABI of the GB300 acoustic FWI engine.
 *
 * Drop-in boundary for GeoPVI's geopvi/forward/fwi2d solver.  The entry
 * points fall in three groups:
 *
 *  1. Exact replacements of the reference's C entry points that the Cython
 *     module `aco2d` binds (geopvi/forward/fwi2d/pyacofwi2D.h:2-3,
 *     pyacofwi2D.pyx:4-6): `fwi_2D` and `forward_2D`, same names, same
 *     argument meaning, host buffers, parameters read from the positional
 *     text file.  They return a status instead of calling exit().
 *  2. The parameter reader (read_parameters, fdtd2D_modelling.c:1328-1379)
 *     as a typed struct, so callers can skip the text file.
 *  3. The batched device API: every (sample, shot) solve of a batch runs on
 *     one GPU, stream-ordered, in caller-owned device buffers.  It replaces
 *     the per-sample loop of Posterior.fwi / Posterior.fwi_parallel
 *     (geopvi/forward/fwi2d/posterior.py:112-149).
 *
 * Plain pointers and sizes only; `stream` is a cudaStream_t passed as void*.
 * No entry point exits or aborts; all return GB_FWI2D_OK (0) or a negative
 * status code.
 */
#ifndef GEOPVI_FWI2D_H
#define GEOPVI_FWI2D_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define GB_FWI2D_OK 0
#define GB_FWI2D_ENOENT (-2)     /* parameter file missing */
#define GB_FWI2D_E2BIG (-7)      /* batch needs more than the static scratch (gb_fwi2d_batch_noalloc) */
#define GB_FWI2D_ENOMEM (-12)    /* device memory / workspace too small */
#define GB_FWI2D_EINVAL (-22)    /* bad geometry, sizes or pointers */
#define GB_FWI2D_ENOTSUP (-95)   /* a combination this library does not run (the exact gradient or the
                                    allocation-free entry with laplace_solver = 1), or the FFT
                                    library the pseudo-spectral mode loads is missing */
#define GB_FWI2D_ENAN (-1001)    /* NaN/Inf in the velocity input */
#define GB_FWI2D_ECUDA (-1002)   /* a CUDA runtime call failed */
#define GB_FWI2D_ETIMEOUT (-1003) /* a bounded device wait gave up (status word set) */

/* Solver parameters, in the order and with the types read_parameters uses
 * (fdtd2D_modelling.c:1328-1356; file layout written by
 * prepare_fwi_parameters, posterior.py:27-68).  Lc is the value in the file
 * (the half-order); the solver uses Lc+1 internally (fdtd2D_modelling.c:70). */
typedef struct gb_fwi2d_params {
    int nx, nz, pml0, Lc, laplace_solver, ns, nt, ds, ns0, depths, depthr, nr, dr, nr0,
        nt_interval;
    float dx, dz, dt, f0;
} gb_fwi2d_params;

/* Flags for gb_fwi2d_batch. */
#define GB_FWI2D_IMAGING 0x1u    /* run_fwi = 0: zero-lag imaging (record = obs, psave = p) */
#define GB_FWI2D_PLAIN 0x2u      /* one (sample, shot) per launch, shots in order (comparator) */
#define GB_FWI2D_GRAPH 0x4u      /* capture the step sequence once in a CUDA graph, replay after */
#define GB_FWI2D_CHECKPOINT 0x8u /* keep (p0,p1) every ~sqrt(nt) steps, recompute the forward per
                                    segment in the adjoint: 1.5x the steps, ~sqrt(nt)/nt_save the
                                    stored-field memory; results identical to full storage */
#define GB_FWI2D_FORWARD_ONLY 0x10u /* synthetic data only (forward_2D): no adjoint, no stored field */
#define GB_FWI2D_PROFILE 0x20u   /* time the step-kernel loops with CUDA events (not with GRAPH) */
/* Kernel variant of the FD time step (bits 8-11): 0 lets the library's tuner
 * choose -- the first calls with a given geometry, batch size, wave size and mode
 * each time one variant on the caller's own batch, later calls run the fastest;
 * GB_FWI2D_VARIANT(v) forces variant v (0-3).  Every variant computes the same
 * values bit for bit. */
#define GB_FWI2D_VARIANT_SHIFT 8
#define GB_FWI2D_VARIANT(v) ((unsigned)((v) + 1) << GB_FWI2D_VARIANT_SHIFT)
#define GB_FWI2D_EXACT_GRADIENT 0x40u /* grad = dJ/dv of J = 0.5*sum((syn-obs)^2), the exact discrete
                                        adjoint of the FD scheme (FP32), instead of backward_IO's
                                        gradient.  No counterpart in the reference.  Not with IMAGING;
                                        with CHECKPOINT the forward levels are kept per ~sqrt(nt)-step
                                        segment instead of for all nt steps */

/* read_parameters (fdtd2D_modelling.c:1328): parse the positional file. */
int gb_fwi2d_read_params(const char *path, gb_fwi2d_params *out);

/* Check a parameter set the way the solver needs it (grid, geometry inside
 * the padded grid, FD order, time sampling).  GB_FWI2D_OK or EINVAL.  laplace_solver 0
 * selects the FD stencil, 1 the pseudo-spectral Laplacian (double 2-D transforms through
 * cuFFT, loaded on first use). */
int gb_fwi2d_validate(const gb_fwi2d_params *p);

/* Drop-in for fwi_2D (fdtd2D_modelling.c:18-353, bound at pyacofwi2D.pyx:4).
 * Host buffers: vel_inner[nz*nx], record_obs[ns*nt*nr] (shot, time, receiver),
 * record_syn[ns*nt*nr] written, grad[nz*nx] ACCUMULATED (+=) as in the
 * reference.  run_fwi = 1: misfit gradient; 0: imaging condition. */
int fwi_2D(char input_file[200], float *vel_inner, float *record_syn, float *record_obs,
           float *grad, int run_fwi, int verbose);

/* Drop-in for forward_2D (fdtd2D_modelling.c:356-675, bound at pyacofwi2D.pyx:5):
 * synthetic data only, record_syn[ns*nt*nr]. */
int forward_2D(char input_file[200], float *vel_inner, float *record_syn, int run_fwi, int verbose);

/* Device-memory bytes gb_fwi2d_batch needs for `nsamples` models when at
 * most `max_resident` (sample, shot) solves hold their wavefield state at
 * once (0 = all of them).  The state of one solve is three padded wavefields,
 * the stored forward wavefield (or its checkpoints) and a gradient
 * accumulator; the batch runs in ceil(nsamples*ns / max_resident) waves. */
size_t gb_fwi2d_workspace_bytes(const gb_fwi2d_params *p, int nsamples, int max_resident,
                                unsigned flags);

/* Batched misfit + gradient on the device (replaces the sample loop of
 * Posterior.fwi, posterior.py:112-129, and the per-sample aco2d.fwi call,
 * pyacofwi2D.pyx:11-30).  Device pointers:
 *   vel    [nsamples][nz*nx]       velocity models (float32)
 *   obs    [ns][nt][nr]            observed data, shared by all samples
 *   syn    [nsamples][ns][nt][nr]  synthetic data out (may be NULL: kept in workspace)
 *   grad   [nsamples][nz*nx]       gradient out (overwritten, reference scaling)
 *   misfit [nsamples]              0.5*sum((syn-obs)^2) out, FP64 (may be NULL)
 * work/work_bytes: device workspace of at least
 * gb_fwi2d_workspace_bytes(p, nsamples, max_resident, flags).
 * Stream-ordered on `stream`; returns after enqueueing all work. */
int gb_fwi2d_batch(const gb_fwi2d_params *p, int nsamples, const float *vel, const float *obs,
                   float *syn, float *grad, double *misfit, unsigned flags, int max_resident,
                   void *work, size_t work_bytes, void *stream);

/* One entry of an uneven batch: its own parameter set (grid, shots, nt, f0
 * ...), number of models and device buffers, laid out as in gb_fwi2d_batch. */
typedef struct gb_fwi2d_instance {
    gb_fwi2d_params params;
    int nsamples;
    const float *vel;   /* [nsamples][nz*nx] */
    const float *obs;   /* [ns][nt][nr] */
    float *syn;         /* [nsamples][ns][nt][nr], or NULL */
    float *grad;        /* [nsamples][nz*nx], or NULL with GB_FWI2D_FORWARD_ONLY */
    double *misfit;     /* [nsamples], or NULL */
} gb_fwi2d_instance;

/* The smallest workspace for gb_fwi2d_run_instances; 0 if an instance is
 * invalid.  Fused instances (below) need their per-instance buffers and one
 * resident solve of the largest; the others reuse one workspace in stream
 * order and need the largest instance's gb_fwi2d_workspace_bytes.  A larger
 * workspace lets more solves share a wave. */
size_t gb_fwi2d_instances_workspace_bytes(const gb_fwi2d_instance *inst, int n, int max_resident,
                                          unsigned flags);

/* An uneven batch -- instances with different parameter sets -- on one
 * stream and one workspace.  Replaces the per-sample loop of
 * geopvi/forward/fwi2d/posterior.py:112-149 for callers whose samples belong
 * to different inversions.
 *
 * Fused (flags without GB_FWI2D_PLAIN, CHECKPOINT, EXACT_GRADIENT or GRAPH;
 * finite-difference instances; GB_FWI2D_VARIANT does not apply): the solves
 * of all instances
 * of one FD order are packed, longest nt first, into waves that fill
 * work_bytes (at most max_resident solves each when max_resident > 0), and a
 * wave advances all its solves -- of any grid, acquisition and time axis --
 * in one kernel launch per time step, with full storage of the forward
 * field.  Otherwise, and for pseudo-spectral instances, each instance runs
 * through the gb_fwi2d_batch path in turn.  Results are bit for bit those of
 * the instances run alone.
 *
 * Every instance is checked before anything is enqueued: an invalid one
 * returns its status (GB_FWI2D_EINVAL; GB_FWI2D_ENOMEM when work_bytes is
 * below gb_fwi2d_instances_workspace_bytes) and nothing runs.  A fused call
 * copies a small host table to the device, which stream capture does not
 * allow: on a stream being captured it returns GB_FWI2D_ENOTSUP, again
 * before anything is enqueued (GB_FWI2D_GRAPH runs the instances unfused,
 * each captured and replayed as gb_fwi2d_batch does).  The
 * workspace's status word (gb_fwi2d_status) collects the flags of every
 * instance of the call.  Concurrency across streams and memory admission for
 * mixed workloads are geopvi_gb300/scheduler.py's. */
int gb_fwi2d_run_instances(const gb_fwi2d_instance *inst, int n, unsigned flags, int max_resident,
                           void *work, size_t work_bytes, void *stream);

/* Host only: the number of fused waves gb_fwi2d_run_instances would run for
 * these instances in work_bytes (pseudo-spectral instances, which run alone,
 * count none); GB_FWI2D_EINVAL for flags that do not fuse or an invalid
 * instance, GB_FWI2D_ENOMEM below gb_fwi2d_instances_workspace_bytes.  Lets a
 * caller size the workspace: more bytes, fewer and wider waves. */
int gb_fwi2d_instances_waves(const gb_fwi2d_instance *inst, int n, unsigned flags, int max_resident,
                             size_t work_bytes);

/* Allocation-free variant of gb_fwi2d_batch.  No counterpart in the
 * reference (whose solver allocates and frees its own buffers on every call).
 *
 * For callers that cannot allocate device memory: a host whose device memory
 * belongs to another runtime or to a fixed pool, a latency-critical loop in
 * which an allocation would synchronize the device, or a plain C/FFI caller
 * with no way to provide a workspace.  Instead of a caller workspace it uses a
 * fixed array of GB_FWI2D_STATIC_SCRATCH_BYTES that the library reserves on
 * every GPU that loads it, until the process exits.  It calls no cudaMalloc,
 * cudaFree or allocating library routine.
 *
 * Inputs and outputs are the caller's device buffers, as in gb_fwi2d_batch
 * (syn may be NULL).  flags: GB_FWI2D_IMAGING, GB_FWI2D_FORWARD_ONLY,
 * GB_FWI2D_PLAIN and GB_FWI2D_CHECKPOINT only; with CHECKPOINT a solve keeps
 * ~sqrt(nt) wavefield pairs instead of its stored field, so a gradient batch
 * of realistic size fits (a 120 x 250, nt 2000 solve: ~26 MB instead of
 * ~250 MB).  The batch is split into as many waves as the scratch needs; a
 * batch whose per-sample state alone (padded v*dt, gradient accumulators,
 * synthetic data when syn is NULL) plus one resident solve does not fit
 * returns GB_FWI2D_E2BIG.  All work runs on `stream` alone: no stream or
 * event is created, and no host memory is copied (the boundary-weight table
 * is built by a kernel).  gb_fwi2d_status(NULL, stream) reads the status
 * word of the last call on the current device.
 *
 * The first call on a device looks up the array's device address (once per
 * device, with that device current); make that first call before any stream
 * capture.  Every call shares the one array, which keeps the last call's
 * contents (each call clears what must start at zero): calls that overlap on
 * the GPU -- on different streams, or from different threads -- race and
 * corrupt each other's results; serialize them. */
#define GB_FWI2D_STATIC_SCRATCH_BYTES (64u << 20)
int gb_fwi2d_batch_noalloc(const gb_fwi2d_params *p, int nsamples, const float *vel, const float *obs,
                           float *syn, float *grad, double *misfit, unsigned flags, void *stream);

/* Waits for `stream`, then reads the device status word at the start of a
 * workspace used by gb_fwi2d_batch: GB_FWI2D_OK, or GB_FWI2D_ETIMEOUT if a
 * kernel's bounded wait for its staged tiles gave up (results invalid).
 * work = NULL reads the status of gb_fwi2d_batch_noalloc on the current
 * device. */
int gb_fwi2d_status(const void *work, void *stream);

/* Diagnostic: the number of auxiliary CUDA streams the library holds (one
 * per device and host thread that ran gb_fwi2d_batch's two-stream schedule;
 * released by gb_fwi2d_release_caches).  No counterpart in the reference. */
int gb_fwi2d_side_stream_count(void);

/* Number of kernel launches the last gb_fwi2d_batch call on this thread
 * enqueued (graph replays count the kernels inside the graph). */
long long gb_fwi2d_last_launch_count(void);

/* gb_fwi2d_batch calls made with GB_FWI2D_PROFILE on this thread wrap each
 * pass's run of time-step kernels in a pair of CUDA events.  This waits for
 * the events recorded since the previous read, returns the summed device time
 * of those step kernels in milliseconds (negative if there were none) and in
 * *launches the number of step-kernel launches covered, then clears them. */
double gb_fwi2d_profile_step_ms(long long *launches);

/* The FD step variant the tuner settled on for this geometry, batch size
 * (nsamples), wave size (max_resident as passed to gb_fwi2d_batch) and flags:
 * 0-3, or -1 while variants remain untried.  No counterpart in the reference. */
int gb_fwi2d_tuned_variant(const gb_fwi2d_params *p, int nsamples, int max_resident, unsigned flags);

/* Release cached device tables and CUDA graphs held by the library. */
void gb_fwi2d_release_caches(void);

/* Library version string. */
const char *gb_fwi2d_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GEOPVI_FWI2D_H */

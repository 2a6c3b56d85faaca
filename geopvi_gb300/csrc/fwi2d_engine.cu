// fwi2d_engine.cu -- host side of the GB300 acoustic FWI engine and its C ABI.
//
// Replaces the drivers fwi_2D / forward_2D (geopvi/forward/fwi2d/
// fdtd2D_modelling.c:18-353, 356-675) and the per-sample loop of
// Posterior.fwi (geopvi/forward/fwi2d/posterior.py:112-129).  The reference
// runs shots one after another on the CPU, re-reads its parameter file and
// re-allocates every buffer per sample; here every (sample, shot) solve of a
// batch advances together, one fused kernel launch per time step, in a
// caller-owned device workspace, optionally replayed from a CUDA graph.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/geopvi_fwi2d.h"
#include "fwi2d_kernels.cuh"
#include "fwi2d_exact_adjoint.cuh"
#include "fwi2d_pstd.cuh"

namespace gbfwi {

// ---------------------------------------------------------------------------
// Parameter derivation (host)
// ---------------------------------------------------------------------------

// The reference's pi literal (fdtd2D_modelling.c:15).
static const double kRefPi = 3.1415926;

struct Derived {
    Geom g;
    std::vector<float> rik;   // Ricker wavelet per time step
    std::vector<BlendCoef> coef;  // boundary weights w and 1 - w (fdtd2D_modelling.c:227-230)
    bool blend_fp32 = false;      // every (1 - w) * q is exact in double
    std::vector<float> kk;        // pseudo-spectral mode: |k|^2 per padded cell, dense [ntz][ntx]
};

static int round_up(int v, int m) { return (v + m - 1) / m * m; }

// fd_coefficient (fdtd2D_modelling.c:1272-1326): double literals stored as
// float, from the same table the kernels use as immediates.
template <int H>
static void copy_weights(float *fd)
{
    for (int i = 0; i <= H; ++i) fd[i] = fd_weight<H>(i);
}

static void fd_weights(int Lc, float *fd)
{
    for (int i = 0; i < 8; ++i) fd[i] = 0.0f;
    switch (Lc) {
    case 4: copy_weights<3>(fd); break;
    case 5: copy_weights<4>(fd); break;
    case 6: copy_weights<5>(fd); break;
    case 7: copy_weights<6>(fd); break;
    default: break;
    }
}

// getrik (fdtd2D_modelling.c:1084-1093): the squared phase is held in a
// float, the wavelet evaluated in double and stored as float.
static void ricker(int nt, float dt, float f0, std::vector<float> &rik)
{
    rik.resize(nt);
    for (int it = 0; it < nt; ++it) {
        const float phase = (float)it * dt - 1.0f / f0;
        const double arg = kRefPi * f0 * (double)phase;
        const float a = (float)(arg * arg);
        rik[it] = (float)((1.0 - 2.0 * a) * std::exp((double)(-a)));
    }
}

static int validate(const gb_fwi2d_params &p)
{
    if (p.nx <= 0 || p.nz <= 0 || p.ns <= 0 || p.nt <= 0 || p.nr <= 0) return GB_FWI2D_EINVAL;
    if (p.pml0 <= 0 || p.nt_interval <= 0) return GB_FWI2D_EINVAL;
    if (!(p.dx > 0.0f) || !(p.dz > 0.0f) || !(p.dt > 0.0f) || !(p.f0 > 0.0f)) return GB_FWI2D_EINVAL;
    if (p.laplace_solver != 0 && p.laplace_solver != 1) return GB_FWI2D_EINVAL;
    if (p.Lc < 3 || p.Lc > 6) return GB_FWI2D_EINVAL;     // fd_coefficient: Lc+1 in 4..7
    if (p.nr > 1 && p.dr == 0) return GB_FWI2D_EINVAL;    // receivers would share one cell
    // The pseudo-spectral mode sets Lc = 0 before pml = pml0 + Lc (fdtd2D_modelling.c:75-78).
    const long long Lc = p.laplace_solver == 1 ? 0 : p.Lc + 1, pml = p.pml0 + Lc;
    const long long ntz = p.nz + 2 * pml, ntx = p.nx + 2 * pml;
    if (ntz > (1 << 20) || ntx > (1 << 20) || ntz * ntx > (1LL << 31)) return GB_FWI2D_EINVAL;
    const long long s_iz = pml + p.depths, r_iz = pml + p.depthr;
    if (s_iz < 0 || s_iz >= ntz || r_iz < 0 || r_iz >= ntz) return GB_FWI2D_EINVAL;
    for (long long is : {0LL, (long long)p.ns - 1}) {
        long long s_ix = is * p.ds + pml + p.ns0;
        if (s_ix < 0 || s_ix >= ntx) return GB_FWI2D_EINVAL;
    }
    for (long long ir : {0LL, (long long)p.nr - 1}) {
        long long r_ix = pml + ir * p.dr + p.nr0;
        if (r_ix < 0 || r_ix >= ntx) return GB_FWI2D_EINVAL;
    }
    return GB_FWI2D_OK;
}

// Exhaustive proof, per divisor y, that div_const (kernels) returns the
// correctly rounded x/y: every significand of the binade [1, 2) is checked
// against the host's IEEE division; the quotient, the FMA remainder and the
// correction scale exactly with x, so the result holds for every
// 2^-56 <= |x| <= 2^56 while y stays within [2^-20, 2^20].  Cached per y.
static bool division_is_exact(float y)
{
    static std::mutex m;
    static std::map<uint32_t, bool> cache;
    uint32_t key;
    std::memcpy(&key, &y, sizeof key);
    {
        std::lock_guard<std::mutex> lk(m);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    bool ok = std::isfinite(y) && y >= 0x1p-20f && y <= 0x1p20f;
    const float r = 1.0f / y;
    for (uint32_t mant = 0; ok && mant < (1u << 23); ++mant) {
        const uint32_t bits = 0x3F800000u | mant;
        float x;
        std::memcpy(&x, &bits, sizeof x);
        const float q0 = x * r;
        const float rem = std::fma(-q0, y, x);
        const float q = std::fma(rem, r, q0);
        if (q != x / y) ok = false;
    }
    std::lock_guard<std::mutex> lk(m);
    cache[key] = ok;
    return ok;
}

// Number of significant bits of a finite double (0 for zero).
static int significant_bits(double v)
{
    if (v == 0.0) return 0;
    int e;
    double m = std::frexp(std::fabs(v), &e);  // m in [0.5, 1)
    uint64_t bits = (uint64_t)std::ldexp(m, 53);
    int n = 53;
    while (n > 0 && !(bits & 1u)) {
        bits >>= 1;
        --n;
    }
    return n;
}

// wavenumber (fdtd2D_modelling.c:1127-1184): |k|^2 of the padded grid's DFT
// bins.  dkx = 1/ntx/dx is stored as float; each component 2 pi dkx j (pi the
// reference's 3.1415926, j = min(ix, ntx - ix) with the upper half starting
// at ceil(ntx/2)) is stored as float; the squares are summed in double and
// the sum stored as float.
static void wavenumber(int ntx, int ntz, float dx, float dz, std::vector<float> &k)
{
    const float dkz = (float)(1.0 / ntz / dz), dkx = (float)(1.0 / ntx / dx);
    const int ax = ntx / 2 * 2 < ntx ? ntx / 2 + 1 : ntx / 2;
    const int az = ntz / 2 * 2 < ntz ? ntz / 2 + 1 : ntz / 2;
    k.assign((size_t)ntx * ntz, 0.0f);
    for (int iz = 0; iz < ntz; ++iz)
        for (int ix = 0; ix < ntx; ++ix) {
            const float kz = (float)(2 * kRefPi * dkz * (iz < az ? iz : ntz - iz));
            const float kx = (float)(2 * kRefPi * dkx * (ix < ax ? ix : ntx - ix));
            k[(size_t)iz * ntx + ix] = (float)((double)kx * (double)kx + (double)kz * (double)kz);
        }
}

// Memory column of padded ix = 0.  The step kernel's 32-column tiles are
// rim-only (no column in [Lc, ntx - Lc): zeros stored, no stencil), interior
// (every column in [pml, ntx - pml): the lean sweep) or general (absorbing
// strips: per-cell region tests and blends for the whole warp, about 2.5x
// an interior tile).  The offset minimises that cost; the smallest wins ties.
static int column_offset(int ntx, int Lc, int pml)
{
    int best = 0;
    long long best_cost = -1;
    for (int xoff = 0; xoff < kTileX; ++xoff) {
        const int tiles = (xoff + ntx + kTileX - 1) / kTileX;
        long long cost = 0;
        for (int t = 0; t < tiles; ++t) {
            const int lo = t * kTileX - xoff, hi = lo + kTileX;
            if (hi <= Lc || lo >= ntx - Lc) cost += 1;
            else if (lo >= pml && hi <= ntx - pml) cost += 4;
            else cost += 10;
        }
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = xoff;
        }
    }
    return best;
}

static int derive(const gb_fwi2d_params &p, Derived &d)
{
    int st = validate(p);
    if (st) return st;
    Geom &g = d.g;
    std::memset(&g, 0, sizeof g);
    // The pseudo-spectral Laplacian has no stencil halo: the reference sets
    // Lc = 0 before pml = pml0 + Lc (fdtd2D_modelling.c:75-78), so its
    // absorbing strips start at the grid's edge and there is no rim.
    g.Lc = p.laplace_solver == 1 ? 0 : p.Lc + 1;
    g.pml = p.pml0 + g.Lc;
    g.pml0 = p.pml0;
    g.ntz = p.nz + 2 * g.pml;
    g.ntx = p.nx + 2 * g.pml;
    g.xoff = column_offset(g.ntx, g.Lc, g.pml);
    g.pitch = round_up(g.xoff + g.ntx, kTileX);
    g.nx = p.nx;
    g.nz = p.nz;
    // Interior arrays (snapshots, gradient sums) share the tiles' 128-byte
    // lines: interior column 0 sits at the memory column of padded ix = pml.
    g.ioff = (g.xoff + g.pml) % kTileX;
    g.ipitch = round_up(g.ioff + p.nx, kTileX);
    g.s_iz = g.pml + p.depths;
    g.r_iz = g.pml + p.depthr;
    g.r_ix0 = g.pml + p.nr0;
    g.dr = p.dr;
    g.nr = p.nr;
    g.ds = p.ds;
    g.s_ix0 = g.pml + p.ns0;
    g.ns = p.ns;
    g.nt = p.nt;
    g.nti = p.nt_interval;
    g.nt_save = p.nt / p.nt_interval + ((p.nt % p.nt_interval) ? 1 : 0);
    g.tiles_x = g.pitch / kTileX;
    g.tiles_z = (g.ntz + kTileZ - 1) / kTileZ;
    g.fstride = (long long)g.ntz * g.pitch;
    g.pstride = (long long)g.nz * g.ipitch;
    g.dx = p.dx;
    g.dz = p.dz;
    g.dt = p.dt;
    fd_weights(g.Lc, g.fd);
    g.rdx = 1.0f / p.dx;
    g.rdz = 1.0f / p.dz;
    g.fast_dx = division_is_exact(p.dx) ? 1 : 0;
    g.fast_dz = division_is_exact(p.dz) ? 1 : 0;
    ricker(p.nt, p.dt, p.f0, d.rik);
    g.pstd = p.laplace_solver == 1 ? 1 : 0;
    if (g.pstd) wavenumber(g.ntx, g.ntz, p.dx, p.dz, d.kk);
    d.coef.resize(p.pml0);
    d.blend_fp32 = true;
    for (int i = 0; i < p.pml0; ++i) {
        BlendCoef &c = d.coef[i];
        blend_coef_init(c, i, p.pml0);  // w = 1 - i/pml0, fdtd2D_modelling.c:229
        // The FP32 blend needs bh + bl == 1 - w exactly and (1 - w) * q exact in
        // double for any float q: 1 - w may hold at most 53 - 24 = 29 significant bits.
        if ((double)c.bh + (double)c.bl != c.omw || significant_bits(c.omw) > 29) d.blend_fp32 = false;
    }
    return GB_FWI2D_OK;
}

// ---------------------------------------------------------------------------
// Workspace layout
// ---------------------------------------------------------------------------

struct Layout {
    size_t status, vdt, ring, psave, gacc, syn, part, total;
    size_t ring2, ckpt;  // checkpointing only: the adjoint's ring and the stored (p0, p1) pairs
    size_t store, lam, nu, gpad;  // exact gradient only: forward levels, adjoint levels and their
                                  // a beta lambda, padded dJ/dv
    size_t abeta, cells;      // exact gradient only: per-sample (v dt)^2 beta, the geometry's cell table
    size_t taps;              // exact gradient only: per-sample blend taps (kTapPlanes fields)
    size_t spec;              // pseudo-spectral mode: real field + half spectrum per resident solve
    int resident;
    int ckpt_k, ckpt_nseg;  // checkpointing only: steps per segment, segments
};

// sqrt(nt) checkpointing: segments of K steps (K a multiple of nt_interval,
// so every segment's stored steps are contiguous), one (p0, p1) pair kept
// per segment.
static void checkpoint_plan(const Geom &g, int &K, int &nseg)
{
    const int root = (int)std::ceil(std::sqrt((double)g.nt));
    K = (root + g.nti - 1) / g.nti * g.nti;
    nseg = (g.nt + K - 1) / K;
}

constexpr int kMisfitBlocks = 64;  // partial sums per sample for the misfit

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Exact gradient: the adjoint needs every forward level, kept either for all
// nt steps (one segment) or, with checkpointing, for one ceil(sqrt(nt))-step
// segment at a time: store holds the segment's levels P^{i0-1} .. P^{i0+K},
// K+2 of them, which the forward steps write in place.
static Layout plan_layout_exact(const Geom &g, int nsamples, int resident, bool syn_in_work, bool checkpoint)
{
    Layout L{};
    const long long ninst = (long long)nsamples * g.ns;
    L.resident = resident;
    L.ckpt_k = checkpoint ? std::max(1, (int)std::ceil(std::sqrt((double)g.nt))) : g.nt;
    L.ckpt_nseg = (g.nt + L.ckpt_k - 1) / L.ckpt_k;
    const size_t field = sizeof(float) * g.fstride;
    size_t off = 0;
    L.status = off; off = align256(off + sizeof(int));
    L.vdt = off;    off = align256(off + field * nsamples);
    L.ring = off;   off = align256(off + field * 3 * resident);
    L.ckpt = off;
    if (L.ckpt_nseg > 1) off = align256(off + field * 2 * L.ckpt_nseg * resident);
    L.store = off;  off = align256(off + field * (L.ckpt_k + 2) * resident);
    L.lam = off;    off = align256(off + field * 3 * resident);
    L.nu = off;     off = align256(off + field * 3 * resident);
    L.gpad = off;   off = align256(off + field * ninst);
    L.abeta = off;  off = align256(off + field * nsamples);
    L.cells = off;  off = align256(off + sizeof(int4) * (size_t)g.ntz * g.ntx);
    L.taps = off;   off = align256(off + field * kTapPlanes * nsamples);
    L.psave = L.gacc = off;
    L.syn = off;
    if (syn_in_work) off = align256(off + sizeof(float) * (size_t)ninst * g.nt * g.nr);
    L.part = off;   off = align256(off + sizeof(double) * kMisfitBlocks * nsamples);
    L.total = off;
    return L;
}

static Layout plan_layout(const Geom &g, int nsamples, int resident, bool syn_in_work,
                          bool forward_only, bool checkpoint = false, bool exact = false)
{
    Layout L{};
    const long long ninst = (long long)nsamples * g.ns;
    if (resident <= 0 || resident > ninst) resident = (int)ninst;
    if (exact && !forward_only) return plan_layout_exact(g, nsamples, resident, syn_in_work, checkpoint);
    L.resident = resident;
    checkpoint = checkpoint && !forward_only;
    long long snaps = g.nt_save;  // stored steps per resident solve
    if (checkpoint) {
        checkpoint_plan(g, L.ckpt_k, L.ckpt_nseg);
        snaps = L.ckpt_k / g.nti;
    }
    size_t off = 0;
    L.status = off; off = align256(off + sizeof(int));
    L.vdt = off;   off = align256(off + sizeof(float) * g.fstride * nsamples);
    L.ring = off;  off = align256(off + sizeof(float) * g.fstride * 3 * resident);
    if (checkpoint) {
        L.ring2 = off; off = align256(off + sizeof(float) * g.fstride * 3 * resident);
        L.ckpt = off;  off = align256(off + sizeof(float) * g.fstride * 2 * L.ckpt_nseg * resident);
    }
    L.psave = off;
    if (!forward_only) off = align256(off + sizeof(float) * g.pstride * snaps * resident);
    L.gacc = off;
    if (!forward_only) off = align256(off + sizeof(float) * g.pstride * ninst);
    L.syn = off;
    if (syn_in_work) off = align256(off + sizeof(float) * (size_t)ninst * g.nt * g.nr);
    L.part = off;  off = align256(off + sizeof(double) * kMisfitBlocks * nsamples);
    L.spec = off;
    if (g.pstd)
        off = align256(off + align256(sizeof(double) * (size_t)g.ntz * g.ntx * resident) +
                       sizeof(double2) * (size_t)g.ntz * (g.ntx / 2 + 1) * resident);
    L.total = off;
    return L;
}

// ---------------------------------------------------------------------------
// Auxiliary kernels
// ---------------------------------------------------------------------------

// Padded v*dt for every sample: get_velp's replication (a clamp) times dt,
// the float product that powf(v*dt, 2) and s = v*dt/dx start from.
__global__ void k_prepare(const Geom g, const float *__restrict__ vel, float *__restrict__ vdt,
                          int nsamples)
{
    const long long total = (long long)nsamples * g.fstride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(e / g.fstride);
        const long long r = e - (long long)s * g.fstride;
        const int iz = (int)(r / g.pitch);
        const int ix = (int)(r - (long long)iz * g.pitch) - g.xoff;
        float v = 0.0f;
        if (ix >= 0 && ix < g.ntx)
            v = fm(padded_velocity(g, vel + (long long)s * g.nx * g.nz, iz, ix), g.dt);
        vdt[e] = v;
    }
}

// grad[s][cell] = sum over shots, in double, of the per-shot accumulated
// sum(psave * p2), times the reference's per-term factor
// -2/powf(v,3) * nt_interval * dt (FWI) or nt_interval * dt (imaging).  In FWI
// mode the stored field is p2 - 2 p1 + p0, not the reference's
// (p2 - 2 p1 + p0)/dt/dt (backward_IO's psave, fdtd2D_modelling.c:902-939):
// the 1/dt^2 is applied here, once per cell in FP64, instead of two
// correctly rounded divisions per cell and stored step.
__global__ void k_reduce_grad(const Geom g, const float *__restrict__ gacc,
                              const float *__restrict__ vel, float *__restrict__ grad,
                              int nsamples, int imaging)
{
    const long long cells = (long long)g.nz * g.nx;
    const long long total = (long long)nsamples * cells;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(e / cells);
        const long long k = e - (long long)s * cells;
        const int iz = (int)(k / g.nx), ix = (int)(k - (long long)iz * g.nx);
        const long long pc = (long long)iz * g.ipitch + ix + g.ioff;
        double acc = 0.0;
        for (int shot = 0; shot < g.ns; ++shot)
            acc += (double)gacc[((long long)s * g.ns + shot) * g.pstride + pc];
        double coef = (double)g.nti * (double)g.dt;
        if (!imaging) {
            const double v = (double)vel[e];
            const float v3 = __double2float_rn(v * v * v);  // powf(v, 3) as a rounded float
            coef = (-2.0 / (double)v3) * coef / ((double)g.dt * (double)g.dt);
        }
        grad[e] = __double2float_rn(coef * acc);
    }
}

// Misfit 0.5*sum((syn-obs)^2) per sample: float residual as the reference
// forms it (record -= obs), squares summed in double.  Two fixed-order
// passes keep the result deterministic.
__global__ void k_misfit_partial(const float *__restrict__ syn, const float *__restrict__ obs,
                                 long long per_sample, double *__restrict__ part)
{
    const int s = blockIdx.y;
    const float *sy = syn + (long long)s * per_sample;
    double acc = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per_sample;
         e += (long long)gridDim.x * blockDim.x) {
        const float r = fs(sy[e], obs[e]);
        acc += (double)r * (double)r;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double warp_sums[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) warp_sums[wid] = acc;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        acc = lane < nw ? warp_sums[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) part[(long long)s * gridDim.x + blockIdx.x] = acc;
    }
}

__global__ void k_misfit_final(const double *__restrict__ part, double *__restrict__ misfit,
                               int nsamples)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsamples) return;
    double acc = 0.0;
    for (int i = 0; i < kMisfitBlocks; ++i) acc += part[(long long)s * kMisfitBlocks + i];
    misfit[s] = 0.5 * acc;
}

// The boundary weights of derive() (w = 1 - i/pml0, fdtd2D_modelling.c:227-230,
// the split of 1 - w and blend_fast's constants) built on the device, for
// callers that must not copy from host memory.  blend_coef_init uses only
// correctly rounded IEEE operations, so the table equals the host's bit for bit.
__global__ void k_blend_coef(int pml0, BlendCoef *coef)
{
    for (int i = threadIdx.x; i < pml0; i += blockDim.x) {
        BlendCoef c;
        blend_coef_init(c, i, pml0);
        coef[i] = c;
    }
}

// ---------------------------------------------------------------------------
// Cached per-device tables and graphs
// ---------------------------------------------------------------------------

struct DeviceTables {
    BlendCoef *coef = nullptr;
};

struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
};

static std::mutex g_mutex;
static std::map<std::pair<int, int>, DeviceTables> g_tables;  // (device, pml0)
static std::map<std::vector<long long>, GraphEntry> g_graphs;
static thread_local long long t_last_launches = 0;

// Event pairs around the step-kernel loops of profiled calls, accumulated
// until gb_fwi2d_profile_step_ms reads (and clears) them.
struct StepProfile {
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> spans;
    long long launches = 0;
    void reset()
    {
        for (auto &e : spans) {
            cudaEventDestroy(e.first);
            cudaEventDestroy(e.second);
        }
        spans.clear();
        launches = 0;
    }
};
static thread_local StepProfile t_profile;

static int get_tables(const Derived &d, DeviceTables &out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GB_FWI2D_ECUDA;
    std::lock_guard<std::mutex> lk(g_mutex);
    auto key = std::make_pair(dev, d.g.pml0);
    auto it = g_tables.find(key);
    if (it != g_tables.end()) {
        out = it->second;
        return GB_FWI2D_OK;
    }
    DeviceTables t;
    const size_t bytes = sizeof(BlendCoef) * d.coef.size();
    if (cudaMalloc(&t.coef, bytes) != cudaSuccess) return GB_FWI2D_ENOMEM;
    if (cudaMemcpy(t.coef, d.coef.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(t.coef);
        return GB_FWI2D_ECUDA;
    }
    g_tables[key] = t;
    out = t;
    return GB_FWI2D_OK;
}

// ---------------------------------------------------------------------------
// Launch sequence
// ---------------------------------------------------------------------------

// cuTensorMapEncodeTiled, fetched from the driver through the runtime.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

// Encoding a tensor map needs a current driver context, and a host thread
// that has made no runtime call that binds one (cudaGetDevice and
// cudaGetLastError do not) has none.  Bind the current device's primary
// context then -- but leave a context the caller made current alone.
static bool ensure_context()
{
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
    });
    CUcontext ctx = nullptr;
    if (get_current && get_current(&ctx) == CUDA_SUCCESS && ctx) return true;
    int dev = 0;
    return cudaGetDevice(&dev) == cudaSuccess && cudaSetDevice(dev) == cudaSuccess;
}

// A 3-D fp32 tensor map over `depth` padded fields [depth][ntz][pitch] with a
// (box_x, box_z, 1) box; out-of-range elements of a box read as zero.
static bool make_map(CUtensorMap &m, void *base, const Geom &g, long long depth, int box_x, int box_z)
{
    auto enc = tensor_map_encoder();
    if (!enc || !ensure_context()) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.pitch, (cuuint64_t)g.ntz, (cuuint64_t)depth};
    const cuuint64_t strides[2] = {(cuuint64_t)g.pitch * 4, (cuuint64_t)g.fstride * 4};
    const cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_z, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct Maps {
    CUtensorMap p1;
};

// First failure status of the launches being enqueued on this thread.
static thread_local int t_enqueue_error = 0;

// Second stream of the main loop's two-halves schedule, per (device, host
// thread), with its fork / join events.  Kept for the process (a graph
// capture records work on it) and freed by gb_fwi2d_release_caches.
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
static std::mutex g_side_mutex;
static std::map<std::pair<int, std::thread::id>, SideStream> g_side;

// This thread's side stream on the current device; created on first use
// unless `create` is false (a stream being captured by the caller).
static const SideStream *side_stream(bool create)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_side_mutex);
    const auto key = std::make_pair(dev, std::this_thread::get_id());
    auto it = g_side.find(key);
    if (it != g_side.end()) return &it->second;
    if (!create) return nullptr;
    SideStream ss;
    if (cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    if (cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ss.join, cudaEventDisableTiming) != cudaSuccess) {
        if (ss.fork) cudaEventDestroy(ss.fork);
        cudaStreamDestroy(ss.s);
        return nullptr;
    }
    return &(g_side[key] = ss);
}

// Waves of at least this many resident solves run as two halves on two
// streams: each half's steps form their own chain, so the ramp and tail of
// one half's launches overlap the other half's work.
constexpr int kSplitMinResident = 32;

static bool make_maps(Maps &m, const Geom &g, float *ring, int resident)
{
    return make_map(m.p1, ring, g, 3LL * resident, kBoxX, kTileZ + 2 * (g.Lc - 1));
}

// overlap: the previous operation on `st` is the step before this one, and
// this step may be launched programmatically (its blocks become resident
// while that step drains; k_step waits on it before any global access).
template <int H, int U, int MINB>
static void launch_step_variant(bool adj, const Maps &m, const Geom &g, const Batch &b, int nres,
                                const StepArgs &sa, cudaStream_t st, bool overlap)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nres, g.tiles_x * g.tiles_z);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = TileShape<H>::kSmem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = overlap ? 1 : 0;
    const cudaError_t e = adj ? cudaLaunchKernelEx(&cfg, k_step<H, true, U, MINB>, m.p1, g, b, sa)
                              : cudaLaunchKernelEx(&cfg, k_step<H, false, U, MINB>, m.p1, g, b, sa);
    if (e != cudaSuccess) t_enqueue_error = GB_FWI2D_ECUDA;
}

template <int H>
static void launch_step(bool adj, const Maps &m, const Geom &g, const Batch &b, int nres,
                        const StepArgs &sa, cudaStream_t st, int variant, bool overlap)
{
    static_assert(kNumStepVariants == 4, "one case per entry of kStepVariants");
    constexpr StepVariant v1 = kStepVariants[1], v2 = kStepVariants[2], v3 = kStepVariants[3],
                          v0 = kStepVariants[0];
    switch (variant) {
    case 1: launch_step_variant<H, v1.rows, v1.min_blocks>(adj, m, g, b, nres, sa, st, overlap); break;
    case 2: launch_step_variant<H, v2.rows, v2.min_blocks>(adj, m, g, b, nres, sa, st, overlap); break;
    case 3: launch_step_variant<H, v3.rows, v3.min_blocks>(adj, m, g, b, nres, sa, st, overlap); break;
    default: launch_step_variant<H, v0.rows, v0.min_blocks>(adj, m, g, b, nres, sa, st, overlap); break;
    }
}

// ---------------------------------------------------------------------------
// Pseudo-spectral mode: cuFFT, loaded on first use (the FD path needs no
// FFT library), batched 2-D Z2Z plans cached per (device, grid, batch).
// ---------------------------------------------------------------------------
struct CufftApi {
    decltype(&cufftPlanMany) plan_many = nullptr;
    decltype(&cufftSetStream) set_stream = nullptr;
    decltype(&cufftExecD2Z) exec_d2z = nullptr;
    decltype(&cufftExecZ2D) exec_z2d = nullptr;
    decltype(&cufftDestroy) destroy = nullptr;
};

static const CufftApi *cufft_api()
{
    static CufftApi api;
    static bool tried = false, ok = false;
    std::lock_guard<std::mutex> lk(g_mutex);
    if (!tried) {
        tried = true;
        void *h = nullptr;
        for (const char *name : {"libcufft.so.12", "libcufft.so", "/usr/local/cuda/lib64/libcufft.so.12"})
            if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
        if (h) {
            api.plan_many = (decltype(api.plan_many))dlsym(h, "cufftPlanMany");
            api.set_stream = (decltype(api.set_stream))dlsym(h, "cufftSetStream");
            api.exec_d2z = (decltype(api.exec_d2z))dlsym(h, "cufftExecD2Z");
            api.exec_z2d = (decltype(api.exec_z2d))dlsym(h, "cufftExecZ2D");
            api.destroy = (decltype(api.destroy))dlsym(h, "cufftDestroy");
            ok = api.plan_many && api.set_stream && api.exec_d2z && api.exec_z2d && api.destroy;
        }
    }
    return ok ? &api : nullptr;
}

static std::map<std::tuple<int, int, int, int, int>, cufftHandle> g_fft_plans;  // (device, ntz, ntx, batch, dir)
static std::map<std::tuple<int, int, int, uint32_t, uint32_t>, float *> g_kk_tables;  // (device, ntz, ntx, dx, dz)

// Batched 2-D plans for `batch` fields: real [ntz][ntx] -> half spectrum
// [ntz][ntx/2+1] (forward, D2Z) or back (inverse, Z2D), out of place.
static int fft_plan(const Geom &g, int batch, bool inverse, cufftHandle *out)
{
    const CufftApi *api = cufft_api();
    if (!api) return GB_FWI2D_ENOTSUP;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GB_FWI2D_ECUDA;
    std::lock_guard<std::mutex> lk(g_mutex);
    const auto key = std::make_tuple(dev, g.ntz, g.ntx, batch, inverse ? 1 : 0);
    auto it = g_fft_plans.find(key);
    if (it != g_fft_plans.end()) {
        *out = it->second;
        return GB_FWI2D_OK;
    }
    cufftHandle h;
    int n[2] = {g.ntz, g.ntx};
    int rn[2] = {g.ntz, g.ntx}, cn[2] = {g.ntz, g.ntx / 2 + 1};
    const int rdist = g.ntz * g.ntx, cdist = g.ntz * (g.ntx / 2 + 1);
    const cufftResult r = inverse ? api->plan_many(&h, 2, n, cn, 1, cdist, rn, 1, rdist, CUFFT_Z2D, batch)
                                  : api->plan_many(&h, 2, n, rn, 1, rdist, cn, 1, cdist, CUFFT_D2Z, batch);
    if (r != CUFFT_SUCCESS) return GB_FWI2D_ENOMEM;
    g_fft_plans[key] = h;
    *out = h;
    return GB_FWI2D_OK;
}

// The |k|^2 table of a geometry on the current device (cached).
static int kk_table(const Derived &d, const float **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GB_FWI2D_ECUDA;
    uint32_t bx, bz;
    std::memcpy(&bx, &d.g.dx, 4);
    std::memcpy(&bz, &d.g.dz, 4);
    std::lock_guard<std::mutex> lk(g_mutex);
    const auto key = std::make_tuple(dev, d.g.ntz, d.g.ntx, bx, bz);
    auto it = g_kk_tables.find(key);
    if (it != g_kk_tables.end()) {
        *out = it->second;
        return GB_FWI2D_OK;
    }
    float *t = nullptr;
    const size_t bytes = sizeof(float) * d.kk.size();
    if (cudaMalloc(&t, bytes) != cudaSuccess) return GB_FWI2D_ENOMEM;
    if (cudaMemcpy(t, d.kk.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(t);
        return GB_FWI2D_ECUDA;
    }
    g_kk_tables[key] = t;
    *out = t;
    return GB_FWI2D_OK;
}

// One pseudo-spectral time step of the wave's nres solves: pack p1, forward
// transform, times -|k|^2, inverse transform, then the per-cell update and
// the rest of the step.  Returns the number of this library's kernels.
static int step_pstd(bool adj, const Geom &g, const Batch &b, int nres, const StepArgs &sa, cudaStream_t st)
{
    cufftHandle fwd, inv;
    const CufftApi *api = cufft_api();
    if (!api || fft_plan(g, nres, false, &fwd) != GB_FWI2D_OK || fft_plan(g, nres, true, &inv) != GB_FWI2D_OK) {
        t_enqueue_error = GB_FWI2D_ENOTSUP;
        return 0;
    }
    const long long n = (long long)g.ntz * g.ntx;
    double *real = b.spec;
    cufftDoubleComplex *half = reinterpret_cast<cufftDoubleComplex *>(
        (char *)b.spec + align256(sizeof(double) * (size_t)n * b.spec_resident));
    const dim3 grid((unsigned)std::min<long long>((n + 255) / 256, 1024), nres);
    k_pstd_pack<<<grid, 256, 0, st>>>(g, b.ring, (sa.k + 1) % 3, real);
    if (api->set_stream(fwd, st) != CUFFT_SUCCESS || api->exec_d2z(fwd, real, half) != CUFFT_SUCCESS)
        t_enqueue_error = GB_FWI2D_ECUDA;
    k_pstd_scale<<<grid, 256, 0, st>>>(g, b.kk, reinterpret_cast<double2 *>(half));
    if (api->set_stream(inv, st) != CUFFT_SUCCESS || api->exec_z2d(inv, half, real) != CUFFT_SUCCESS)
        t_enqueue_error = GB_FWI2D_ECUDA;
    const dim3 cells((unsigned)((n + 255) / 256), nres);
    if (adj)
        k_step_pstd<true><<<cells, 256, 0, st>>>(g, b, sa, real);
    else
        k_step_pstd<false><<<cells, 256, 0, st>>>(g, b, sa, real);
    return 3;
}

// One time step of the wave; returns the number of this library's kernels.
static int step(bool adj, const Maps &m, const Geom &g, const Batch &b, int nres, const StepArgs &sa,
                cudaStream_t st, int variant, bool overlap = false)
{
    if (g.pstd) return step_pstd(adj, g, b, nres, sa, st);
    switch (g.Lc - 1) {
    case 3: launch_step<3>(adj, m, g, b, nres, sa, st, variant, overlap); break;
    case 4: launch_step<4>(adj, m, g, b, nres, sa, st, variant, overlap); break;
    case 5: launch_step<5>(adj, m, g, b, nres, sa, st, variant, overlap); break;
    default: launch_step<6>(adj, m, g, b, nres, sa, st, variant, overlap); break;
    }
    return 1;
}

struct Call {
    const Derived *d;
    DeviceTables tab;
    Layout L;
    int nsamples;
    const float *vel, *obs;
    float *syn, *grad;
    double *misfit;
    unsigned flags;
    char *work;
    bool profile;
    Maps maps;
    Maps maps2;  // checkpointing: the adjoint's ring; exact gradient: the store
    Maps maps3;  // exact gradient: nu beside the adjoint levels
    const float *kk = nullptr;  // pseudo-spectral mode: |k|^2 table on the device
    int variant = 0;            // k_step variant (kStepVariants)
    bool single_stream = false; // never fork onto the side stream (no stream or event is created)
    bool clear_status = true;   // zero the status word first (false: keep an earlier call's flags)
    // Tuning: waves [0, trials.size()) run variant trials[i] between events
    // trial_ev[i]; later waves run `variant`.
    std::vector<int> trials;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> trial_ev;
    int wave_variant(long long wave) const { return wave < (long long)trials.size() ? trials[wave] : variant; }
};

static int grid_for(long long n, int threads)
{
    long long b = (n + threads - 1) / threads;
    return (int)std::min<long long>(std::max<long long>(b, 1), 152 * 16);
}

// One wave with sqrt(nt) checkpointing: the forward pass keeps (p0, p1) at the
// start of every K-step segment instead of every stored step; the adjoint then
// walks the segments backwards, restoring each pair into the forward ring,
// recomputing that segment's forward steps (which store its snapshots) and
// running the segment's adjoint steps in a second ring.  The recomputation runs
// the same kernel on the same inputs, so the snapshots -- and the gradient --
// are bit for bit those of full storage.
static long long enqueue_checkpointed(const Call &c, Batch b, int nres, cudaStream_t st)
{
    Geom g = c.d->g;
    const int K = c.L.ckpt_k, nseg = c.L.ckpt_nseg;
    g.nt_save = K / g.nti;  // snapshot slots per resident solve: one segment's
    float *ring = (float *)(c.work + c.L.ring);
    float *ring2 = (float *)(c.work + c.L.ring2);
    float *ck = (float *)(c.work + c.L.ckpt);
    const size_t fbytes = sizeof(float) * g.fstride;
    const size_t ring_pitch = 3 * fbytes, ck_pitch = 2 * (size_t)nseg * fbytes;
    long long launches = 0;
    auto profile_span = [&](cudaEvent_t &e0, cudaEvent_t &e1) {
        e0 = e1 = nullptr;
        if (c.profile && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess)
            cudaEventRecord(e0, st);
    };
    auto close_span = [&](cudaEvent_t e0, cudaEvent_t e1, long long n) {
        if (!e1) return;
        cudaEventRecord(e1, st);
        t_profile.spans.emplace_back(e0, e1);
        t_profile.launches += n;
    };
    cudaEvent_t e0, e1;

    // forward: data only, checkpoints at segment starts
    b.ring = ring;
    b.store = 0;
    cudaMemset2DAsync(ring, ring_pitch, 0, 2 * fbytes, nres, st);
    profile_span(e0, e1);
    for (int k = 0; k < g.nt; ++k) {
        if (k % K == 0) {
            const int s = k / K;
            cudaMemcpy2DAsync((char *)ck + (size_t)2 * s * fbytes, ck_pitch, (char *)ring + (size_t)(k % 3) * fbytes,
                              ring_pitch, fbytes, nres, cudaMemcpyDeviceToDevice, st);
            cudaMemcpy2DAsync((char *)ck + (size_t)(2 * s + 1) * fbytes, ck_pitch,
                              (char *)ring + (size_t)((k + 1) % 3) * fbytes, ring_pitch, fbytes, nres,
                              cudaMemcpyDeviceToDevice, st);
        }
        const StepArgs sa = ring_step(k, k, -1, c.d->rik[k]);
        launches += step(false, c.maps, g, b, nres, sa, st, c.variant);
    }
    close_span(e0, e1, g.nt);

    // adjoint, segment by segment from the last
    cudaMemset2DAsync(ring2, ring_pitch, 0, 2 * fbytes, nres, st);
    Batch ba = b;
    ba.ring = ring2;
    b.store = 1;
    profile_span(e0, e1);
    for (int s = nseg - 1; s >= 0; --s) {
        const int k0 = s * K, k1 = std::min(k0 + K, g.nt), snap0 = k0 / g.nti;
        cudaMemcpy2DAsync((char *)ring + (size_t)(k0 % 3) * fbytes, ring_pitch, (char *)ck + (size_t)2 * s * fbytes,
                          ck_pitch, fbytes, nres, cudaMemcpyDeviceToDevice, st);
        cudaMemcpy2DAsync((char *)ring + (size_t)((k0 + 1) % 3) * fbytes, ring_pitch,
                          (char *)ck + (size_t)(2 * s + 1) * fbytes, ck_pitch, fbytes, nres,
                          cudaMemcpyDeviceToDevice, st);
        for (int k = k0; k < k1; ++k) {  // recompute the segment's forward steps, storing them
            const StepArgs sa = ring_step(k, k, (k % g.nti) == 0 ? k / g.nti - snap0 : -1, c.d->rik[k]);
            launches += step(false, c.maps, g, b, nres, sa, st, c.variant);
        }
        for (int it = k1 - 1; it >= k0; --it) {  // the segment's adjoint steps
            const StepArgs sa = ring_step(g.nt - 1 - it, it, (it % g.nti) == 0 ? it / g.nti - snap0 : -1, 0.0f);
            launches += step(true, c.maps2, g, ba, nres, sa, st, c.variant);
        }
    }
    close_span(e0, e1, 2LL * g.nt);
    return launches;
}

// overlap: the previous operation on `st` is a step kernel, and this one may
// be launched programmatically (it waits for that step before reading
// anything the step writes).
template <int H>
static void launch_adjoint_exact(const Call &c, const ExactBatch &x, int nres, int k, int lev1, float rik,
                                 cudaStream_t st, bool overlap)
{
    const Geom &g = c.d->g;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(g.tiles_x * g.tiles_z), nres);
    cfg.blockDim = dim3(kAdjThreads);
    cfg.dynamicSmemBytes = AdjShape<H>::kSmem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = overlap ? 1 : 0;
    if (cudaLaunchKernelEx(&cfg, k_adjoint_tile<H>, c.maps3.p1, c.maps2.p1, g, x, k, lev1, rik) != cudaSuccess)
        t_enqueue_error = GB_FWI2D_ECUDA;
}

static void adjoint_exact(const Call &c, const ExactBatch &x, int nres, int k, int lev1, float rik, cudaStream_t st,
                          bool overlap)
{
    switch (c.d->g.Lc - 1) {
    case 3: launch_adjoint_exact<3>(c, x, nres, k, lev1, rik, st, overlap); break;
    case 4: launch_adjoint_exact<4>(c, x, nres, k, lev1, rik, st, overlap); break;
    case 5: launch_adjoint_exact<5>(c, x, nres, k, lev1, rik, st, overlap); break;
    default: launch_adjoint_exact<6>(c, x, nres, k, lev1, rik, st, overlap); break;
    }
}

// Exact gradient.  Per wave: the forward pass (data, and either every level
// into `store` or a (p0, p1) pair per segment), then the segments from the
// last: restore the pair, recompute the segment's levels into `store`, and
// run its adjoint steps k = i1 .. i0+1, each of which needs lambda^{k+1},
// lambda^{k+2} and the levels P^{k-1}, P^{k-2}.  The forward steps write
// their levels straight into `store` (a ring of K+2 levels that does not
// wrap), so no level is copied.
static long long enqueue_exact(const Call &c, cudaStream_t st)
{
    const Geom &g = c.d->g;
    const Layout &L = c.L;
    long long launches = 0;
    float *vdt = (float *)(c.work + L.vdt);
    float *ring = (float *)(c.work + L.ring);
    float *ck = (float *)(c.work + L.ckpt);
    float *store = (float *)(c.work + L.store);
    float *lam = (float *)(c.work + L.lam);
    float *nu = (float *)(c.work + L.nu);
    float *gpad = (float *)(c.work + L.gpad);
    float *syn = c.syn ? c.syn : (float *)(c.work + L.syn);
    double *part = (double *)(c.work + L.part);
    int *status = (int *)(c.work + L.status);
    const long long ninst = (long long)c.nsamples * g.ns;
    const int K = L.ckpt_k, nseg = L.ckpt_nseg, levels = K + 2;
    const size_t fbytes = sizeof(float) * g.fstride;
    const size_t ring_pitch = 3 * fbytes, store_pitch = (size_t)levels * fbytes, ck_pitch = 2 * (size_t)nseg * fbytes;

    k_prepare<<<grid_for((long long)c.nsamples * g.fstride, 256), 256, 0, st>>>(g, c.vel, vdt, c.nsamples);
    float *abeta = (float *)(c.work + L.abeta);
    int4 *cells = (int4 *)(c.work + L.cells);
    float *taps = (float *)(c.work + L.taps);
    k_exact_tables<<<grid_for((long long)c.nsamples * g.fstride, 256), 256, 0, st>>>(g, c.tab.coef, vdt, c.nsamples,
                                                                                   cells, abeta, taps);
    launches += 2;
    if (c.clear_status) cudaMemsetAsync(status, 0, sizeof(int), st);
    cudaMemsetAsync(gpad, 0, fbytes * ninst, st);

    Batch b{};
    b.vdt = vdt;
    b.vel = c.vel;
    b.obs = c.obs;
    b.syn = syn;
    b.ring = ring;
    b.levels = 3;
    b.tm_slot0 = 0;
    b.coef = c.tab.coef;
    b.blend_fp32 = c.d->blend_fp32 ? 1 : 0;
    b.status = status;
    Batch bs = b;  // forward steps writing into the store
    bs.ring = store;
    bs.levels = levels;
    ExactBatch x;
    x.vdt = vdt;
    x.abeta = abeta;
    x.cells = cells;
    x.obs = c.obs;
    x.syn = syn;
    x.lam = lam;
    x.nu = nu;
    x.store = store;
    x.store_pitch = (long long)levels * g.fstride;
    x.store_levels = levels;
    x.gpad = gpad;
    x.coef = c.tab.coef;
    x.status = status;
    x.taps = taps;
    x.rdx2 = 1.0f / (g.dx * g.dx);
    x.rdz2 = 1.0f / (g.dz * g.dz);
    x.dtdx = g.dt / g.dx;

    // prev_step: the last operation enqueued on st is a step kernel, so the
    // next may be launched programmatically.
    bool prev_step = false;
    // step it with p0 = store level l, p1 = l + 1, p2 = l + 2
    auto fwd_store = [&](int it, int l, int nres) {
        StepArgs sa = ring_step(it, it, -1, c.d->rik[it]);
        sa.l0 = l;
        sa.l1 = l + 1;
        sa.l2 = l + 2;
        launches += step(false, c.maps2, g, bs, nres, sa, st, c.variant, prev_step);
        prev_step = true;
    };
    const int wave = (c.flags & GB_FWI2D_PLAIN) ? 1 : L.resident;
    for (long long i0 = 0; i0 < ninst; i0 += wave) {
        const int nres = (int)std::min<long long>(wave, ninst - i0);
        b.inst0 = bs.inst0 = x.inst0 = (int)i0;
        prev_step = false;
        if (nseg == 1) {  // every level in the store: P^-1 = P^0 = 0, step it writes level it + 2
            cudaMemset2DAsync(store, store_pitch, 0, 2 * fbytes, nres, st);
            for (int it = 0; it < g.nt; ++it) fwd_store(it, it, nres);
        } else {
            cudaMemset2DAsync(ring, ring_pitch, 0, 2 * fbytes, nres, st);
            for (int it = 0; it < g.nt; ++it) {
                if (it % K == 0) {
                    const int s = it / K;  // the step's (p0, p1) = (P^{it-1}, P^it)
                    for (int h = 0; h < 2; ++h)
                        cudaMemcpy2DAsync((char *)ck + (size_t)(2 * s + h) * fbytes, ck_pitch,
                                          (char *)ring + (size_t)((it + h) % 3) * fbytes, ring_pitch, fbytes, nres,
                                          cudaMemcpyDeviceToDevice, st);
                    prev_step = false;
                }
                launches += step(false, c.maps, g, b, nres, ring_step(it, it, -1, c.d->rik[it]), st, c.variant,
                                 prev_step);
                prev_step = true;
            }
        }
        // lambda^{nt+1} = lambda^{nt+2} = 0, and nu with them (its pad columns stay zero)
        cudaMemsetAsync(lam, 0, 3 * fbytes * (size_t)nres, st);
        cudaMemsetAsync(nu, 0, 3 * fbytes * (size_t)nres, st);
        prev_step = false;
        for (int s = nseg - 1; s >= 0; --s) {
            const int i0s = s * K, i1s = std::min(i0s + K, g.nt);
            if (nseg > 1) {
                // the pair (P^{i0s-1}, P^{i0s}) into store levels 0, 1; recompute the segment
                cudaMemcpy2DAsync(store, store_pitch, (char *)ck + (size_t)(2 * s) * fbytes, ck_pitch, 2 * fbytes,
                                  nres, cudaMemcpyDeviceToDevice, st);
                prev_step = false;
                for (int it = i0s; it <= i1s - 2; ++it) fwd_store(it, it - i0s, nres);
            }
            for (int k = i1s; k >= i0s + 1; --k) {
                adjoint_exact(c, x, nres, k, k - i0s, c.d->rik[k - 1], st, prev_step);
                prev_step = true;
                ++launches;
            }
        }
    }
    if (c.grad) {
        k_reduce_exact<<<grid_for((long long)c.nsamples * g.nz * g.nx, 256), 256, 0, st>>>(g, gpad, c.grad,
                                                                                           c.nsamples);
        ++launches;
    }
    if (c.misfit) {
        k_misfit_partial<<<dim3(kMisfitBlocks, c.nsamples), 256, 0, st>>>(syn, c.obs, (long long)g.ns * g.nt * g.nr,
                                                                          part);
        k_misfit_final<<<(c.nsamples + 127) / 128, 128, 0, st>>>(part, c.misfit, c.nsamples);
        launches += 2;
    }
    return launches;
}

// Enqueue the whole batch on `st`; returns the number of kernel launches.
static long long enqueue(const Call &c, cudaStream_t st)
{
    if ((c.flags & GB_FWI2D_EXACT_GRADIENT) && !(c.flags & GB_FWI2D_FORWARD_ONLY)) return enqueue_exact(c, st);
    const Geom &g = c.d->g;
    long long launches = 0;
    float *vdt = (float *)(c.work + c.L.vdt);
    float *ring = (float *)(c.work + c.L.ring);
    float *gacc = (float *)(c.work + c.L.gacc);
    float *syn = c.syn ? c.syn : (float *)(c.work + c.L.syn);
    double *part = (double *)(c.work + c.L.part);
    int *status = (int *)(c.work + c.L.status);
    const bool imaging = (c.flags & GB_FWI2D_IMAGING) != 0;
    const bool plain = (c.flags & GB_FWI2D_PLAIN) != 0;
    const bool fwd_only = (c.flags & GB_FWI2D_FORWARD_ONLY) != 0;
    const long long ninst = (long long)c.nsamples * g.ns;

    k_prepare<<<grid_for((long long)c.nsamples * g.fstride, 256), 256, 0, st>>>(g, c.vel, vdt,
                                                                                c.nsamples);
    ++launches;
    if (c.clear_status) cudaMemsetAsync(status, 0, sizeof(int), st);
    if (!fwd_only) cudaMemsetAsync(gacc, 0, sizeof(float) * g.pstride * ninst, st);

    Batch b;
    b.vdt = vdt;
    b.vel = c.vel;
    b.obs = c.obs;
    b.syn = syn;
    b.ring = ring;
    b.psave = (float *)(c.work + c.L.psave);
    b.gacc = gacc;
    b.coef = c.tab.coef;
    b.blend_fp32 = c.d->blend_fp32 ? 1 : 0;
    b.imaging = imaging ? 1 : 0;
    b.store = fwd_only ? 0 : 1;
    b.status = status;
    b.spec = (double *)(c.work + c.L.spec);
    b.spec_resident = c.L.resident;
    b.kk = c.kk;
    b.slot0 = 0;
    b.levels = 3;
    b.tm_slot0 = 0;
    const Maps &maps = c.maps;

    const int wave = plain ? 1 : c.L.resident;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    const SideStream *side = (g.pstd || wave < kSplitMinResident || c.single_stream)
                                 ? nullptr
                                 : side_stream(cs == cudaStreamCaptureStatusNone);
    const bool ckpt = (c.flags & GB_FWI2D_CHECKPOINT) && !fwd_only;
    for (long long i0 = 0; i0 < ninst && ckpt; i0 += wave) {
        const int nres = (int)std::min<long long>(wave, ninst - i0);
        b.inst0 = (int)i0;
        const long long wi = i0 / wave;
        Call cw = c;
        cw.variant = c.wave_variant(wi);
        if (wi < (long long)c.trials.size()) cudaEventRecord(c.trial_ev[wi].first, st);
        launches += enqueue_checkpointed(cw, b, nres, st);
        if (wi < (long long)c.trials.size()) cudaEventRecord(c.trial_ev[wi].second, st);
    }
    for (long long i0 = 0; i0 < ninst && !ckpt; i0 += wave) {
        const int nres = (int)std::min<long long>(wave, ninst - i0);
        b.inst0 = (int)i0;
        const long long wi = i0 / wave;
        const int variant = c.wave_variant(wi);
        if (wi < (long long)c.trials.size()) cudaEventRecord(c.trial_ev[wi].first, st);
        for (int pass = 0; pass < (fwd_only ? 1 : 2); ++pass) {
            const bool adj = pass == 1;
            // p0 and p1 of step 0 start at zero (wavefield_initialization).
            cudaMemset2DAsync(ring, sizeof(float) * 3 * g.fstride, 0, sizeof(float) * 2 * g.fstride,
                              nres, st);
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (c.profile && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess)
                cudaEventRecord(e0, st);
            const bool split = side && nres >= kSplitMinResident;
            const int nlo = split ? nres / 2 : nres;
            Batch bhi = b;
            bhi.slot0 = nlo;
            if (split) {  // fork: the second half's chain on the side stream
                cudaEventRecord(side->fork, st);
                cudaStreamWaitEvent(side->s, side->fork, 0);
            }
            for (int k = 0; k < g.nt; ++k) {
                const int it = adj ? g.nt - 1 - k : k;
                const StepArgs sa = ring_step(k, it, (it % g.nti) == 0 ? it / g.nti : -1, adj ? 0.0f : c.d->rik[it]);
                launches += step(adj, maps, g, b, nlo, sa, st, variant, k > 0);
                if (split) launches += step(adj, maps, g, bhi, nres - nlo, sa, side->s, variant, k > 0);
            }
            if (split) {  // join
                cudaEventRecord(side->join, side->s);
                cudaStreamWaitEvent(st, side->join, 0);
            }
            if (e1) {
                cudaEventRecord(e1, st);
                t_profile.spans.emplace_back(e0, e1);
                t_profile.launches += g.nt;
            }
        }
        if (wi < (long long)c.trials.size()) cudaEventRecord(c.trial_ev[wi].second, st);
    }
    if (c.grad && !fwd_only) {
        k_reduce_grad<<<grid_for((long long)c.nsamples * g.nz * g.nx, 256), 256, 0, st>>>(
            g, gacc, c.vel, c.grad, c.nsamples, imaging ? 1 : 0);
        ++launches;
    }
    if (c.misfit) {
        k_misfit_partial<<<dim3(kMisfitBlocks, c.nsamples), 256, 0, st>>>(
            syn, c.obs, (long long)g.ns * g.nt * g.nr, part);
        k_misfit_final<<<(c.nsamples + 127) / 128, 128, 0, st>>>(part, c.misfit, c.nsamples);
        launches += 2;
    }
    return launches;
}

// ---------------------------------------------------------------------------
// Fused launches over instances of different geometry (gb_fwi2d_run_instances)
//
// The solves of every instance of a chunk (one FD order, full storage) are
// packed into waves that fill the caller's workspace; the solves of a wave,
// whatever their instance, advance together: one k_step_multi launch per time
// step.  Instances are sorted by nt, longest first, so the solves of a wave
// have similar time axes and the ones still running at step k are a prefix of
// the wave -- a launch's grid is that prefix's blocks.  This replaces one
// launch per instance, wave and step, whose fixed cost dominates small grids
// (the reference's per-sample loop, geopvi/forward/fwi2d/posterior.py:112-149,
// runs the instances one after another).
//
// Each solve computes exactly what it computes in gb_fwi2d_batch -- the same
// tile code, its own ring, stored field and gradient slot -- so the results
// are those of the instances run alone, bit for bit.
// ---------------------------------------------------------------------------
struct FusedInst {
    const gb_fwi2d_instance *x;
    Derived d;
    DeviceTables tab;
    long long ninst;                   // its solves: nsamples * ns
    size_t vdt, gacc, syn, part, rik;  // buffers kept for the whole chunk (byte offsets in work)
    size_t keep;                       // their bytes
    size_t solve_bytes;                // ring and stored field of one resident solve
};

struct FusedPiece {
    int inst;             // index of its instance in the chunk
    int inst0, r;         // solves [inst0, inst0 + r) of that instance
    size_t ring, psave;   // byte offsets in work
};

// The pieces of a wave that share a grid (grid_key), at most kMaxPieces:
// one k_step_multi launch per step.
struct FusedLaunch {
    std::vector<int> pieces;  // indices into the wave's pieces, longest nt first
    int maxnt = 0;
    MultiArgs args;           // the launch's parameter (the first half of its solves when split)
    bool split = false;       // the second half runs as its own launch on the side stream
    MultiArgs args_hi;
};

// Split a launch's table at solve `at` (among its tm_slot0 order): solves
// below stay, the rest move to `hi` -- a piece that straddles `at` is cut in
// two.  Each half's first blocks start again at 0.
static void split_args(MultiArgs &lo, MultiArgs &hi, int at, const Geom &g, bool fwd_only)
{
    MultiArgs all = lo;
    hi = all;
    lo.npieces = hi.npieces = 0;
    int blo = 0, bhi = 0;
    const int tiles = g.tiles_x * g.tiles_z;
    for (int q = 0; q < all.npieces; ++q) {
        const PieceArgs &pc = all.piece[q];
        const int s0 = pc.tm_slot0, s1 = pc.tm_slot0 + pc.nres;
        if (s0 < at) {
            PieceArgs a = pc;
            a.nres = std::min(s1, at) - s0;
            a.first_block = blo;
            lo.first[lo.npieces] = blo;
            lo.piece[lo.npieces++] = a;
            blo += a.nres * tiles;
        }
        if (s1 > at) {
            PieceArgs b = pc;
            const int cut = std::max(0, at - s0);  // solves of this piece in the first half
            b.inst0 += cut;
            b.tm_slot0 += cut;
            b.nres -= cut;
            b.ring += (size_t)3 * g.fstride * cut;
            if (!fwd_only) b.psave += (size_t)pc.nt_save * g.pstride * cut;
            b.first_block = bhi;
            hi.first[hi.npieces] = bhi;
            hi.piece[hi.npieces++] = b;
            bhi += b.nres * tiles;
        }
    }
    lo.first[lo.npieces] = blo;
    hi.first[hi.npieces] = bhi;
}

struct FusedWave {
    std::vector<FusedPiece> pieces;
    std::vector<FusedLaunch> launches;
    int maxnt = 0;
};

// Every Geom field but the acquisition and the time axis, which the pieces
// of one k_step_multi launch share (the kernel reads them from its parameter).
static std::vector<long long> grid_key(const Geom &g)
{
    std::vector<long long> k = {g.ntx, g.ntz, g.pitch, g.xoff, g.nx, g.nz, g.ipitch, g.ioff, g.pml, g.Lc, g.pml0,
                                g.tiles_x, g.tiles_z, g.fast_dx, g.fast_dz, g.pstd, g.fstride, g.pstride};
    uint32_t u;
    for (float f : {g.dx, g.dz, g.dt, g.rdx, g.rdz, g.fd[0], g.fd[1], g.fd[2], g.fd[3], g.fd[4], g.fd[5], g.fd[6],
                    g.fd[7]}) {
        std::memcpy(&u, &f, 4);
        k.push_back(u);
    }
    return k;
}

static void fused_inst_sizes(FusedInst &f, bool fwd_only)
{
    const Geom &g = f.d.g;
    f.keep = align256(sizeof(float) * g.fstride * f.x->nsamples);
    if (!fwd_only) f.keep += align256(sizeof(float) * g.pstride * f.ninst);
    if (!f.x->syn) f.keep += align256(sizeof(float) * (size_t)f.ninst * g.nt * g.nr);
    f.keep += align256(sizeof(double) * kMisfitBlocks * f.x->nsamples);
    f.keep += align256(sizeof(float) * g.nt);
    f.solve_bytes = sizeof(float) * g.fstride * 3 + (fwd_only ? 0 : sizeof(float) * g.pstride * g.nt_save);
}

static size_t piece_bytes(const FusedInst &f, int r, bool fwd_only)
{
    const Geom &g = f.d.g;
    return align256(sizeof(float) * g.fstride * 3 * r) +
           (fwd_only ? 0 : align256(sizeof(float) * g.pstride * g.nt_save * r));
}

constexpr size_t kFusedHeader = 256;  // the call's status word

// The smallest workspace that runs the instance fused: the status word, its
// kept buffers and one resident solve.
static size_t fused_min_bytes(const FusedInst &f, bool fwd_only)
{
    return kFusedHeader + f.keep + piece_bytes(f, 1, fwd_only);
}

// Flags under which gb_fwi2d_run_instances fuses instances (full storage,
// the reference's gradient, launches enqueued directly; the fused kernel has
// one variant, so a forced variant does not apply to it).
static bool fusable(unsigned flags)
{
    return !(flags & (GB_FWI2D_PLAIN | GB_FWI2D_CHECKPOINT | GB_FWI2D_EXACT_GRADIENT | GB_FWI2D_GRAPH));
}

static bool fused_instance(const gb_fwi2d_instance &x, unsigned flags, FusedInst &f)
{
    f.x = &x;
    if (derive(x.params, f.d)) return false;
    f.ninst = (long long)x.nsamples * f.d.g.ns;
    fused_inst_sizes(f, (flags & GB_FWI2D_FORWARD_ONLY) != 0);
    return true;
}

// Pack the chunk's solves into waves of at most `avail` bytes (and at most
// max_resident solves when that is positive), in the chunk's order.
// Returns false when some solve does not fit at all.
static bool plan_waves(const std::vector<FusedInst> &fi, size_t avail, int max_resident, bool fwd_only,
                       std::vector<FusedWave> &waves)
{
    waves.clear();
    waves.emplace_back();
    size_t used = 0;
    long long res = 0;
    for (int i = 0; i < (int)fi.size(); ++i) {
        long long s0 = 0;
        while (s0 < fi[i].ninst) {
            const long long left = fi[i].ninst - s0;
            long long r = used < avail ? (long long)((avail - used) / fi[i].solve_bytes) : 0;
            r = std::min(r, left);
            if (max_resident > 0) r = std::min(r, (long long)max_resident - res);
            while (r > 0 && used + piece_bytes(fi[i], (int)r, fwd_only) > avail) --r;
            if (r <= 0) {
                if (waves.back().pieces.empty()) return false;
                waves.emplace_back();
                used = 0;
                res = 0;
                continue;
            }
            FusedPiece pc;
            pc.inst = i;
            pc.inst0 = (int)s0;
            pc.r = (int)r;
            pc.ring = pc.psave = 0;  // placed when the chunk runs
            used += piece_bytes(fi[i], (int)r, fwd_only);
            res += r;
            waves.back().pieces.push_back(pc);
            waves.back().maxnt = std::max(waves.back().maxnt, fi[i].d.g.nt);
            s0 += r;
        }
    }
    return true;
}

// How gb_fwi2d_run_instances runs a fusable call: chunks (one FD order each;
// instances of one grid together, longest nt first; an instance joins a chunk
// while the status word, the kept buffers and one solve of the widest
// instance still fit), each with its waves; pseudo-spectral instances run
// alone, after the chunks.
struct FusedPlan {
    std::vector<std::vector<FusedInst>> chunks;
    std::vector<std::vector<FusedWave>> waves;
    std::vector<int> alone;
};

static int plan_instances(const gb_fwi2d_instance *inst, int n, unsigned flags, int max_resident,
                          size_t work_bytes, FusedPlan &plan)
{
    const bool fwd_only = (flags & GB_FWI2D_FORWARD_ONLY) != 0;
    std::vector<FusedInst> all(n);
    for (int i = 0; i < n; ++i)
        if (!fused_instance(inst[i], flags, all[i])) return GB_FWI2D_EINVAL;
    std::vector<int> order;
    for (int i = 0; i < n; ++i) order.push_back(i);
    std::vector<std::vector<long long>> keys(n);
    for (int i = 0; i < n; ++i) keys[i] = grid_key(all[i].d.g);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const Geom &ga = all[a].d.g, &gb = all[b].d.g;
        if (ga.Lc != gb.Lc) return ga.Lc < gb.Lc;
        if (keys[a] != keys[b]) return keys[a] < keys[b];
        return ga.nt > gb.nt;
    });
    std::vector<FusedInst> chunk;
    size_t kept = 0, widest = 0;
    auto close = [&]() -> int {
        if (chunk.empty()) return GB_FWI2D_OK;
        std::vector<FusedWave> waves;
        if (kFusedHeader + kept >= work_bytes ||
            !plan_waves(chunk, work_bytes - kFusedHeader - kept, max_resident, fwd_only, waves))
            return GB_FWI2D_ENOMEM;
        plan.chunks.push_back(chunk);
        plan.waves.push_back(waves);
        chunk.clear();
        kept = widest = 0;
        return GB_FWI2D_OK;
    };
    for (int idx : order) {
        FusedInst &f = all[idx];
        if (f.d.g.pstd) {  // the pseudo-spectral step is not fused
            plan.alone.push_back(idx);
            continue;
        }
        const size_t w = std::max(widest, piece_bytes(f, 1, fwd_only));
        if (!chunk.empty() && (chunk[0].d.g.Lc != f.d.g.Lc || kFusedHeader + kept + f.keep + w > work_bytes)) {
            const int st = close();
            if (st) return st;
        }
        chunk.push_back(f);
        kept += f.keep;
        widest = std::max(widest, piece_bytes(f, 1, fwd_only));
    }
    return close();
}

template <int H, int NP>
static void launch_multi_np(bool adj, const MultiArgs &full, int nact, int k, cudaStream_t st, bool overlap)
{
    constexpr StepVariant v = kStepVariants[0];
    MultiArgsN<NP> a;
    a.tm = full.tm;
    a.gc = full.gc;
    a.coef = full.coef;
    a.status = full.status;
    a.blend_fp32 = full.blend_fp32;
    a.imaging = full.imaging;
    a.store = full.store;
    a.npieces = full.npieces;
    for (int q = 0; q <= NP; ++q) a.first[q] = full.first[q];
    for (int q = 0; q < NP; ++q) a.piece[q] = full.piece[q];
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)full.first[nact]);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = TileShape<H>::kSmem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = overlap ? 1 : 0;
    const cudaError_t e =
        adj ? cudaLaunchKernelEx(&cfg, k_step_multi<H, true, v.rows, v.min_blocks, NP>, a, nact, k)
            : cudaLaunchKernelEx(&cfg, k_step_multi<H, false, v.rows, v.min_blocks, NP>, a, nact, k);
    if (e != cudaSuccess) t_enqueue_error = GB_FWI2D_ECUDA;
}

// The smallest parameter table that holds the launch's pieces.
template <int H>
static void launch_multi(bool adj, const MultiArgs &args, int nact, int k, cudaStream_t st, bool overlap)
{
    static_assert(kMaxPieces == 16, "tables of 1, 4 and 16 pieces");
    if (args.npieces <= 1)
        launch_multi_np<H, 1>(adj, args, nact, k, st, overlap);
    else if (args.npieces <= 4)
        launch_multi_np<H, 4>(adj, args, nact, k, st, overlap);
    else
        launch_multi_np<H, 16>(adj, args, nact, k, st, overlap);
}

// Enqueue one chunk (instances of one FD order, grouped by grid, longest nt
// first) laid out as: the status word, the instances' kept buffers (Ricker
// tables first: they are copied from the host in one transfer), then one wave
// region reused by every wave.  Returns the number of kernels enqueued, or -1
// when a tensor map or copy failed.
static long long run_fused_chunk(std::vector<FusedInst> &fi, std::vector<FusedWave> &waves, unsigned flags,
                                 char *work, cudaStream_t st, bool clear_status)
{
    const bool imaging = (flags & GB_FWI2D_IMAGING) != 0;
    const bool fwd_only = (flags & GB_FWI2D_FORWARD_ONLY) != 0;
    const bool profile = (flags & GB_FWI2D_PROFILE) != 0;
    const int H = fi[0].d.g.Lc - 1;
    int *status = (int *)work;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cs);
    const SideStream *side = side_stream(cs == cudaStreamCaptureStatusNone);
    size_t off = kFusedHeader;
    for (auto &f : fi) {
        f.rik = off;
        off = align256(off + sizeof(float) * f.d.g.nt);
    }
    const size_t tables_end = off;
    for (auto &f : fi) {  // the other kept buffers
        const Geom &g = f.d.g;
        f.vdt = off;  off = align256(off + sizeof(float) * g.fstride * f.x->nsamples);
        f.gacc = off; if (!fwd_only) off = align256(off + sizeof(float) * g.pstride * f.ninst);
        f.syn = off;  if (!f.x->syn) off = align256(off + sizeof(float) * (size_t)f.ninst * g.nt * g.nr);
        f.part = off; off = align256(off + sizeof(double) * kMisfitBlocks * f.x->nsamples);
    }
    const size_t wave_base = off;
    std::vector<char> host(tables_end - kFusedHeader, 0);
    for (auto &f : fi) std::memcpy(host.data() + (f.rik - kFusedHeader), f.d.rik.data(), sizeof(float) * f.d.g.nt);

    for (auto &w : waves) {
        // Launches: the wave's pieces by grid, in order of first appearance,
        // at most kMaxPieces - 1 each (a split cuts one piece in two).
        w.launches.clear();
        std::vector<std::vector<long long>> keys;
        for (int j = 0; j < (int)w.pieces.size(); ++j) {
            const auto key = grid_key(fi[w.pieces[j].inst].d.g);
            size_t c = 0;
            while (c < keys.size() && !(keys[c] == key && (int)w.launches[c].pieces.size() < kMaxPieces - 1)) ++c;
            if (c == keys.size()) {
                keys.push_back(key);
                w.launches.emplace_back();
            }
            w.launches[c].pieces.push_back(j);
            w.launches[c].maxnt = std::max(w.launches[c].maxnt, fi[w.pieces[j].inst].d.g.nt);
        }
        // Per launch: its pieces' rings back to back (one tensor map covers
        // them), then their stored fields; within the planned bytes, which
        // counted each ring rounded up on its own.
        size_t used = 0;
        for (auto &l : w.launches) {
            const FusedInst &f0 = fi[w.pieces[l.pieces[0]].inst];
            const Geom &g0 = f0.d.g;
            MultiArgs &A = l.args;
            std::memset(&A, 0, sizeof A);
            const size_t base = wave_base + used;
            int slots = 0, blocks = 0;
            for (size_t q = 0; q < l.pieces.size(); ++q) {
                FusedPiece &pc = w.pieces[l.pieces[q]];
                const FusedInst &f = fi[pc.inst];
                const Geom &g = f.d.g;
                pc.ring = base + sizeof(float) * g.fstride * 3 * slots;
                PieceArgs &P = A.piece[q];
                P.vdt = (const float *)(work + f.vdt);
                P.vel = f.x->vel;
                P.obs = f.x->obs;
                P.rik = (const float *)(work + f.rik);
                P.syn = f.x->syn ? f.x->syn : (float *)(work + f.syn);
                P.ring = (float *)(work + pc.ring);
                P.gacc = (float *)(work + f.gacc);
                P.s_iz = g.s_iz;
                P.r_iz = g.r_iz;
                P.r_ix0 = g.r_ix0;
                P.dr = g.dr;
                P.nr = g.nr;
                P.ds = g.ds;
                P.s_ix0 = g.s_ix0;
                P.ns = g.ns;
                P.nt = g.nt;
                P.nti = g.nti;
                P.nt_save = g.nt_save;
                P.inst0 = pc.inst0;
                P.tm_slot0 = slots;
                P.nres = pc.r;
                P.first_block = blocks;
                A.first[q] = blocks;
                slots += pc.r;
                blocks += pc.r * g.tiles_x * g.tiles_z;
            }
            A.first[l.pieces.size()] = blocks;
            used = align256(used + sizeof(float) * g0.fstride * 3 * slots);
            for (size_t q = 0; q < l.pieces.size(); ++q) {
                FusedPiece &pc = w.pieces[l.pieces[q]];
                const Geom &g = fi[pc.inst].d.g;
                pc.psave = wave_base + used;
                A.piece[q].psave = (float *)(work + pc.psave);
                if (!fwd_only) used = align256(used + sizeof(float) * g.pstride * g.nt_save * pc.r);
            }
            if (!make_map(A.tm, work + base, g0, 3LL * slots, kBoxX, kTileZ + 2 * (g0.Lc - 1))) return -1;
            A.gc = g0;
            A.coef = f0.tab.coef;
            A.status = status;
            A.blend_fp32 = f0.d.blend_fp32 ? 1 : 0;
            A.imaging = imaging ? 1 : 0;
            A.store = fwd_only ? 0 : 1;
            A.npieces = (int)l.pieces.size();
            // Launches of at least kSplitMinResident solves run as two halves on
            // two streams, so the tail of one half's step overlaps the other's.
            l.split = side != nullptr && slots >= kSplitMinResident;
            if (l.split) split_args(A, l.args_hi, slots / 2, g0, fwd_only);
        }
    }
    // From pageable memory: the copy has taken the host image when it returns.
    if (!host.empty() &&
        cudaMemcpyAsync(work + kFusedHeader, host.data(), host.size(), cudaMemcpyHostToDevice, st) != cudaSuccess)
        return -1;
    long long launches = 0;
    if (clear_status) cudaMemsetAsync(status, 0, sizeof(int), st);
    for (const auto &f : fi) {
        const Geom &g = f.d.g;
        k_prepare<<<grid_for((long long)f.x->nsamples * g.fstride, 256), 256, 0, st>>>(g, f.x->vel,
                                                                                     (float *)(work + f.vdt),
                                                                                     f.x->nsamples);
        ++launches;
        if (!fwd_only) cudaMemsetAsync(work + f.gacc, 0, sizeof(float) * g.pstride * f.ninst, st);
    }
    for (const auto &w : waves) {
        for (int pass = 0; pass < (fwd_only ? 1 : 2); ++pass) {
            const bool adj = pass == 1;
            for (const auto &pc : w.pieces) {  // p0 and p1 of step 0 start at zero (wavefield_initialization)
                const Geom &g = fi[pc.inst].d.g;
                cudaMemset2DAsync(work + pc.ring, sizeof(float) * 3 * g.fstride, 0, sizeof(float) * 2 * g.fstride,
                                  pc.r, st);
            }
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (profile && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess)
                cudaEventRecord(e0, st);
            bool forked = false;
            for (const auto &l : w.launches) forked |= l.split;
            if (forked) {  // fork: the second halves' chain on the side stream
                cudaEventRecord(side->fork, st);
                cudaStreamWaitEvent(side->s, side->fork, 0);
            }
            std::vector<int> nact, nact_hi;
            for (const auto &l : w.launches) {
                nact.push_back(l.args.npieces);
                nact_hi.push_back(l.split ? l.args_hi.npieces : 0);
            }
            // Each step waits for the launch before it on its stream; the first
            // of a pass on each stream follows the rings' reset and launches normally.
            bool started = false, started_hi = false;
            auto launch = [&](const MultiArgs &a, int &na, int k, cudaStream_t s, bool &on) {
                while (na > 0 && a.piece[na - 1].nt <= k) --na;  // the pieces still running: a prefix
                if (na == 0) return;
                switch (H) {
                case 3: launch_multi<3>(adj, a, na, k, s, on); break;
                case 4: launch_multi<4>(adj, a, na, k, s, on); break;
                case 5: launch_multi<5>(adj, a, na, k, s, on); break;
                default: launch_multi<6>(adj, a, na, k, s, on); break;
                }
                on = true;
                ++launches;
            };
            for (int k = 0; k < w.maxnt; ++k) {
                for (size_t li = 0; li < w.launches.size(); ++li) {
                    const FusedLaunch &l = w.launches[li];
                    launch(l.args, nact[li], k, st, started);
                    if (l.split) launch(l.args_hi, nact_hi[li], k, side->s, started_hi);
                }
            }
            if (forked) {  // join
                cudaEventRecord(side->join, side->s);
                cudaStreamWaitEvent(st, side->join, 0);
            }
            if (e1) {
                cudaEventRecord(e1, st);
                t_profile.spans.emplace_back(e0, e1);
                for (const auto &l : w.launches) t_profile.launches += l.maxnt * (l.split ? 2 : 1);
            }
        }
    }
    for (const auto &f : fi) {
        const Geom &g = f.d.g;
        if (f.x->grad && !fwd_only) {
            k_reduce_grad<<<grid_for((long long)f.x->nsamples * g.nz * g.nx, 256), 256, 0, st>>>(
                g, (float *)(work + f.gacc), f.x->vel, f.x->grad, f.x->nsamples, imaging ? 1 : 0);
            ++launches;
        }
        if (f.x->misfit) {
            const float *syn = f.x->syn ? f.x->syn : (const float *)(work + f.syn);
            k_misfit_partial<<<dim3(kMisfitBlocks, f.x->nsamples), 256, 0, st>>>(
                syn, f.x->obs, (long long)g.ns * g.nt * g.nr, (double *)(work + f.part));
            k_misfit_final<<<(f.x->nsamples + 127) / 128, 128, 0, st>>>((double *)(work + f.part), f.x->misfit,
                                                                         f.x->nsamples);
            launches += 2;
        }
    }
    return launches;
}

static std::vector<long long> graph_key(const Call &c, int dev)
{
    const Geom &g = c.d->g;
    std::vector<long long> k;
    k.push_back(dev);
    const int *gi = (const int *)&g;
    for (size_t i = 0; i < sizeof(Geom) / sizeof(int); ++i) k.push_back(gi[i]);
    k.push_back(c.nsamples);
    k.push_back((long long)(uintptr_t)c.vel);
    k.push_back((long long)(uintptr_t)c.obs);
    k.push_back((long long)(uintptr_t)c.syn);
    k.push_back((long long)(uintptr_t)c.grad);
    k.push_back((long long)(uintptr_t)c.misfit);
    k.push_back((long long)(uintptr_t)c.work);
    k.push_back(c.flags);
    k.push_back(c.L.resident);
    k.push_back(c.variant);
    // The Ricker table depends on f0, which Geom does not hold.
    for (float r : {c.d->rik.empty() ? 0.0f : c.d->rik[0], c.d->rik.size() > 1 ? c.d->rik[1] : 0.0f}) {
        int bits;
        std::memcpy(&bits, &r, sizeof bits);
        k.push_back(bits);
    }
    return k;
}

// ---------------------------------------------------------------------------
// Variant tuner.  Every k_step variant computes the same values bit for bit,
// so the caller's own work serves as trials: while a (geometry, batch size,
// wave size, mode) has untried variants, each wave of a call runs one of them
// between two events (a six-wave batch tries all four in its first call);
// later calls read the finished timings -- polled, never waited for -- and
// run the fastest.  Calls with trials run eagerly; graph capture starts once
// the choice is made.
// ---------------------------------------------------------------------------
struct TuneState {
    bool measured[kNumStepVariants] = {};
    bool inflight[kNumStepVariants] = {};
    float ms[kNumStepVariants] = {};
    cudaEvent_t e0[kNumStepVariants] = {}, e1[kNumStepVariants] = {};
    int best = 0;  // fastest measured (the default until one is measured)
    bool done = false;
};
static std::mutex g_tune_mutex;
static std::map<std::vector<long long>, TuneState> g_tune;

static std::vector<long long> tune_key(const Geom &g, int nsamples, int resident, unsigned flags, int dev)
{
    std::vector<long long> k{dev, nsamples, resident,
                             (long long)(flags & (GB_FWI2D_IMAGING | GB_FWI2D_PLAIN | GB_FWI2D_CHECKPOINT |
                                                  GB_FWI2D_FORWARD_ONLY | GB_FWI2D_EXACT_GRADIENT))};
    const int *gi = (const int *)&g;
    for (size_t i = 0; i < sizeof(Geom) / sizeof(int); ++i) k.push_back(gi[i]);
    return k;
}

// Read the trials whose events have completed (g_tune_mutex held).
static void tune_harvest(TuneState &t)
{
    bool all = true;
    for (int v = 0; v < kNumStepVariants; ++v) {
        if (t.inflight[v] && cudaEventQuery(t.e1[v]) == cudaSuccess) {
            float ms = 0.0f;
            // An unreadable timing counts as measured and never wins.
            t.ms[v] = cudaEventElapsedTime(&ms, t.e0[v], t.e1[v]) == cudaSuccess ? ms : 3.4e38f;
            t.measured[v] = true;
            t.inflight[v] = false;
        }
        all = all && t.measured[v];
    }
    int best = -1;
    for (int v = 0; v < kNumStepVariants; ++v)
        if (t.measured[v] && (best < 0 || t.ms[v] < t.ms[best])) best = v;
    if (best >= 0) t.best = best;
    t.done = all;
}

// The calling batch's plan: trial variants for its first waves (with their
// events) and the variant for the rest.
static void tune_plan(const std::vector<long long> &key, long long nwaves, Call &c)
{
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    TuneState &t = g_tune[key];
    tune_harvest(t);
    c.variant = t.best;
    if (t.done) return;
    for (int v = 0; v < kNumStepVariants && (long long)c.trials.size() < nwaves; ++v) {
        if (t.measured[v] || t.inflight[v]) continue;
        if (!t.e0[v] && (cudaEventCreate(&t.e0[v]) != cudaSuccess || cudaEventCreate(&t.e1[v]) != cudaSuccess)) {
            t.measured[v] = true;  // no events: leave this variant out
            t.ms[v] = 3.4e38f;
            continue;
        }
        t.inflight[v] = true;
        c.trials.push_back(v);
        c.trial_ev.emplace_back(t.e0[v], t.e1[v]);
    }
}

static int run_graph(const Call &c, cudaStream_t st, long long &launches)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GB_FWI2D_ECUDA;
    std::vector<long long> key = graph_key(c, dev);
    {
        std::lock_guard<std::mutex> lk(g_mutex);
        auto it = g_graphs.find(key);
        if (it != g_graphs.end()) {
            launches = it->second.launches;
            return cudaGraphLaunch(it->second.exec, st) == cudaSuccess ? GB_FWI2D_OK
                                                                      : GB_FWI2D_ECUDA;
        }
    }
    side_stream(true);  // created outside the capture
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return GB_FWI2D_ECUDA;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaStreamDestroy(cap);
        return GB_FWI2D_ECUDA;
    }
    long long n = enqueue(c, cap);
    cudaError_t e = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return GB_FWI2D_ECUDA;
    GraphEntry ge;
    e = cudaGraphInstantiate(&ge.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return GB_FWI2D_ECUDA;
    ge.launches = n;
    {
        std::lock_guard<std::mutex> lk(g_mutex);
        g_graphs[key] = ge;
    }
    launches = n;
    return cudaGraphLaunch(ge.exec, st) == cudaSuccess ? GB_FWI2D_OK : GB_FWI2D_ECUDA;
}

}  // namespace gbfwi

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace gbfwi;

namespace {

bool read_line_value(FILE *fp, const char *fmt, void *dst)
{
    char line[256];
    if (!std::fgets(line, sizeof line, fp)) return false;
    if (std::fscanf(fp, "\n") < 0) { /* only whitespace skipped */ }
    if (std::fscanf(fp, fmt, dst) != 1) return false;
    if (std::fscanf(fp, "\n") < 0) { /* end of file after the last value */ }
    return true;
}

}  // namespace

extern "C" {

const char *gb_fwi2d_version(void) { return "geopvi_gb300 fwi2d 0.1 (sm_103a)"; }

int gb_fwi2d_read_params(const char *path, gb_fwi2d_params *out)
{
    if (!path || !out) return GB_FWI2D_EINVAL;
    FILE *fp = std::fopen(path, "r");
    if (!fp) return GB_FWI2D_ENOENT;
    gb_fwi2d_params p;
    int *ints[] = {&p.nx, &p.nz, &p.pml0, &p.Lc, &p.laplace_solver, &p.ns, &p.nt, &p.ds,
                   &p.ns0, &p.depths, &p.depthr, &p.nr, &p.dr, &p.nr0, &p.nt_interval};
    float *floats[] = {&p.dx, &p.dz, &p.dt, &p.f0};
    bool ok = true;
    for (int *v : ints) ok = ok && read_line_value(fp, "%d", v);
    for (float *v : floats) ok = ok && read_line_value(fp, "%f", v);
    std::fclose(fp);
    if (!ok) return GB_FWI2D_EINVAL;
    *out = p;
    return GB_FWI2D_OK;
}

int gb_fwi2d_validate(const gb_fwi2d_params *p)
{
    if (!p) return GB_FWI2D_EINVAL;
    return validate(*p);
}

size_t gb_fwi2d_workspace_bytes(const gb_fwi2d_params *p, int nsamples, int max_resident,
                                unsigned flags)
{
    (void)flags;
    if (!p || nsamples <= 0) return 0;
    Derived d;
    if (derive(*p, d)) return 0;
    return plan_layout(d.g, nsamples, max_resident, true, (flags & GB_FWI2D_FORWARD_ONLY) != 0,
                       (flags & GB_FWI2D_CHECKPOINT) != 0, (flags & GB_FWI2D_EXACT_GRADIENT) != 0)
        .total;
}

// gb_fwi2d_batch's body.  clear_status false keeps the flags that earlier
// work on the same workspace left in its status word (the instances of
// gb_fwi2d_run_instances after the first).
static int batch_impl(const gb_fwi2d_params *p, int nsamples, const float *vel, const float *obs, float *syn,
                      float *grad, double *misfit, unsigned flags, int max_resident, void *work,
                      size_t work_bytes, void *stream, bool clear_status)
{
    t_last_launches = 0;
    if (!p || nsamples <= 0 || !vel || !obs || !work) return GB_FWI2D_EINVAL;
    cudaGetLastError();  // an earlier, unrelated error must not fail this call
    Derived d;
    int st = derive(*p, d);
    if (st) return st;
    const bool ckpt = (flags & GB_FWI2D_CHECKPOINT) != 0;
    const bool exact = (flags & GB_FWI2D_EXACT_GRADIENT) != 0;
    if (exact && (flags & GB_FWI2D_IMAGING)) return GB_FWI2D_EINVAL;
    if (exact && d.g.pstd && !(flags & GB_FWI2D_FORWARD_ONLY)) return GB_FWI2D_ENOTSUP;  // transposes the FD stencil
    Layout L = plan_layout(d.g, nsamples, max_resident, true, (flags & GB_FWI2D_FORWARD_ONLY) != 0, ckpt, exact);
    if (work_bytes < L.total) return GB_FWI2D_ENOMEM;
    Call c;
    c.d = &d;
    c.L = L;
    c.nsamples = nsamples;
    c.vel = vel;
    c.obs = obs;
    c.syn = syn;
    c.grad = grad;
    c.misfit = misfit;
    c.flags = flags;
    c.work = (char *)work;
    c.profile = (flags & GB_FWI2D_PROFILE) && !(flags & GB_FWI2D_GRAPH);
    c.clear_status = clear_status;
    // The step kernel's tensor maps (the pseudo-spectral step reads the ring directly).
    if (!d.g.pstd && !make_maps(c.maps, d.g, (float *)(c.work + L.ring), L.resident))
        return GB_FWI2D_ECUDA;
    if (ckpt && !exact && !d.g.pstd && !(flags & GB_FWI2D_FORWARD_ONLY) &&
        !make_maps(c.maps2, d.g, (float *)(c.work + L.ring2), L.resident))
        return GB_FWI2D_ECUDA;
    if (exact && !d.g.pstd && !(flags & GB_FWI2D_FORWARD_ONLY)) {  // the store and nu, as the step's tiles
        const int box_z = kTileZ + 2 * (d.g.Lc - 1);
        if (!make_map(c.maps2.p1, (float *)(c.work + L.store), d.g, (long long)(L.ckpt_k + 2) * L.resident, kBoxX,
                      box_z) ||
            !make_map(c.maps3.p1, (float *)(c.work + L.nu), d.g, 3LL * L.resident, kBoxX, box_z))
            return GB_FWI2D_ECUDA;
    }
    st = get_tables(d, c.tab);
    if (st) return st;
    if (d.g.pstd) {
        // The transform plans exist before anything is enqueued: full waves,
        // the last partial wave and single solves (GB_FWI2D_PLAIN).
        st = kk_table(d, &c.kk);
        if (st) return st;
        const long long ninst = (long long)nsamples * d.g.ns;
        cufftHandle h;
        for (long long batch : {(long long)L.resident, ninst % L.resident, 1LL})
            for (bool inverse : {false, true})
                if (batch > 0 && (st = fft_plan(d.g, (int)batch, inverse, &h)) != GB_FWI2D_OK) return st;
    }
    cudaStream_t s = (cudaStream_t)stream;
    long long launches = 0;
    t_enqueue_error = 0;
    // Kernel variant: forced by the flags, or planned by the tuner (FD mode;
    // the exact gradient runs the tuned or default variant without trials).
    const unsigned forced = (flags >> GB_FWI2D_VARIANT_SHIFT) & 0xFu;
    if (forced > (unsigned)kNumStepVariants) return GB_FWI2D_EINVAL;
    if (forced) {
        c.variant = (int)forced - 1;
    } else if (!d.g.pstd) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return GB_FWI2D_ECUDA;
        const long long wave = (flags & GB_FWI2D_PLAIN) ? 1 : L.resident;
        const long long ninst = (long long)nsamples * d.g.ns;
        tune_plan(tune_key(d.g, nsamples, L.resident, flags, dev), exact ? 0 : (ninst + wave - 1) / wave, c);
    }
    if ((flags & GB_FWI2D_GRAPH) && !d.g.pstd && c.trials.empty()) {  // transforms and trials run eagerly
        st = run_graph(c, s, launches);
    } else {
        launches = enqueue(c, s);
        st = cudaGetLastError() == cudaSuccess ? GB_FWI2D_OK : GB_FWI2D_ECUDA;
    }
    if (st == GB_FWI2D_OK && t_enqueue_error) st = t_enqueue_error;
    t_last_launches = launches;
    return st;
}

int gb_fwi2d_batch(const gb_fwi2d_params *p, int nsamples, const float *vel, const float *obs,
                   float *syn, float *grad, double *misfit, unsigned flags, int max_resident,
                   void *work, size_t work_bytes, void *stream)
{
    return batch_impl(p, nsamples, vel, obs, syn, grad, misfit, flags, max_resident, work, work_bytes, stream,
                      true);
}

size_t gb_fwi2d_instances_workspace_bytes(const gb_fwi2d_instance *inst, int n, int max_resident,
                                          unsigned flags)
{
    if (!inst || n <= 0) return 0;
    size_t most = 0;
    for (int i = 0; i < n; ++i) {
        size_t b = gb_fwi2d_workspace_bytes(&inst[i].params, inst[i].nsamples, max_resident, flags);
        if (b == 0) return 0;
        FusedInst f;
        if (fusable(flags) && inst[i].params.laplace_solver != 1 && fused_instance(inst[i], flags, f))
            b = fused_min_bytes(f, (flags & GB_FWI2D_FORWARD_ONLY) != 0);
        most = std::max(most, b);
    }
    return most;
}

int gb_fwi2d_run_instances(const gb_fwi2d_instance *inst, int n, unsigned flags, int max_resident,
                           void *work, size_t work_bytes, void *stream)
{
    t_last_launches = 0;
    if (!inst || n <= 0 || !work) return GB_FWI2D_EINVAL;
    const bool exact = (flags & GB_FWI2D_EXACT_GRADIENT) != 0;
    if (exact && (flags & GB_FWI2D_IMAGING)) return GB_FWI2D_EINVAL;
    if (((flags >> GB_FWI2D_VARIANT_SHIFT) & 0xFu) > (unsigned)kNumStepVariants) return GB_FWI2D_EINVAL;
    for (int i = 0; i < n; ++i) {  // everything checked before anything is enqueued
        const gb_fwi2d_instance &x = inst[i];
        if (x.nsamples <= 0 || !x.vel || !x.obs || (!(flags & GB_FWI2D_FORWARD_ONLY) && !x.grad))
            return GB_FWI2D_EINVAL;
        const int st = gb_fwi2d_validate(&x.params);
        if (st) return st;
        if (exact && x.params.laplace_solver == 1 && !(flags & GB_FWI2D_FORWARD_ONLY)) return GB_FWI2D_ENOTSUP;
        if (gb_fwi2d_instances_workspace_bytes(&x, 1, max_resident, flags) > work_bytes) return GB_FWI2D_ENOMEM;
    }
    long long launches = 0;
    bool first_run = true;  // the status word is cleared once per call
    // One instance through the gb_fwi2d_batch path (waves as its workspace allows).
    auto alone = [&](const gb_fwi2d_instance &x) -> int {
        const int st = batch_impl(&x.params, x.nsamples, x.vel, x.obs, x.syn, x.grad, x.misfit, flags,
                                  max_resident, work, work_bytes, stream, first_run);
        first_run = false;
        launches += t_last_launches;
        return st;
    };
    if (!fusable(flags)) {
        for (int i = 0; i < n; ++i) {
            const int st = alone(inst[i]);
            if (st) {
                t_last_launches = launches;
                return st;
            }
        }
        t_last_launches = launches;
        return GB_FWI2D_OK;
    }
    FusedPlan plan;
    int st = plan_instances(inst, n, flags, max_resident, work_bytes, plan);
    if (st) return st;  // not reached: every instance was checked to fit alone
    cudaGetLastError();
    cudaStream_t s = (cudaStream_t)stream;
    // A fused chunk copies its Ricker tables from pageable host memory, which
    // a stream capture does not allow: refuse before anything is enqueued.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (!plan.chunks.empty() && (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone))
        return GB_FWI2D_ENOTSUP;
    for (size_t c = 0; c < plan.chunks.size() && !st; ++c) {
        for (auto &f : plan.chunks[c]) {
            st = get_tables(f.d, f.tab);
            if (st) break;
        }
        if (st) break;
        t_enqueue_error = 0;
        const long long k = run_fused_chunk(plan.chunks[c], plan.waves[c], flags, (char *)work, s, first_run);
        first_run = false;
        if (k < 0) {
            st = GB_FWI2D_ECUDA;
            break;
        }
        launches += k;
        st = cudaGetLastError() != cudaSuccess ? GB_FWI2D_ECUDA : t_enqueue_error;
    }
    for (size_t i = 0; i < plan.alone.size() && !st; ++i) st = alone(inst[plan.alone[i]]);
    t_last_launches = launches;
    return st;
}

int gb_fwi2d_instances_waves(const gb_fwi2d_instance *inst, int n, unsigned flags, int max_resident,
                             size_t work_bytes)
{
    if (!inst || n <= 0 || !fusable(flags)) return GB_FWI2D_EINVAL;
    for (int i = 0; i < n; ++i) {
        if (inst[i].nsamples <= 0) return GB_FWI2D_EINVAL;
        const int st = gb_fwi2d_validate(&inst[i].params);
        if (st) return st;
        if (gb_fwi2d_instances_workspace_bytes(&inst[i], 1, max_resident, flags) > work_bytes)
            return GB_FWI2D_ENOMEM;
    }
    FusedPlan plan;
    const int st = plan_instances(inst, n, flags, max_resident, work_bytes, plan);
    if (st) return st;
    int waves = 0;
    for (const auto &w : plan.waves) waves += (int)w.size();
    return waves;
}

long long gb_fwi2d_last_launch_count(void) { return t_last_launches; }

int gb_fwi2d_tuned_variant(const gb_fwi2d_params *p, int nsamples, int max_resident, unsigned flags)
{
    if (!p || nsamples <= 0) return GB_FWI2D_EINVAL;
    Derived d;
    int st = derive(*p, d);
    if (st) return st;
    const Layout L = plan_layout(d.g, nsamples, max_resident, true, (flags & GB_FWI2D_FORWARD_ONLY) != 0,
                                 (flags & GB_FWI2D_CHECKPOINT) != 0, (flags & GB_FWI2D_EXACT_GRADIENT) != 0);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GB_FWI2D_ECUDA;
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_tune.find(tune_key(d.g, nsamples, L.resident, flags, dev));
    if (it == g_tune.end()) return -1;
    tune_harvest(it->second);
    return it->second.done ? it->second.best : -1;
}

static int static_scratch(void **out);

int gb_fwi2d_status(const void *work, void *stream)
{
    if (!work) {  // the allocation-free entry point's workspace on the current device
        void *base = nullptr;
        const int st = static_scratch(&base);
        if (st) return st;
        work = base;
    }
    int h = 0;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemcpyAsync(&h, work, sizeof h, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GB_FWI2D_ECUDA;
    return h == kStatusOk ? GB_FWI2D_OK : GB_FWI2D_ETIMEOUT;
}

double gb_fwi2d_profile_step_ms(long long *launches)
{
    if (launches) *launches = t_profile.launches;
    if (t_profile.spans.empty()) return -1.0;
    double total = 0.0;
    for (auto &e : t_profile.spans) {
        float ms = 0.0f;
        if (cudaEventSynchronize(e.second) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e.first, e.second) != cudaSuccess) {
            t_profile.reset();
            return -1.0;
        }
        total += ms;
    }
    t_profile.reset();
    return total;
}

int gb_fwi2d_side_stream_count(void)
{
    std::lock_guard<std::mutex> lk(g_side_mutex);
    return (int)g_side.size();
}

void gb_fwi2d_release_caches(void)
{
    const CufftApi *api = g_fft_plans.empty() ? nullptr : cufft_api();
    std::lock_guard<std::mutex> lk(g_mutex);
    for (auto &kv : g_graphs) cudaGraphExecDestroy(kv.second.exec);
    g_graphs.clear();
    for (auto &kv : g_tables) {
        cudaFree(kv.second.coef);
    }
    g_tables.clear();
    if (api)
        for (auto &kv : g_fft_plans) api->destroy(kv.second);
    g_fft_plans.clear();
    for (auto &kv : g_kk_tables) cudaFree(kv.second);
    g_kk_tables.clear();
    std::lock_guard<std::mutex> lk2(g_side_mutex);
    for (auto &kv : g_side) {
        cudaEventDestroy(kv.second.fork);
        cudaEventDestroy(kv.second.join);
        cudaStreamDestroy(kv.second.s);
    }
    g_side.clear();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Host-buffer drop-ins for fwi_2D / forward_2D
// ---------------------------------------------------------------------------
namespace {

struct HostCallBuffers {
    int dev = -1;
    size_t bytes = 0;
    char *base = nullptr;
    cudaStream_t stream = nullptr;
};
std::mutex g_host_mutex;
HostCallBuffers g_host;

int host_run(const char *input_file, const float *vel_inner, float *record_syn,
             const float *record_obs, float *grad, int run_fwi, int verbose, bool with_grad)
{
    if (!input_file || !vel_inner || !record_syn) return GB_FWI2D_EINVAL;
    gb_fwi2d_params p;
    int st = gb_fwi2d_read_params(input_file, &p);
    if (st) {
        if (verbose) std::printf("Cannot open %s!\n", input_file);
        return st;
    }
    Derived d;
    st = derive(p, d);
    if (st) return st;
    const size_t ncell = (size_t)p.nx * p.nz;
    for (size_t i = 0; i < ncell; ++i)
        if (std::isnan(vel_inner[i])) return GB_FWI2D_ENAN;
    const size_t ndata = (size_t)p.ns * p.nt * p.nr;
    Layout L = plan_layout(d.g, 1, 0, true, !with_grad);
    const size_t o_vel = 0, o_obs = align256(sizeof(float) * ncell);
    const size_t o_syn = align256(o_obs + sizeof(float) * ndata);
    const size_t o_grad = align256(o_syn + sizeof(float) * ndata);
    const size_t o_work = align256(o_grad + sizeof(float) * ncell);
    const size_t need = o_work + L.total;

    std::lock_guard<std::mutex> lk(g_host_mutex);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GB_FWI2D_ECUDA;
    if (g_host.dev != dev || g_host.bytes < need) {
        if (g_host.base) cudaFree(g_host.base);
        if (g_host.stream && g_host.dev != dev) {
            cudaStreamDestroy(g_host.stream);
            g_host.stream = nullptr;
        }
        g_host.base = nullptr;
        g_host.bytes = 0;
        if (cudaMalloc(&g_host.base, need) != cudaSuccess) return GB_FWI2D_ENOMEM;
        g_host.bytes = need;
        g_host.dev = dev;
    }
    if (!g_host.stream && cudaStreamCreateWithFlags(&g_host.stream, cudaStreamNonBlocking) != cudaSuccess)
        return GB_FWI2D_ECUDA;
    cudaStream_t s = g_host.stream;
    char *b = g_host.base;
    if (verbose) {
        std::printf("ntx=%d, ntz=%d\n", d.g.ntx, d.g.ntz);
        std::printf("nx=%d,  nz=%d,  nt=%d,  ns=%d\n", p.nx, p.nz, p.nt, p.ns);
    }
    cudaMemcpyAsync(b + o_vel, vel_inner, sizeof(float) * ncell, cudaMemcpyHostToDevice, s);
    if (with_grad)
        cudaMemcpyAsync(b + o_obs, record_obs, sizeof(float) * ndata, cudaMemcpyHostToDevice, s);
    else
        cudaMemsetAsync(b + o_obs, 0, sizeof(float) * ndata, s);
    unsigned flags = (run_fwi ? 0u : GB_FWI2D_IMAGING) | (with_grad ? 0u : GB_FWI2D_FORWARD_ONLY);
    st = gb_fwi2d_batch(&p, 1, (const float *)(b + o_vel), (const float *)(b + o_obs),
                        (float *)(b + o_syn), with_grad ? (float *)(b + o_grad) : nullptr, nullptr,
                        flags, 0, b + o_work, L.total, s);
    if (st) return st;
    std::vector<float> g(with_grad ? ncell : 0);
    cudaMemcpyAsync(record_syn, b + o_syn, sizeof(float) * ndata, cudaMemcpyDeviceToHost, s);
    if (with_grad) cudaMemcpyAsync(g.data(), b + o_grad, sizeof(float) * ncell, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return GB_FWI2D_ECUDA;
    st = gb_fwi2d_status(b + o_work, s);
    if (st) return st;
    if (with_grad)
        for (size_t i = 0; i < ncell; ++i) grad[i] += g[i];  // the reference accumulates into grad
    return GB_FWI2D_OK;
}

}  // namespace

extern "C" {

int fwi_2D(char input_file[200], float *vel_inner, float *record_syn, float *record_obs,
           float *grad, int run_fwi, int verbose)
{
    if (!record_obs || !grad) return GB_FWI2D_EINVAL;
    return host_run(input_file, vel_inner, record_syn, record_obs, grad, run_fwi, verbose, true);
}

int forward_2D(char input_file[200], float *vel_inner, float *record_syn, int run_fwi, int verbose)
{
    (void)run_fwi;  // forward_2D stores the field either way; only the data are returned
    return host_run(input_file, vel_inner, record_syn, nullptr, nullptr, 1, verbose, false);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free entry point (gb_fwi2d_batch_noalloc)
//
// For callers that cannot allocate device memory -- code that must not call
// cudaMalloc or a pool allocator while it runs (a host whose device memory is
// owned by another runtime or a fixed pool, a latency-critical loop where an
// allocation would synchronize the device), or a plain C caller through an
// FFI that has no way to hand over a workspace.  The workspace then lives in
// a fixed array that this library reserves on every GPU that loads it, for
// the life of the process.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_static_scratch[GB_FWI2D_STATIC_SCRATCH_BYTES];

static constexpr int kMaxDevices = 64;
static std::mutex g_static_mutex;
static void *g_static_addr[kMaxDevices] = {};

// Device address of the static scratch array on the current device.  In host
// code the array's name is only a host-side stand-in, so the address is
// looked up once per device (with that device current) and cached.
static int static_scratch(void **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GB_FWI2D_ECUDA;
    std::lock_guard<std::mutex> lk(g_static_mutex);
    if (!g_static_addr[dev]) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_static_scratch) != cudaSuccess || !ptr) return GB_FWI2D_ECUDA;
        g_static_addr[dev] = ptr;
    }
    *out = g_static_addr[dev];
    return GB_FWI2D_OK;
}

extern "C" int gb_fwi2d_batch_noalloc(const gb_fwi2d_params *p, int nsamples, const float *vel, const float *obs,
                                      float *syn, float *grad, double *misfit, unsigned flags, void *stream)
{
    t_last_launches = 0;
    if (!p || nsamples <= 0 || !vel || !obs) return GB_FWI2D_EINVAL;
    if (flags & ~(GB_FWI2D_IMAGING | GB_FWI2D_FORWARD_ONLY | GB_FWI2D_PLAIN | GB_FWI2D_CHECKPOINT))
        return GB_FWI2D_EINVAL;
    cudaGetLastError();  // an earlier, unrelated error must not fail this call
    Derived d;
    int st = derive(*p, d);
    if (st) return st;
    if (d.g.pstd) return GB_FWI2D_ENOTSUP;  // the transform library allocates its plans
    const bool fwd_only = (flags & GB_FWI2D_FORWARD_ONLY) != 0;
    const bool ckpt = (flags & GB_FWI2D_CHECKPOINT) && !fwd_only;
    // The workspace starts at the array's base (its status word first, where
    // gb_fwi2d_status(NULL, ...) reads it); the weight table sits at the end.
    const size_t coef_bytes = align256(sizeof(BlendCoef) * d.coef.size());
    const size_t cap = GB_FWI2D_STATIC_SCRATCH_BYTES - coef_bytes;
    // Largest resident count whose workspace fits beside the weight table.
    const long long ninst = (long long)nsamples * d.g.ns;
    auto layout = [&](long long resident) {
        return plan_layout(d.g, nsamples, (int)resident, syn == nullptr, fwd_only, ckpt);
    };
    if (layout(1).total > cap) return GB_FWI2D_E2BIG;
    long long lo = 1, hi = ninst;
    while (lo < hi) {
        const long long mid = (lo + hi + 1) / 2;
        if (layout(mid).total <= cap)
            lo = mid;
        else
            hi = mid - 1;
    }
    const Layout L = layout(lo);
    void *base = nullptr;
    st = static_scratch(&base);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    Call c;
    c.d = &d;
    c.L = L;
    c.nsamples = nsamples;
    c.vel = vel;
    c.obs = obs;
    c.syn = syn;
    c.grad = grad;
    c.misfit = misfit;
    c.flags = flags;
    c.work = (char *)base;
    c.profile = false;
    c.single_stream = true;  // the two-halves schedule would create a side stream and events
    c.tab.coef = (BlendCoef *)((char *)base + cap);
    if (!make_maps(c.maps, d.g, (float *)(c.work + L.ring), L.resident)) return GB_FWI2D_ECUDA;
    if (ckpt && !make_maps(c.maps2, d.g, (float *)(c.work + L.ring2), L.resident)) return GB_FWI2D_ECUDA;
    t_enqueue_error = 0;
    // The weight table is built on the device: no host-to-device copy.
    k_blend_coef<<<1, 32, 0, s>>>(d.g.pml0, c.tab.coef);
    const long long launches = 1 + enqueue(c, s);
    t_last_launches = launches;
    st = cudaGetLastError() == cudaSuccess ? GB_FWI2D_OK : GB_FWI2D_ECUDA;
    if (st == GB_FWI2D_OK && t_enqueue_error) st = t_enqueue_error;
    return st;
}

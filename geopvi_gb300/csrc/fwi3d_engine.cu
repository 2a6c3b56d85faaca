// fwi3d_engine.cu -- the 3-D acoustic FWI engine (C ABI in include/geopvi_fwi3d.h).
//
// The scheme is the 2-D reference solver's algorithm
// (geopvi/forward/fwi2d/fdtd2D_modelling.c) on three axes, stated step by
// step in the header; the CPU oracle (oracle/fwi3d_oracle.cpp) follows the
// same FP32 operations, and this engine reproduces them bit for bit.
//
// Per time step of a wave of resident (sample, shot) solves:
//   k3_step    stencil + the six absorbing passes for every padded cell, and
//              the stored d2p/dt2 (forward) or the imaging term (adjoint) of
//              the interior cells;
//   k3_io_fwd  source injection (and the stored value at the source cell),
//              then receiver sampling;  k3_io_adj  residual injection at the
//              receivers (and their imaging terms).
// k3_step: one thread per (x, y) column of a 32 x 8 tile, marching along z
// through a chunk of planes with the z stencil window in registers; x and y
// neighbours come through the read-only cache.  Fields are [z][y][x] with a
// row pitch of 32 floats.  The adjoint runs the same operator backwards; its
// forward field is stored whole or, with GB_FWI3D_CHECKPOINT, as
// ceil(sqrt(nt))-step segments recomputed from checkpoints.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/geopvi_fwi2d.h"
#include "../../include/geopvi_fwi3d.h"
#include "fd_weights.cuh"

namespace gbfwi3 {

using gbfwi::fd_weight;

// Build-time tuning knobs: planes per z chunk (each chunk reloads 2H planes
// of the z window) and resident blocks per SM the registers are capped for.
#ifndef GB_FWI3D_ZCHUNK
#define GB_FWI3D_ZCHUNK 32
#endif
#ifndef GB_FWI3D_MIN_BLOCKS
#define GB_FWI3D_MIN_BLOCKS 4
#endif
#ifndef GB_FWI3D_ZUNROLL
#define GB_FWI3D_ZUNROLL 1
#endif
#define GB_FWI3D_PRAGMA(x) _Pragma(#x)
#define GB_FWI3D_UNROLL(n) GB_FWI3D_PRAGMA(unroll n)

constexpr int kBX = 32;     // tile columns (x), one warp
constexpr int kBY = 8;      // tile rows (y)
constexpr int kZC = GB_FWI3D_ZCHUNK;  // planes per z chunk
constexpr int kMisfitBlocks = 64;

struct Geom3 {
    int ntx, nty, ntz, pitch;  // padded grid, x pitch in floats
    int nx, ny, nz;
    int L, pml, pml0;
    int nt, nti, ns, nr, nu;   // nu: distinct receiver cells
    int tiles_x, tiles_y, chunks_z;
    long long sz;              // z stride (pitch * nty)
    long long fstride;         // floats per padded field
    long long istride;         // floats per interior field (nx * ny * nz)
    float id[3], id2[3];       // 1/d and 1/d^2 for x, y, z
    float idt2, dt;
};

struct Batch3 {
    const float *vdt;   // [nsamples][fstride]  v*dt, padded
    const float *vel;   // [nsamples][ny*nx*nz] model order
    const float *obs;   // [ns][nt][nr]
    float *syn;         // [ninst][nt][nr]
    float *ring;        // [resident][3][fstride]
    float *snap;        // [resident][nsnap][istride]
    float *G;           // [ninst][istride]
    const float *w, *omw;       // [pml0]
    const int *src;             // [ns][3]
    const int *rec;             // [nr][3]
    const int *uoff;            // [nu + 1] receivers of each distinct cell, in receiver order
    const int *uidx;            // [nr]
    int nsnap;                  // stored steps per resident solve
    int inst0;                  // first solve of the wave
};

__device__ __forceinline__ float fmaf_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// ((a * dt) * dt * v) * v: the injection factor of forward_IO / backward_IO.
__device__ __forceinline__ float inject(float a, float dt, float v)
{
    return __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(a, dt), dt), v), v);
}

// One absorbing blend along a face normal: p1a..p1c = p1 at 0, 1, 2 cells
// inward, p0a..p0e = p0 at 0..4 cells inward; s = v dt / d.
__device__ __forceinline__ float blend(float q, float s, float w, float omw, float p1a, float p1b, float p1c,
                                       float p0a, float p0b, float p0c, float p0d, float p0e)
{
    const float t11 = __fmul_rn(__fmul_rn(__fsub_rn(2.0f, s), __fsub_rn(1.0f, s)), 0.5f);
    const float t12 = __fmul_rn(s, __fsub_rn(2.0f, s));
    const float t13 = __fmul_rn(__fmul_rn(s, __fsub_rn(s, 1.0f)), 0.5f);
    const float k0 = __fmul_rn(2.0f, t11), k1 = __fmul_rn(2.0f, t12), k2 = __fmul_rn(2.0f, t13);
    const float k3 = __fmul_rn(t11, t11), k4 = __fmul_rn(k0, t12);
    const float k5 = fmaf_rn(t12, t12, __fmul_rn(k0, t13));
    const float k6 = __fmul_rn(k1, t13), k7 = __fmul_rn(t13, t13);
    float e = __fmul_rn(k0, p1a);
    e = fmaf_rn(k1, p1b, e);
    e = fmaf_rn(k2, p1c, e);
    e = fmaf_rn(-k3, p0a, e);
    e = fmaf_rn(-k4, p0b, e);
    e = fmaf_rn(-k5, p0c, e);
    e = fmaf_rn(-k6, p0d, e);
    e = fmaf_rn(-k7, p0e, e);
    return fmaf_rn(w, e, __fmul_rn(omw, q));
}

// One time step of every resident solve.  blockIdx.x = tile (x fastest, then
// y, then z chunk), blockIdx.y = resident slot.  k: step within the pass
// (ring buffers (k, k+1, k+2) mod 3 = p0, p1, p2); snap >= 0: the slot's
// stored-field index written (forward) or read (adjoint) at this step.
template <int H, bool ADJ>
__global__ void __launch_bounds__(kBX *kBY, GB_FWI3D_MIN_BLOCKS) k3_step(const Geom3 g, const Batch3 b, int k, int snap)
{
    const int slot = blockIdx.y;
    int t = blockIdx.x;
    const int tx = t % g.tiles_x;
    t /= g.tiles_x;
    const int ty = t % g.tiles_y;
    const int cz = t / g.tiles_y;
    const int x = tx * kBX + threadIdx.x, y = ty * kBY + threadIdx.y;
    if (x >= g.ntx || y >= g.nty) return;
    const int z0 = cz * kZC, z1 = min(z0 + kZC, g.ntz);
    const int inst = b.inst0 + slot;
    const int sample = inst / g.ns;
    float *ring = b.ring + (long long)slot * 3 * g.fstride;
    const float *__restrict__ p0 = ring + (long long)(k % 3) * g.fstride;
    const float *__restrict__ p1 = ring + (long long)((k + 1) % 3) * g.fstride;
    float *__restrict__ p2 = ring + (long long)((k + 2) % 3) * g.fstride;
    const long long col = (long long)y * g.pitch + x;
    const int L = g.L;
    if (x < L || x >= g.ntx - L || y < L || y >= g.nty - L) {  // rim column: always zero
        for (int z = z0; z < z1; ++z) p2[z * g.sz + col] = 0.0f;
        return;
    }
    const float *vdc = b.vdt + (long long)sample * g.fstride + col;
    const bool xmin = x < g.pml, xmax = x >= g.ntx - g.pml;
    const bool ymin = y < g.pml, ymax = y >= g.nty - g.pml;
    const bool inner_xy = !(xmin || xmax || ymin || ymax);
    float *sv = nullptr, *Gv = nullptr;
    if (snap >= 0 && inner_xy) {
        const long long j0 = (long long)(y - g.pml) * g.nx + (x - g.pml);
        sv = b.snap + ((long long)slot * b.nsnap + snap) * g.istride + j0;
        if (ADJ) Gv = b.G + (long long)inst * g.istride + j0;
    }
    const long long ps = (long long)g.nx * g.ny;  // interior plane stride
    const long long sy = g.pitch;

    float win[2 * H + 1];
#pragma unroll
    for (int m = 0; m < 2 * H; ++m) {
        const int zz = z0 - H + m;
        win[m] = (zz >= 0 && zz < g.ntz) ? __ldg(p1 + zz * g.sz + col) : 0.0f;
    }
    // this plane's window value, p0 and v*dt, loaded one plane ahead
    float wn = z0 + H < g.ntz ? __ldg(p1 + (z0 + H) * g.sz + col) : 0.0f;
    float p0n = __ldg(p0 + z0 * g.sz + col), vdn = __ldg(vdc + z0 * g.sz);
    // adjoint stored step: the stored field and the accumulator, also a plane ahead
    float svn = 0.0f, gvn = 0.0f;
    if (ADJ && sv && z0 >= g.pml && z0 < g.ntz - g.pml) {
        const long long j = (long long)(z0 - g.pml) * ps;
        svn = __ldg(sv + j);
        gvn = Gv[j];
    }
    GB_FWI3D_UNROLL(GB_FWI3D_ZUNROLL)
    for (int z = z0; z < z1; ++z) {
        win[2 * H] = wn;
        const float p0c = p0n, vd = vdn;
        const float svc = svn, gvc = gvn;
        if (z + 1 < z1) {
            const int zn = z + 1 + H;
            wn = zn < g.ntz ? __ldg(p1 + zn * g.sz + col) : 0.0f;
            p0n = __ldg(p0 + (z + 1) * g.sz + col);
            vdn = __ldg(vdc + (z + 1) * g.sz);
            if (ADJ && sv && z + 1 >= g.pml && z + 1 < g.ntz - g.pml) {
                const long long j = (long long)(z + 1 - g.pml) * ps;
                svn = __ldg(sv + j);
                gvn = Gv[j];
            }
        }
        const long long c = z * g.sz + col;
        float q = 0.0f;
        if (z >= L && z < g.ntz - L) {
            const float pc = win[H];
            float lx = __fmul_rn(fd_weight<H>(0), pc), ly = lx, lz = lx;
#pragma unroll
            for (int m = 1; m <= H; ++m) {
                lx = fmaf_rn(fd_weight<H>(m), __fadd_rn(__ldg(p1 + c + m), __ldg(p1 + c - m)), lx);
                ly = fmaf_rn(fd_weight<H>(m), __fadd_rn(__ldg(p1 + c + m * sy), __ldg(p1 + c - m * sy)), ly);
                lz = fmaf_rn(fd_weight<H>(m), __fadd_rn(win[H + m], win[H - m]), lz);
            }
            float tt = __fmul_rn(lz, g.id2[2]);
            tt = fmaf_rn(ly, g.id2[1], tt);
            tt = fmaf_rn(lx, g.id2[0], tt);
            const float u = fmaf_rn(2.0f, pc, -p0c);
            q = fmaf_rn(__fmul_rn(vd, vd), tt, u);
            const bool zmin = z < g.pml, zmax = z >= g.ntz - g.pml;
            if (zmin) {
                const int wi = z - L;
                const long long d = g.sz;
                q = blend(q, __fmul_rn(vd, g.id[2]), b.w[wi], b.omw[wi], pc, win[H + 1], win[H + 2], p0c,
                          __ldg(p0 + c + d), __ldg(p0 + c + 2 * d), __ldg(p0 + c + 3 * d), __ldg(p0 + c + 4 * d));
            }
            if (zmax) {
                const int wi = g.ntz - L - 1 - z;
                const long long d = -g.sz;
                q = blend(q, __fmul_rn(vd, g.id[2]), b.w[wi], b.omw[wi], pc, win[H - 1], win[H - 2], p0c,
                          __ldg(p0 + c + d), __ldg(p0 + c + 2 * d), __ldg(p0 + c + 3 * d), __ldg(p0 + c + 4 * d));
            }
            if (!inner_xy) {
                if (ymin || ymax) {
                    const int wi = ymin ? y - L : g.nty - L - 1 - y;
                    const long long d = ymin ? sy : -sy;
                    q = blend(q, __fmul_rn(vd, g.id[1]), b.w[wi], b.omw[wi], pc, __ldg(p1 + c + d),
                              __ldg(p1 + c + 2 * d), p0c, __ldg(p0 + c + d), __ldg(p0 + c + 2 * d),
                              __ldg(p0 + c + 3 * d), __ldg(p0 + c + 4 * d));
                }
                if (xmin || xmax) {
                    const int wi = xmin ? x - L : g.ntx - L - 1 - x;
                    const long long d = xmin ? 1 : -1;
                    q = blend(q, __fmul_rn(vd, g.id[0]), b.w[wi], b.omw[wi], pc, __ldg(p1 + c + d),
                              __ldg(p1 + c + 2 * d), p0c, __ldg(p0 + c + d), __ldg(p0 + c + 2 * d),
                              __ldg(p0 + c + 3 * d), __ldg(p0 + c + 4 * d));
                }
            }
            if (sv && z >= g.pml && z < g.ntz - g.pml) {
                const long long j = (long long)(z - g.pml) * ps;
                if (!ADJ)
                    sv[j] = __fmul_rn(__fsub_rn(q, u), g.idt2);
                else
                    Gv[j] = fmaf_rn(svc, q, gvc);
            }
        }
        p2[c] = q;
#pragma unroll
        for (int m = 0; m < 2 * H; ++m) win[m] = win[m + 1];
    }
}

__device__ __forceinline__ long long padded_cell(const Geom3 &g, const int *xyz)
{
    return (long long)(xyz[2] + g.pml) * g.sz + (long long)(xyz[1] + g.pml) * g.pitch + (xyz[0] + g.pml);
}

__device__ __forceinline__ long long interior_cell(const Geom3 &g, const int *xyz)
{
    return ((long long)xyz[2] * g.ny + xyz[1]) * g.nx + xyz[0];
}

__device__ __forceinline__ float model_velocity(const Geom3 &g, const float *vel, const int *xyz)
{
    return vel[((long long)xyz[1] * g.nx + xyz[0]) * g.nz + xyz[2]];
}

// Forward IO of step k (time it): source injection at the shot's cell (and
// the stored d2p/dt2 there, which must include it), then the receivers.
__global__ void k3_io_fwd(const Geom3 g, const Batch3 b, int k, int it, float wav, int snap, int record)
{
    const int slot = blockIdx.x;
    const int inst = b.inst0 + slot;
    const int sample = inst / g.ns, shot = inst - sample * g.ns;
    float *ring = b.ring + (long long)slot * 3 * g.fstride;
    const float *p0 = ring + (long long)(k % 3) * g.fstride;
    const float *p1 = ring + (long long)((k + 1) % 3) * g.fstride;
    float *p2 = ring + (long long)((k + 2) % 3) * g.fstride;
    if (threadIdx.x == 0) {
        const int *s = b.src + 3 * shot;
        const long long c = padded_cell(g, s);
        const float v = model_velocity(g, b.vel + (long long)sample * g.istride, s);
        const float q = __fadd_rn(p2[c], inject(wav, g.dt, v));
        p2[c] = q;
        if (snap >= 0) {
            const float u = fmaf_rn(2.0f, p1[c], -p0[c]);
            b.snap[((long long)slot * b.nsnap + snap) * g.istride + interior_cell(g, s)] =
                __fmul_rn(__fsub_rn(q, u), g.idt2);
        }
    }
    if (!record) return;
    __syncthreads();
    float *out = b.syn + ((long long)inst * g.nt + it) * g.nr;
    for (int r = threadIdx.x; r < g.nr; r += blockDim.x) out[r] = p2[padded_cell(g, b.rec + 3 * r)];
}

// Adjoint IO of step k (time it): residual injection (syn - obs, the
// transpose of receiver sampling), receiver by receiver in receiver order per
// cell, with each injection's imaging term.
__global__ void k3_io_adj(const Geom3 g, const Batch3 b, int k, int it, int snap)
{
    const int slot = blockIdx.x;
    const int inst = b.inst0 + slot;
    const int sample = inst / g.ns, shot = inst - sample * g.ns;
    float *p2 = b.ring + (long long)slot * 3 * g.fstride + (long long)((k + 2) % 3) * g.fstride;
    const float *syn = b.syn + ((long long)inst * g.nt + it) * g.nr;
    const float *obs = b.obs + ((long long)shot * g.nt + it) * g.nr;
    for (int u = threadIdx.x; u < g.nu; u += blockDim.x) {
        const int r0 = b.uoff[u], r1 = b.uoff[u + 1];
        const int *xyz = b.rec + 3 * b.uidx[r0];
        const long long c = padded_cell(g, xyz);
        const long long j = interior_cell(g, xyz);
        float q = p2[c];
        float *Gc = b.G + (long long)inst * g.istride + j;
        const float sv = snap >= 0 ? b.snap[((long long)slot * b.nsnap + snap) * g.istride + j] : 0.0f;
        float gacc = snap >= 0 ? *Gc : 0.0f;
        for (int i = r0; i < r1; ++i) {
            const int r = b.uidx[i];
            const float inj = __fsub_rn(syn[r], obs[r]);
            q = __fadd_rn(q, inj);
            if (snap >= 0) gacc = fmaf_rn(sv, inj, gacc);
        }
        p2[c] = q;
        if (snap >= 0) *Gc = gacc;
    }
}

// Padded v*dt per sample (get_velp's edge replication is a clamp).
__global__ void k3_prepare(const Geom3 g, const float *__restrict__ vel, float *__restrict__ vdt, int nsamples)
{
    const long long total = (long long)nsamples * g.fstride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(e / g.fstride);
        const long long r = e - (long long)s * g.fstride;
        const int z = (int)(r / g.sz);
        const long long rz = r - (long long)z * g.sz;
        const int y = (int)(rz / g.pitch), x = (int)(rz - (long long)y * g.pitch);
        float v = 0.0f;
        if (x < g.ntx) {
            const int jx = min(max(x - g.pml, 0), g.nx - 1);
            const int jy = min(max(y - g.pml, 0), g.ny - 1);
            const int jz = min(max(z - g.pml, 0), g.nz - 1);
            v = __fmul_rn(vel[(long long)s * g.istride + ((long long)jy * g.nx + jx) * g.nz + jz], g.dt);
        }
        vdt[e] = v;
    }
}

// grad (model order) = 2 nt_interval dt^2 / v * sum over shots (in shot order,
// FP64): with P^{k+1} = 2P^k - P^{k-1} + v^2 dt^2 (lap P^k + f), dP^{k+1}/dv =
// (2/v)(P^{k+1} - 2P^k + P^{k-1}) = (2/v) dt^2 * (stored d2p/dt2).
__global__ void k3_reduce_grad(const Geom3 g, const float *__restrict__ G, const float *__restrict__ vel,
                               float *__restrict__ grad, int nsamples)
{
    const long long cells = g.istride;
    const long long total = (long long)nsamples * cells;
    const double coef = 2.0 * ((double)g.nti * (double)g.dt * (double)g.dt);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(e / cells);
        const long long m = e - (long long)s * cells;
        const int iz = (int)(m % g.nz);
        const long long r = m / g.nz;
        const int ix = (int)(r % g.nx), iy = (int)(r / g.nx);
        const long long j = ((long long)iz * g.ny + iy) * g.nx + ix;
        double acc = 0.0;
        for (int shot = 0; shot < g.ns; ++shot) acc += (double)G[((long long)s * g.ns + shot) * cells + j];
        const double v = (double)vel[e];
        grad[e] = (float)(coef * acc / v);
    }
}

__global__ void k3_misfit_partial(const float *__restrict__ syn, const float *__restrict__ obs, long long per_sample,
                                  long long obs_len, double *__restrict__ part)
{
    const int s = blockIdx.y;
    double acc = 0.0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < per_sample;
         e += (long long)gridDim.x * blockDim.x) {
        const double r = (double)syn[(long long)s * per_sample + e] - (double)obs[e % obs_len];
        acc += r * r;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double red[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        part[(long long)s * gridDim.x + blockIdx.x] = t;
    }
}

__global__ void k3_misfit_final(const double *__restrict__ part, double *__restrict__ misfit, int nsamples)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsamples) return;
    double t = 0.0;
    for (int i = 0; i < kMisfitBlocks; ++i) t += part[(long long)s * kMisfitBlocks + i];
    misfit[s] = 0.5 * t;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

struct Host3 {
    Geom3 g;
    std::vector<float> w, omw;
    std::vector<int> uoff, uidx;
};

static int round_up(int v, int m) { return (v + m - 1) / m * m; }

static int validate(const gb_fwi3d_params *p, const gb_fwi3d_acq *a)
{
    if (!p || !a || !a->src || !a->rec || !a->wavelet) return GB_FWI2D_EINVAL;
    if (p->nx < 1 || p->ny < 1 || p->nz < 1 || p->pml0 < 1 || p->Lc < 3 || p->Lc > 6 || p->ns < 1 ||
        p->nr < 1 || p->nt < 1 || p->nt_interval < 1)
        return GB_FWI2D_EINVAL;
    if (!(p->dx > 0) || !(p->dy > 0) || !(p->dz > 0) || !(p->dt > 0) || !std::isfinite(p->dx) ||
        !std::isfinite(p->dy) || !std::isfinite(p->dz) || !std::isfinite(p->dt))
        return GB_FWI2D_EINVAL;
    const long long pml = (long long)p->pml0 + p->Lc + 1;
    if (p->nx + 2 * pml > (1 << 20) || p->ny + 2 * pml > (1 << 20) || p->nz + 2 * pml > (1 << 20))
        return GB_FWI2D_EINVAL;
    for (int s = 0; s < p->ns; ++s) {
        const int *c = a->src + 3 * s;
        if (c[0] < 0 || c[0] >= p->nx || c[1] < 0 || c[1] >= p->ny || c[2] < 0 || c[2] >= p->nz)
            return GB_FWI2D_EINVAL;
    }
    for (int r = 0; r < p->nr; ++r) {
        const int *c = a->rec + 3 * r;
        if (c[0] < 0 || c[0] >= p->nx || c[1] < 0 || c[1] >= p->ny || c[2] < 0 || c[2] >= p->nz)
            return GB_FWI2D_EINVAL;
    }
    for (int it = 0; it < p->nt; ++it)
        if (!std::isfinite(a->wavelet[it])) return GB_FWI2D_EINVAL;
    return GB_FWI2D_OK;
}

static void derive(const gb_fwi3d_params &p, const gb_fwi3d_acq &a, Host3 &h)
{
    Geom3 &g = h.g;
    std::memset(&g, 0, sizeof g);
    g.L = p.Lc + 1;
    g.pml0 = p.pml0;
    g.pml = p.pml0 + g.L;
    g.nx = p.nx; g.ny = p.ny; g.nz = p.nz;
    g.ntx = p.nx + 2 * g.pml; g.nty = p.ny + 2 * g.pml; g.ntz = p.nz + 2 * g.pml;
    g.pitch = round_up(g.ntx, kBX);
    g.sz = (long long)g.pitch * g.nty;
    g.fstride = g.sz * g.ntz;
    g.istride = (long long)p.nx * p.ny * p.nz;
    g.nt = p.nt; g.nti = p.nt_interval; g.ns = p.ns; g.nr = p.nr;
    g.tiles_x = (g.ntx + kBX - 1) / kBX;
    g.tiles_y = (g.nty + kBY - 1) / kBY;
    g.chunks_z = (g.ntz + kZC - 1) / kZC;
    const double d[3] = {p.dx, p.dy, p.dz};
    for (int i = 0; i < 3; ++i) {
        g.id[i] = (float)(1.0 / d[i]);
        g.id2[i] = (float)(1.0 / (d[i] * d[i]));
    }
    g.idt2 = (float)(1.0 / ((double)p.dt * (double)p.dt));
    g.dt = p.dt;
    h.w.resize(p.pml0);
    h.omw.resize(p.pml0);
    for (int i = 0; i < p.pml0; ++i) {
        h.w[i] = (float)(1.0 - (double)i / p.pml0);
        h.omw[i] = (float)(1.0 - (double)h.w[i]);
    }
    // receivers grouped by cell, each group in receiver order
    std::vector<std::pair<long long, int>> rc(p.nr);
    for (int r = 0; r < p.nr; ++r) {
        const int *c = a.rec + 3 * r;
        rc[r] = {((long long)c[2] * p.ny + c[1]) * p.nx + c[0], r};
    }
    std::stable_sort(rc.begin(), rc.end(), [](const auto &u, const auto &v) { return u.first < v.first; });
    h.uoff.clear();
    h.uidx.resize(p.nr);
    for (int i = 0; i < p.nr; ++i) {
        if (i == 0 || rc[i].first != rc[i - 1].first) h.uoff.push_back(i);
        h.uidx[i] = rc[i].second;
    }
    h.uoff.push_back(p.nr);
    g.nu = (int)h.uoff.size() - 1;
}

struct Layout3 {
    size_t tab_src, tab_rec, tab_uoff, tab_uidx, tab_w, tab_omw;
    size_t vdt, ring, ring2, ckpt, snap, G, syn, part, total;
    int resident, K, nseg, nsnap;
};

static size_t a256(size_t v) { return (v + 255) & ~(size_t)255; }

static Layout3 plan(const Geom3 &g, int nsamples, int resident, bool fwd_only, bool ckpt, bool syn_in_work)
{
    Layout3 L{};
    const long long ninst = (long long)nsamples * g.ns;
    if (resident <= 0 || resident > ninst) resident = (int)ninst;
    resident = std::min(resident, 65535);
    L.resident = resident;
    if (fwd_only) {
        L.K = g.nt;
        L.nseg = 1;
        L.nsnap = 0;
    } else if (ckpt) {
        const int root = (int)std::ceil(std::sqrt((double)g.nt));
        L.K = (root + g.nti - 1) / g.nti * g.nti;
        L.nseg = (g.nt + L.K - 1) / L.K;
        L.nsnap = (L.K + g.nti - 1) / g.nti;
    } else {
        L.K = g.nt;
        L.nseg = 1;
        L.nsnap = (g.nt + g.nti - 1) / g.nti;
    }
    const size_t f = sizeof(float) * (size_t)g.fstride, fi = sizeof(float) * (size_t)g.istride;
    size_t off = 0;
    L.tab_src = off;   off = a256(off + sizeof(int) * 3 * g.ns);
    L.tab_rec = off;   off = a256(off + sizeof(int) * 3 * g.nr);
    L.tab_uoff = off;  off = a256(off + sizeof(int) * (g.nr + 1));
    L.tab_uidx = off;  off = a256(off + sizeof(int) * g.nr);
    L.tab_w = off;     off = a256(off + sizeof(float) * g.pml0);
    L.tab_omw = off;   off = a256(off + sizeof(float) * g.pml0);
    L.vdt = off;       off = a256(off + f * nsamples);
    L.ring = off;      off = a256(off + f * 3 * resident);
    L.ring2 = L.ckpt = L.snap = L.G = off;
    if (!fwd_only) {
        L.ring2 = off; off = a256(off + f * 3 * resident);
        L.ckpt = off;
        if (L.nseg > 1) off = a256(off + f * 2 * (size_t)L.nseg * resident);
        L.snap = off;  off = a256(off + fi * (size_t)L.nsnap * resident);
        L.G = off;     off = a256(off + fi * (size_t)ninst);
    }
    L.syn = off;
    if (syn_in_work) off = a256(off + sizeof(float) * (size_t)ninst * g.nt * g.nr);
    L.part = off;      off = a256(off + sizeof(double) * kMisfitBlocks * nsamples);
    L.total = off;
    return L;
}

static thread_local long long t_launches = 0;

static int grid_for(long long n, int block)
{
    return (int)std::min<long long>((n + block - 1) / block, 152LL * 32);
}

template <int H>
static void launch_step(bool adj, const Geom3 &g, const Batch3 &b, int nres, int k, int snap, cudaStream_t st)
{
    const dim3 grid(g.tiles_x * g.tiles_y * g.chunks_z, nres), block(kBX, kBY);
    if (adj)
        k3_step<H, true><<<grid, block, 0, st>>>(g, b, k, snap);
    else
        k3_step<H, false><<<grid, block, 0, st>>>(g, b, k, snap);
}

static void step(bool adj, const Geom3 &g, const Batch3 &b, int nres, int k, int snap, cudaStream_t st)
{
    switch (g.L - 1) {
    case 3: launch_step<3>(adj, g, b, nres, k, snap, st); break;
    case 4: launch_step<4>(adj, g, b, nres, k, snap, st); break;
    case 5: launch_step<5>(adj, g, b, nres, k, snap, st); break;
    default: launch_step<6>(adj, g, b, nres, k, snap, st); break;
    }
    ++t_launches;
}

}  // namespace gbfwi3

using namespace gbfwi3;

extern "C" {

int gb_fwi3d_validate(const gb_fwi3d_params *p, const gb_fwi3d_acq *a) { return validate(p, a); }

int gb_fwi3d_workspace_size(const gb_fwi3d_params *p, const gb_fwi3d_acq *a, int nsamples, int max_resident,
                            unsigned flags, size_t *bytes)
{
    if (!bytes || nsamples < 1) return GB_FWI2D_EINVAL;
    const int st = validate(p, a);
    if (st) return st;
    Host3 h;
    derive(*p, *a, h);
    *bytes = plan(h.g, nsamples, max_resident, (flags & GB_FWI3D_FORWARD_ONLY) != 0,
                  (flags & GB_FWI3D_CHECKPOINT) != 0, true)
                 .total;
    return GB_FWI2D_OK;
}

int gb_fwi3d_max_resident(const gb_fwi3d_params *p, const gb_fwi3d_acq *a, int nsamples, unsigned flags,
                          size_t budget)
{
    if (nsamples < 1 || validate(p, a)) return 0;
    Host3 h;
    derive(*p, *a, h);
    const bool fo = (flags & GB_FWI3D_FORWARD_ONLY) != 0, ck = (flags & GB_FWI3D_CHECKPOINT) != 0;
    long long lo = 0, hi = std::min<long long>((long long)nsamples * p->ns, 65535);
    while (lo < hi) {
        const long long mid = (lo + hi + 1) / 2;
        if (plan(h.g, nsamples, (int)mid, fo, ck, true).total <= budget)
            lo = mid;
        else
            hi = mid - 1;
    }
    return (int)lo;
}

long long gb_fwi3d_last_launches(void) { return t_launches; }

int gb_fwi3d_run(const gb_fwi3d_params *p, const gb_fwi3d_acq *a, int nsamples, const float *vel, const float *obs,
                 float *syn, float *grad, double *misfit, void *work, size_t work_bytes, int max_resident,
                 unsigned flags, void *stream)
{
    t_launches = 0;
    if (nsamples < 1 || !vel || !work) return GB_FWI2D_EINVAL;
    int st0 = validate(p, a);
    if (st0) return st0;
    const bool fwd_only = (flags & GB_FWI3D_FORWARD_ONLY) != 0;
    const bool ckpt = (flags & GB_FWI3D_CHECKPOINT) != 0;
    if (!fwd_only && (!obs || !grad)) return GB_FWI2D_EINVAL;
    if (misfit && !obs) return GB_FWI2D_EINVAL;
    Host3 h;
    derive(*p, *a, h);
    const Geom3 &g = h.g;
    const Layout3 L = plan(g, nsamples, max_resident, fwd_only, ckpt, syn == nullptr);
    if (L.total > work_bytes) return GB_FWI2D_ENOMEM;
    cudaStream_t st = (cudaStream_t)stream;
    char *w = (char *)work;
    auto up = [&](size_t off, const void *src, size_t n) {
        if (n) cudaMemcpyAsync(w + off, src, n, cudaMemcpyHostToDevice, st);
    };
    up(L.tab_src, a->src, sizeof(int) * 3 * g.ns);
    up(L.tab_rec, a->rec, sizeof(int) * 3 * g.nr);
    up(L.tab_uoff, h.uoff.data(), sizeof(int) * h.uoff.size());
    up(L.tab_uidx, h.uidx.data(), sizeof(int) * h.uidx.size());
    up(L.tab_w, h.w.data(), sizeof(float) * h.w.size());
    up(L.tab_omw, h.omw.data(), sizeof(float) * h.omw.size());

    const long long ninst = (long long)nsamples * g.ns;
    Batch3 b{};
    b.vdt = (float *)(w + L.vdt);
    b.vel = vel;
    b.obs = obs;
    b.syn = syn ? syn : (float *)(w + L.syn);
    b.ring = (float *)(w + L.ring);
    b.snap = (float *)(w + L.snap);
    b.G = (float *)(w + L.G);
    b.w = (const float *)(w + L.tab_w);
    b.omw = (const float *)(w + L.tab_omw);
    b.src = (const int *)(w + L.tab_src);
    b.rec = (const int *)(w + L.tab_rec);
    b.uoff = (const int *)(w + L.tab_uoff);
    b.uidx = (const int *)(w + L.tab_uidx);
    b.nsnap = L.nsnap;
    Batch3 ba = b;  // the adjoint's ring
    ba.ring = (float *)(w + L.ring2);

    k3_prepare<<<grid_for((long long)nsamples * g.fstride, 256), 256, 0, st>>>(g, vel, (float *)b.vdt, nsamples);
    ++t_launches;
    if (!fwd_only) cudaMemsetAsync(b.G, 0, sizeof(float) * (size_t)g.istride * ninst, st);
    const size_t fb = sizeof(float) * (size_t)g.fstride;
    const int io_threads = 256;
    float *ck = (float *)(w + L.ckpt);
    const size_t ck_pitch = 2 * (size_t)L.nseg * fb;
    const size_t ring_pitch = 3 * fb;
    for (long long i0 = 0; i0 < ninst; i0 += L.resident) {
        const int nres = (int)std::min<long long>(L.resident, ninst - i0);
        b.inst0 = ba.inst0 = (int)i0;
        // forward: data; the stored field (one segment) or the checkpoints
        cudaMemsetAsync(b.ring, 0, 3 * fb * (size_t)nres, st);
        for (int k = 0; k < g.nt; ++k) {
            if (!fwd_only && L.nseg > 1 && k % L.K == 0) {
                const int s = k / L.K;
                for (int hh = 0; hh < 2; ++hh)
                    cudaMemcpy2DAsync((char *)ck + (size_t)(2 * s + hh) * fb, ck_pitch,
                                      (char *)b.ring + (size_t)((k + hh) % 3) * fb, ring_pitch, fb, nres,
                                      cudaMemcpyDeviceToDevice, st);
            }
            const int snap = (!fwd_only && L.nseg == 1 && k % g.nti == 0) ? k / g.nti : -1;
            step(false, g, b, nres, k, snap, st);
            k3_io_fwd<<<nres, io_threads, 0, st>>>(g, b, k, k, a->wavelet[k], snap, 1);
            ++t_launches;
        }
        if (fwd_only) continue;
        // adjoint, segment by segment from the last
        cudaMemsetAsync(ba.ring, 0, 3 * fb * (size_t)nres, st);
        for (int s = L.nseg - 1; s >= 0; --s) {
            const int k0 = s * L.K, k1 = std::min(k0 + L.K, g.nt);
            if (L.nseg > 1) {
                for (int hh = 0; hh < 2; ++hh)
                    cudaMemcpy2DAsync((char *)b.ring + (size_t)((k0 + hh) % 3) * fb, ring_pitch,
                                      (char *)ck + (size_t)(2 * s + hh) * fb, ck_pitch, fb, nres,
                                      cudaMemcpyDeviceToDevice, st);
                for (int k = k0; k < k1; ++k) {
                    const int snap = k % g.nti == 0 ? (k - k0) / g.nti : -1;
                    step(false, g, b, nres, k, snap, st);
                    k3_io_fwd<<<nres, io_threads, 0, st>>>(g, b, k, k, a->wavelet[k], snap, 0);
                    ++t_launches;
                }
            }
            for (int it = k1 - 1; it >= k0; --it) {
                const int ka = g.nt - 1 - it;
                const int snap = it % g.nti == 0 ? (L.nseg == 1 ? it / g.nti : (it - k0) / g.nti) : -1;
                step(true, g, ba, nres, ka, snap, st);
                k3_io_adj<<<nres, io_threads, 0, st>>>(g, ba, ka, it, snap);
                ++t_launches;
            }
        }
    }
    if (grad && !fwd_only) {
        k3_reduce_grad<<<grid_for((long long)nsamples * g.istride, 256), 256, 0, st>>>(g, b.G, vel, grad, nsamples);
        ++t_launches;
    }
    if (misfit) {
        double *part = (double *)(w + L.part);
        const long long per = (long long)g.ns * g.nt * g.nr;
        k3_misfit_partial<<<dim3(kMisfitBlocks, nsamples), 256, 0, st>>>(b.syn, obs, per, per, part);
        k3_misfit_final<<<(nsamples + 127) / 128, 128, 0, st>>>(part, misfit, nsamples);
        t_launches += 2;
    }
    return cudaGetLastError() == cudaSuccess ? GB_FWI2D_OK : GB_FWI2D_ECUDA;
}

}  // extern "C"

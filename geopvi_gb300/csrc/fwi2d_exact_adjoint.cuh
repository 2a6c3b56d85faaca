// fwi2d_exact_adjoint.cuh -- exact discrete adjoint of the FD scheme.
//
// The reference's gradient (backward_IO, geopvi/forward/fwi2d/
// fdtd2D_modelling.c:941-978) back-propagates the residual with the forward
// operator and correlates it with the stored second time derivative: a
// continuous-adjoint approximation, about dt * dJ/dv and a few degrees off
// in direction.  Finite-difference checks of dJ/dv need the transpose of the
// scheme itself.  One step maps the two previous levels linearly,
//   p2_c = beta_c * S_c + sum_b gamma_{c,b} * E_{c,b} (+ source),
// S_c the stencil value 2 p1 - p0 + a_c (Dxx + Dzz) p1 inside the stencil
// region (a_c = (v dt)^2) and the copied p1_c outside it, E_{c,b} the
// one-way extrapolation of boundary blend b (top/bottom first, then
// left/right) with weight w_b: beta = prod (1 - w_b), gamma_1 = w_1 (1 - w_2),
// gamma_2 = w_2.  With lambda^k = dJ/dP^k for J = 1/2 sum |R P^{t+1} - obs_t|^2,
//   lambda^k = R^T r_{k-1} + A1^T lambda^{k+1} + A0^T lambda^{k+2},
//   dJ/dv_c += lambda^{t+1}_c * d p2_c / d v_c  (step t: p1 = P^t, p0 = P^{t-1}).
// k_adjoint_tile computes lambda^k for every cell as a gather over the
// cells whose update reads it, and accumulates the padded-grid gradient;
// k_reduce_exact sums it back onto the interior cells that get_velp's
// padding replicates.  FP32 arithmetic: this path has no reference output to
// match bit for bit; the FP64 oracle of the same recursion is its check.
#pragma once

#include "fwi2d_kernels.cuh"

namespace gbfwi {

struct ExactBatch {
    const float *vdt;      // [nsamples][fstride] padded v*dt
    const float *abeta;    // [nsamples][fstride] (v dt)^2 beta on stencil cells, 0 elsewhere
    const int4 *cells;     // [ntz][ntx] packed CellInfo of the geometry (cell_pack)
    const float *obs;      // [ns][nt][nr]
    const float *syn;      // [nsamples*ns][nt][nr]
    float *lam;            // [resident][3][fstride] adjoint levels
    float *nu;             // [resident][3][fstride] a_c beta_c lambda_c beside each level of lam
    const float *store;    // [resident][levels][fstride] forward levels of the segment
    long long store_pitch; // floats between resident slots of `store`
    int store_levels;      // levels per resident slot of `store`
    float *gpad;           // [nsamples*ns][fstride] padded-grid dJ/dv
    const float *taps;     // [nsamples][16][fstride] blend taps per cell: kBandZ.. then kBandX..
    const BlendCoef *coef; // boundary weights
    int *status;           // device error word (0 = ok)
    float rdx2, rdz2;      // 1 / dx^2, 1 / dz^2
    float dtdx;            // dt / dx: d s / d v for s = v dt / dx
    int inst0;
};

// Planes of ExactBatch::taps for one sample: for the z blend (top / bottom
// band) of a cell c and then for its x blend (left / right), its weight
// gamma times the coefficients of p1 at 0, 1, 2 steps inward (2 t11, 2 t12,
// 2 t13) and of p0 at 0..4 steps inward (t11^2, 2 t11 t12, t12^2 + 2 t11 t13,
// 2 t12 t13, t13^2): the entries of A1 and A0 that the blend puts in row c.
constexpr int kBandZ = 0, kBandX = 8, kTapPlanes = 16;

// Blend facts of one padded cell: blends applied in order (top/bottom, then
// left/right), their inward steps and weights, beta and gamma.
struct CellInfo {
    bool sten;   // in the stencil region
    int nb;      // blends 0..2
    int dir[2];  // 0 top (+z inward), 1 bottom (-z), 2 left (+x), 3 right (-x)
    float beta, gam[2];
};

__device__ __forceinline__ CellInfo cell_info(const Geom &g, const BlendCoef *coef, int iz, int ix)
{
    CellInfo ci;
    ci.sten = iz >= g.Lc && iz < g.ntz - g.Lc && ix >= g.Lc && ix < g.ntx - g.Lc;
    float w[2] = {0.0f, 0.0f};
    ci.nb = 0;
    ci.dir[0] = ci.dir[1] = -1;
    if (iz >= g.Lc && iz < g.pml) { ci.dir[ci.nb] = 0; w[ci.nb++] = coef[iz - g.Lc].w; }
    else if (iz >= g.ntz - g.pml && iz < g.ntz - g.Lc) { ci.dir[ci.nb] = 1; w[ci.nb++] = coef[g.ntz - g.Lc - iz - 1].w; }
    if (ix >= g.Lc && ix < g.pml) { ci.dir[ci.nb] = 2; w[ci.nb++] = coef[ix - g.Lc].w; }
    else if (ix >= g.ntx - g.pml && ix < g.ntx - g.Lc) { ci.dir[ci.nb] = 3; w[ci.nb++] = coef[g.ntx - g.Lc - ix - 1].w; }
    ci.beta = 1.0f;
    ci.gam[0] = ci.gam[1] = 0.0f;
    if (ci.nb == 1) {
        ci.beta = 1.0f - w[0];
        ci.gam[0] = w[0];
    } else if (ci.nb == 2) {
        ci.beta = (1.0f - w[0]) * (1.0f - w[1]);
        ci.gam[0] = w[0] * (1.0f - w[1]);
        ci.gam[1] = w[1];
    }
    return ci;
}

// CellInfo packed into 16 bytes: x = sten | nb << 1 | (dir0 + 1) << 4 |
// (dir1 + 1) << 8, then beta, gam0, gam1 as float bits.  The same for every
// sample of a geometry, so it is built once and read through the cache.
__device__ __forceinline__ int4 cell_pack(const CellInfo &c)
{
    return make_int4((c.sten ? 1 : 0) | (c.nb << 1) | ((c.dir[0] + 1) << 4) | ((c.dir[1] + 1) << 8),
                     __float_as_int(c.beta), __float_as_int(c.gam[0]), __float_as_int(c.gam[1]));
}

__device__ __forceinline__ CellInfo cell_unpack(int4 v)
{
    CellInfo c;
    c.sten = (v.x & 1) != 0;
    c.nb = (v.x >> 1) & 3;
    c.dir[0] = ((v.x >> 4) & 15) - 1;
    c.dir[1] = ((v.x >> 8) & 15) - 1;
    c.beta = __int_as_float(v.y);
    c.gam[0] = __int_as_float(v.z);
    c.gam[1] = __int_as_float(v.w);
    return c;
}

// Extrapolation weights of s = v dt / dx (abc_for_p's t11, t12, t13).
struct Taps {
    float t11, t12, t13;
};
__device__ __forceinline__ Taps taps_of(float s)
{
    return Taps{(2.0f - s) * (1.0f - s) * 0.5f, s * (2.0f - s), s * (s - 1.0f) * 0.5f};
}

// The geometry's cell table and each sample's (v dt)^2 beta field and blend taps.
__global__ void k_exact_tables(const Geom g, const BlendCoef *coef, const float *__restrict__ vdt, int nsamples,
                               int4 *__restrict__ cells, float *__restrict__ abeta, float *__restrict__ taps)
{
    const long long n = (long long)g.ntz * g.ntx;
    for (long long d = blockIdx.x * (long long)blockDim.x + threadIdx.x; d < n;
         d += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(d / g.ntx), ix = (int)(d - (long long)iz * g.ntx);
        cells[d] = cell_pack(cell_info(g, coef, iz, ix));
    }
    const long long m = (long long)nsamples * g.fstride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e % g.fstride;
        const int iz = (int)(r / g.pitch), ix = (int)(r - (long long)iz * g.pitch) - g.xoff;
        float a = 0.0f, gz = 0.0f, gx = 0.0f;
        if (ix >= 0 && ix < g.ntx) {
            const CellInfo c = cell_info(g, coef, iz, ix);
            if (c.sten) a = vdt[e] * vdt[e] * c.beta;
            for (int bb = 0; bb < c.nb; ++bb) (c.dir[bb] <= 1 ? gz : gx) = c.gam[bb];
        }
        abeta[e] = a;
        const Taps t = taps_of(vdt[e] / g.dx);
        const float cf[8] = {2.0f * t.t11, 2.0f * t.t12, 2.0f * t.t13, t.t11 * t.t11, 2.0f * t.t11 * t.t12,
                             t.t12 * t.t12 + 2.0f * t.t11 * t.t13, 2.0f * t.t12 * t.t13, t.t13 * t.t13};
        float *tp = taps + (e / g.fstride) * kTapPlanes * g.fstride + r;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            tp[(kBandZ + q) * g.fstride] = gz * cf[q];
            tp[(kBandX + q) * g.fstride] = gx * cf[q];
        }
    }
}


// Step k of the backward recursion for every cell of every resident solve:
// lambda^k into lam[k % 3] (and nu = a beta lambda^k beside it), and
// dJ/dv_j += lambda^k_j * d p2_j / d v_j of forward step k-1, whose inputs
// P^{k-1} and P^{k-2} sit in store levels `lev1` and lev1 - 1.  rik_prev =
// the Ricker value of step k-1.  lambda^k_j gathers over the cells whose
// update reads j: R^T r_{k-1} at receivers, the stencil's transpose
// (a_c beta_c lambda_c of the cross around j, plus 2 beta_j lambda^{k+1}_j -
// beta_j lambda^{k+2}_j on stencil cells, beta_j lambda^{k+1}_j elsewhere:
// the copied level) and the blends' transposes within 4 cells of a band.
//
// One block per (tile of kTileX x kTileZ cells, resident solve); the two
// stencil gathers read shared memory, staged by TMA: nu of level k+1 (written
// beside lambda^{k+1} by the previous step, so a tap of A1^T is one shared
// load instead of two global ones; zero outside the stencil region, in the
// pad columns and, by the copy's fill, outside the grid) and the forward
// level P^{k-1} for the Laplacian of d p2 / d v.  Band taps stay global
// loads.  Tiles entirely in the stencil region and four or more cells away
// from every band take constants for their cell facts.
constexpr int kAdjRowsPerThread = 2;                              // rows r0 and r0 + kTileZ / 2
constexpr int kAdjThreads = kTileX * kTileZ / kAdjRowsPerThread;  // 256
constexpr int kAdjMinBlocks = 5;  // resident blocks per SM: each waits on its tiles' copy first

template <int H>
struct AdjShape {
    static constexpr int kTile = TileShape<H>::kP1Floats;  // floats of one staged tile
    static constexpr int kBytes = 2 * 4 * kTile;            // TMA bytes per block
    static constexpr int kSmem = kBytes + 16;               // + the mbarrier
};

template <int H>
__global__ void __launch_bounds__(kAdjThreads, kAdjMinBlocks)
    k_adjoint_tile(const __grid_constant__ CUtensorMap tm_nu, const __grid_constant__ CUtensorMap tm_store,
                   const Geom g, const ExactBatch b, int k, int lev1, float rik_prev)
{
    constexpr int R = kAdjRowsPerThread, RS = kTileZ / R;  // rows per thread, their spacing
    using AS = AdjShape<H>;
    extern __shared__ __align__(1024) float smem[];
    float *s_nu = smem, *s_p1 = smem + AS::kTile;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + 2 * AS::kTile);  // [0] nu, [1] P^{k-1}
    const int slot = blockIdx.y;
    const int inst = b.inst0 + slot;
    const int sample = inst / g.ns, shot = inst - sample * g.ns;
    const int trow = blockIdx.x / g.tiles_x, tcol = blockIdx.x - trow * g.tiles_x;
    const int col0 = tcol * kTileX, row0 = trow * kTileZ;
    const int lane = threadIdx.x & 31, rr0 = threadIdx.x >> 5;  // tile rows rr0 + q * RS
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    const long long P = g.pitch;
    const float *vdt = b.vdt + (long long)sample * g.fstride;
    float *l_base = b.lam + (long long)slot * 3 * g.fstride;
    const float *lam1 = l_base + (long long)((k + 1) % 3) * g.fstride;  // lambda^{k+1}
    const float *lam2 = l_base + (long long)((k + 2) % 3) * g.fstride;  // lambda^{k+2}
    float *lam0 = l_base + (long long)(k % 3) * g.fstride;
    float *nu0 = b.nu + ((long long)slot * 3 + k % 3) * g.fstride;
    const float *ab = b.abeta + (long long)sample * g.fstride;
    const float *st = b.store + (long long)slot * b.store_pitch;
    const float *p1 = st + (long long)lev1 * g.fstride;
    const float *p0 = p1 - g.fstride;
    const float rdx2 = b.rdx2, rdz2 = b.rdz2;
    // Block-uniform: every cell of the tile in the stencil region, no blend
    // tap within reach (4 cells), so sten = 1, nb = 0, beta = 1.
    const int ix0 = col0 - g.xoff;
    const bool plain = ix0 >= g.pml + 4 && ix0 + kTileX <= g.ntx - g.pml - 4 && row0 >= g.pml + 4 &&
                       row0 + kTileZ <= g.ntz - g.pml - 4;

    // The per-sample fields are constant through the call: read them while
    // the previous step drains.
    const int ix = ix0 + lane;
    const bool col_live = ix >= 0 && ix < g.ntx;
    const long long j0 = (long long)(row0 + rr0) * P + col0 + lane;
    float l1v[R], l2v[R], abv[R], vdv[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
        const bool live = col_live && row0 + rr0 + q * RS < g.ntz;
        abv[q] = live ? __ldg(ab + j0 + q * RS * P) : 0.0f;
        vdv[q] = live ? __ldg(vdt + j0 + q * RS * P) : 0.0f;
    }
    // Below here every read may see the previous step's writes (lambda^{k+1},
    // nu^{k+1}, the gradient accumulator): launched programmatically, this
    // step waits for it first.
    grid_dependency_wait();
    grid_launch_dependents();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&bar[0], AS::kBytes / 2);
        tma_load_3d(s_nu, &tm_nu, &bar[0], col0 - kHaloX, row0 - H, slot * 3 + (k + 1) % 3);
        mbar_arrive_expect_tx(&bar[1], AS::kBytes / 2);
        tma_load_3d(s_p1, &tm_store, &bar[1], col0 - kHaloX, row0 - H, slot * b.store_levels + lev1);
    }
#pragma unroll
    for (int q = 0; q < R; ++q) {
        const bool live = col_live && row0 + rr0 + q * RS < g.ntz;
        l1v[q] = live ? lam1[j0 + q * RS * P] : 0.0f;
        l2v[q] = live ? lam2[j0 + q * RS * P] : 0.0f;
    }
    if (!mbar_wait_bounded(&bar[0], 0)) {
        if (threadIdx.x == 0) atomicOr(b.status, kStatusTmaTimeout);
        // the copies may still land: wait again (bounded) for both before retiring
        mbar_wait_bounded(&bar[0], 0);
        mbar_wait_bounded(&bar[1], 0);
        return;
    }
    const int sc = lane + kHaloX;
    if (plain) {
        // Every cell a stencil cell with beta = 1 and no blend within reach:
        // the same arithmetic as below with those facts as constants, and
        // 32-bit offsets within the fields (a field is far below 2^31 cells).
        const int jp = (row0 + rr0) * g.pitch + col0 + lane;
        float outp[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const int rr = rr0 + q * RS;
            const int iz = row0 + rr;
            const int j = jp + q * RS * g.pitch;
            const float *sn = s_nu + (rr + H) * kBoxX + sc;
            float out = 0.0f;
            if (iz == g.r_iz) {  // R^T r_{k-1}
                const int ir = receiver_of(g, ix);
                if (ir >= 0) {
                    const long long t = (long long)(k - 1) * g.nr + ir;
                    out += b.syn[(long long)inst * g.nt * g.nr + t] - b.obs[(long long)shot * g.nt * g.nr + t];
                }
            }
            out += 2.0f * l1v[q] + fd_weight<H>(0) * (rdx2 + rdz2) * sn[0];
            out -= l2v[q];
#pragma unroll
            for (int m = 1; m <= H; ++m)
                out += fd_weight<H>(m) * (rdx2 * (sn[m] + sn[-m]) + rdz2 * (sn[m * kBoxX] + sn[-m * kBoxX]));
            lam0[j] = out;
            nu0[j] = abv[q] * out;
            outp[q] = out;
        }
        if (!mbar_wait_bounded(&bar[1], 0)) {
            if (threadIdx.x == 0) atomicOr(b.status, kStatusTmaTimeout);
            mbar_wait_bounded(&bar[1], 0);
            return;
        }
        float *gp = b.gpad + (long long)inst * g.fstride;
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const float out = outp[q];
            if (out == 0.0f) continue;
            const int rr = rr0 + q * RS;
            const int iz = row0 + rr;
            const int j = jp + q * RS * g.pitch;
            const float *sp1 = s_p1 + (rr + H) * kBoxX + sc;
            float lx = fd_weight<H>(0) * sp1[0], lz = lx;
#pragma unroll
            for (int m = 1; m <= H; ++m) {
                lx += fd_weight<H>(m) * (sp1[m] + sp1[-m]);
                lz += fd_weight<H>(m) * (sp1[m * kBoxX] + sp1[-m * kBoxX]);
            }
            float d = 2.0f * vdv[q] * g.dt * (lx * rdx2 + lz * rdz2);
            if (iz == g.s_iz && ix == g.s_ix0 + shot * g.ds) d += 2.0f * rik_prev * g.dt * vdv[q];
            gp[j] += out * d;
        }
        return;
    }
    float outv[R];
    int4 cpk[R];  // each row's cell facts, packed (cell_pack)
#pragma unroll
    for (int q = 0; q < R; ++q) {
        outv[q] = 0.0f;
        if (!col_live) continue;
        const int rr = rr0 + q * RS;
        const int iz = row0 + rr;
        if (iz >= g.ntz) continue;
        const long long j = j0 + q * RS * P;
        const float *sn = s_nu + (rr + H) * kBoxX + sc;  // nu^{k+1} at j in the tile
        float out = 0.0f;
        if (iz == g.r_iz) {  // R^T r_{k-1}
            const int ir = receiver_of(g, ix);
            if (ir >= 0) {
                const long long t = (long long)(k - 1) * g.nr + ir;
                out += b.syn[(long long)inst * g.nt * g.nr + t] - b.obs[(long long)shot * g.nt * g.nr + t];
            }
        }
        CellInfo cj;
        if (plain) {
            cj.sten = true;
            cj.nb = 0;
            cj.dir[0] = cj.dir[1] = -1;
            cj.beta = 1.0f;
            cj.gam[0] = cj.gam[1] = 0.0f;
        } else {
            cj = cell_unpack(__ldg(b.cells + (long long)iz * g.ntx + ix));
        }
        if (cj.sten) {
            out += 2.0f * cj.beta * l1v[q] + fd_weight<H>(0) * (rdx2 + rdz2) * sn[0];
            out -= cj.beta * l2v[q];
        } else {
            out += cj.beta * l1v[q];
        }
#pragma unroll
        for (int m = 1; m <= H; ++m)
            out += fd_weight<H>(m) * (rdx2 * (sn[m] + sn[-m]) + rdz2 * (sn[m * kBoxX] + sn[-m * kBoxX]));
        if (!plain) {
            // A1^T and A0^T of the blends: cells c whose band's extrapolation
            // reads j, 0..4 steps inward of c, with their tabled taps.
            const float *tz = b.taps + (long long)sample * kTapPlanes * g.fstride;
            const float *tx = tz + (long long)kBandX * g.fstride;
            const long long fs = g.fstride;
            if (iz >= g.Lc && iz - 4 < g.pml) {  // top band, c = j - kk rows
#pragma unroll
                for (int kk = 0; kk <= 4; ++kk) {
                    const int cz = iz - kk;
                    if (cz < g.Lc || cz >= g.pml) continue;
                    const long long c = j - kk * P;
                    if (kk < 3) out += __ldg(tz + kk * fs + c) * __ldg(lam1 + c);
                    out -= __ldg(tz + (3 + kk) * fs + c) * __ldg(lam2 + c);
                }
            }
            if (iz < g.ntz - g.Lc && iz + 4 >= g.ntz - g.pml) {  // bottom band, c = j + kk rows
#pragma unroll
                for (int kk = 0; kk <= 4; ++kk) {
                    const int cz = iz + kk;
                    if (cz < g.ntz - g.pml || cz >= g.ntz - g.Lc) continue;
                    const long long c = j + kk * P;
                    if (kk < 3) out += __ldg(tz + kk * fs + c) * __ldg(lam1 + c);
                    out -= __ldg(tz + (3 + kk) * fs + c) * __ldg(lam2 + c);
                }
            }
            if (ix >= g.Lc && ix - 4 < g.pml) {  // left band, c = j - kk columns
#pragma unroll
                for (int kk = 0; kk <= 4; ++kk) {
                    const int cx = ix - kk;
                    if (cx < g.Lc || cx >= g.pml) continue;
                    const long long c = j - kk;
                    if (kk < 3) out += __ldg(tx + kk * fs + c) * __ldg(lam1 + c);
                    out -= __ldg(tx + (3 + kk) * fs + c) * __ldg(lam2 + c);
                }
            }
            if (ix < g.ntx - g.Lc && ix + 4 >= g.ntx - g.pml) {  // right band, c = j + kk columns
#pragma unroll
                for (int kk = 0; kk <= 4; ++kk) {
                    const int cx = ix + kk;
                    if (cx < g.ntx - g.pml || cx >= g.ntx - g.Lc) continue;
                    const long long c = j + kk;
                    if (kk < 3) out += __ldg(tx + kk * fs + c) * __ldg(lam1 + c);
                    out -= __ldg(tx + (3 + kk) * fs + c) * __ldg(lam2 + c);
                }
            }
        }
        lam0[j] = out;
        nu0[j] = abv[q] * out;
        outv[q] = out;
        cpk[q] = cell_pack(cj);
    }
    // Every thread waits for the second tile, so the block retires only after
    // its copy has landed.
    if (!mbar_wait_bounded(&bar[1], 0)) {
        if (threadIdx.x == 0) atomicOr(b.status, kStatusTmaTimeout);
        mbar_wait_bounded(&bar[1], 0);
        return;
    }
    if (!col_live) return;
#pragma unroll
    for (int q = 0; q < R; ++q) {
        const float out = outv[q];
        if (out == 0.0f) continue;
        const int rr = rr0 + q * RS;
        const int iz = row0 + rr;
        const long long j = j0 + q * RS * P;
        const CellInfo cj = cell_unpack(cpk[q]);

        // d p2_j / d v_j of step k-1 (v dt^2 = (v dt) dt, d s / d v = dt / dx)
        float d = 0.0f;
        if (cj.sten) {
            const float *sp1 = s_p1 + (rr + H) * kBoxX + sc;
            float lx = fd_weight<H>(0) * sp1[0], lz = lx;
#pragma unroll
            for (int m = 1; m <= H; ++m) {
                lx += fd_weight<H>(m) * (sp1[m] + sp1[-m]);
                lz += fd_weight<H>(m) * (sp1[m * kBoxX] + sp1[-m * kBoxX]);
            }
            d += cj.beta * 2.0f * vdv[q] * g.dt * (lx * rdx2 + lz * rdz2);
        }
        if (cj.nb) {
            const float s = vdv[q] * g.rdx;
            const Taps t = taps_of(s);
            const float u11 = (2.0f * s - 3.0f) * 0.5f, u12 = 2.0f - 2.0f * s, u13 = (2.0f * s - 1.0f) * 0.5f;
            for (int bb = 0; bb < cj.nb; ++bb) {
                const long long sp = cj.dir[bb] == 0 ? P : cj.dir[bb] == 1 ? -P : cj.dir[bb] == 2 ? 1 : -1;
                const float dE = 2.0f * (u11 * p1[j] + u12 * p1[j + sp] + u13 * p1[j + 2 * sp]) -
                                 2.0f * t.t11 * u11 * p0[j] - 2.0f * (u11 * t.t12 + t.t11 * u12) * p0[j + sp] -
                                 2.0f * (t.t12 * u12 + u11 * t.t13 + t.t11 * u13) * p0[j + 2 * sp] -
                                 2.0f * (u12 * t.t13 + t.t12 * u13) * p0[j + 3 * sp] -
                                 2.0f * t.t13 * u13 * p0[j + 4 * sp];
                d += cj.gam[bb] * dE * b.dtdx;
            }
        }
        if (iz == g.s_iz && ix == g.s_ix0 + shot * g.ds) d += 2.0f * rik_prev * g.dt * vdv[q];
        b.gpad[(long long)inst * g.fstride + j] += out * d;
    }
}

// grad[s][cell] = sum over shots and over the padded cells that replicate
// the interior cell (get_velp is a clamp, fdtd2D_modelling.c:1187-1238),
// summed in double.
__global__ void k_reduce_exact(const Geom g, const float *__restrict__ gpad, float *__restrict__ grad,
                               int nsamples)
{
    const long long cells = (long long)g.nz * g.nx;
    const long long total = (long long)nsamples * cells;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(e / cells);
        const long long kk = e - (long long)s * cells;
        const int jz = (int)(kk / g.nx), jx = (int)(kk - (long long)jz * g.nx);
        const int z0 = jz == 0 ? 0 : jz + g.pml, z1 = jz == g.nz - 1 ? g.ntz - 1 : jz + g.pml;
        const int x0 = jx == 0 ? 0 : jx + g.pml, x1 = jx == g.nx - 1 ? g.ntx - 1 : jx + g.pml;
        double acc = 0.0;
        for (int shot = 0; shot < g.ns; ++shot) {
            const float *gp = gpad + ((long long)s * g.ns + shot) * g.fstride;
            for (int iz = z0; iz <= z1; ++iz)
                for (int ix = x0; ix <= x1; ++ix) acc += (double)gp[(long long)iz * g.pitch + ix + g.xoff];
        }
        grad[e] = (float)acc;
    }
}

}  // namespace gbfwi

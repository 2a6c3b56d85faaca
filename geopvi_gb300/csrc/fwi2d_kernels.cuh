// fwi2d_kernels.cuh -- sm_103a kernels of the 2-D acoustic FWI engine.
//
// One fused kernel advances every (sample, shot) solve of a wave by one time
// step: the 2*(Lc-1)-order Laplacian stencil (fdtd_2d_calculate_p,
// geopvi/forward/fwi2d/fdtd2D_modelling.c:756-780), the hybrid one-way
// absorbing boundary (abc_for_p, :833-900), Ricker source injection and
// receiver sampling (forward_IO, :902-939) or residual injection and the
// zero-lag imaging/gradient term (backward_IO, :941-978).  updata_p's copies
// (:1053-1066) become a rotation of three buffers, so no step copies a field.
//
// Data movement: one block -- a single warp -- owns a 32-column x 16-row tile
// of one solve.  An elected lane stages the previous time level with its
// stencil halo into shared memory with one TMA tensor load completing on an
// mbarrier; the warp then sweeps its 16 rows, keeping the z-stencil window in
// registers, reading the level before (p0) and v*dt with coalesced loads, and
// writes the new level, the stored snapshot (forward) or the gradient
// accumulator (adjoint) with coalesced 128-byte row stores.  One warp per
// block lets a warp of cheap interior rows retire without waiting for a
// slower absorbing-strip warp of the same tile (4-warp blocks of 64 rows
// were 5 % slower on the 200 x 400 batch, 2-warp blocks no faster than 4).
//
// Arithmetic follows the reference operation by operation: __fmul_rn /
// __fadd_rn / __fsub_rn never contract into FMA; divisions by the constant
// dx, dz, dt use a correctly rounded quotient (see div_const); the boundary
// blend is carried out in double exactly as the C expression promotes it.
// The forward data therefore match the reference bit for bit.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "fd_weights.cuh"
#include "fwi2d_exact.h"

namespace gbfwi {

constexpr int kTileX = 32;    // columns per tile: one warp
constexpr int kWarpRows = 16; // rows each warp sweeps
constexpr int kWarps = 1;     // warps per block, stacked in z
constexpr int kTileZ = kWarpRows * kWarps;  // 16 rows per tile
constexpr int kHaloX = 8;     // x halo of the staged tiles (TMA x offsets stay 16-byte aligned)
constexpr int kBoxX = kTileX + 2 * kHaloX;  // 48 staged columns
constexpr int kThreads = kTileX * kWarps;   // 128

// Kernel variants: rows per block of the interior sweep (U; loads run one
// block ahead) and resident blocks per SM the registers are capped for
// (65536 / (32 * blocks) registers a thread).  All variants compute the same
// values bit for bit; the engine's tuner times them on the caller's own
// batches and keeps the fastest per geometry and batch shape.  (2, 32) is the
// default: on the 200 x 400 grid four-row blocks overflow the instruction
// cache (the unrolled row bodies carry inline exact fallbacks) and fewer
// blocks per SM lose latency hiding.
struct StepVariant {
    int rows, min_blocks;
};
constexpr StepVariant kStepVariants[] = {{2, 32}, {4, 32}, {1, 32}, {2, 24}};
constexpr int kNumStepVariants = sizeof(kStepVariants) / sizeof(kStepVariants[0]);


// Geometry shared by every solve of one launch (one parameter set).
struct Geom {
    int ntx, ntz;        // padded grid (fdtd2D_modelling.c:86-87)
    int pitch, xoff;     // row pitch in floats; memory column of padded ix = 0
    int nx, nz, ipitch;  // interior grid and the row pitch of interior arrays
    int ioff;            // memory column of interior ix = pml in interior arrays
    int pml, Lc, pml0;   // Lc here is the reference's Lc after Lc += 1
    int s_iz, r_iz, r_ix0, dr, nr;
    int ds, s_ix0;       // source column of shot is: s_ix0 + is*ds
    int ns, nt, nti, nt_save;
    int tiles_x, tiles_z;
    int fast_dx, fast_dz;  // the host proved div_const exact for this divisor
    int pstd;            // laplace_solver = 1: pseudo-spectral Laplacian
    long long fstride;   // floats per padded field (ntz * pitch)
    long long pstride;   // floats per interior snapshot (nz * ipitch)
    float dx, dz, dt;
    float rdx, rdz;      // RN(1/dx), RN(1/dz)
    float fd[8];
};

// Where the solves of a wave live.  Solve `inst` = sample * ns + shot.
struct Batch {
    const float *vdt;    // [nsamples][fstride]   padded v*dt per sample
    const float *vel;    // [nsamples][nz*nx]      inner velocity per sample
    const float *obs;    // [ns][nt][nr]
    float *syn;          // [nsamples*ns][nt][nr]
    float *ring;         // [resident][levels][fstride]
    float *psave;        // [resident][nt_save][pstride]
    float *gacc;         // [nsamples*ns][pstride]
    const BlendCoef *coef;  // [pml0] boundary weight w, 1 - w split in floats and as double
    int blend_fp32;      // the host proved (1 - w) * q exact in double for every weight
    int *status;         // device error word (0 = ok)
    int inst0;           // first solve of this wave
    int slot0;           // first resident slot of this launch (the wave's second half)
    int levels;          // fields per resident slot of `ring`: 3, or the levels of a stored segment
    int tm_slot0;        // resident slot of ring[0] in the tensor map's fields (a map over several rings)
    int imaging;         // run_fwi == 0
    int store;           // forward pass stores the wavefield for the adjoint
    double *spec;        // pseudo-spectral mode: [resident][ntz][ntx] real array, then the
                         // [resident][ntz][ntx/2+1] half spectrum right after it
    const float *kk;     // pseudo-spectral mode: |k|^2 per padded cell (wavenumber)
    int spec_resident;   // pseudo-spectral mode: solves the real array holds (the half
                         // spectrum starts after them)
};

// Per-launch step data.
struct StepArgs {
    int k;        // step within the pass
    int l0, l1, l2;  // ring levels of p0, p1, p2: (k%3, (k+1)%3, (k+2)%3) in a 3-level ring
    int it;       // time index
    int snap;     // snapshot index it/nt_interval, or -1 when it % nt_interval != 0
    float rik;    // Ricker value at it (forward)
};

// StepArgs of step k of a pass over a 3-level ring.
__host__ __device__ __forceinline__ StepArgs ring_step(int k, int it, int snap, float rik)
{
    StepArgs sa;
    sa.k = k;
    sa.l0 = k % 3;
    sa.l1 = (k + 1) % 3;
    sa.l2 = (k + 2) % 3;
    sa.it = it;
    sa.snap = snap;
    sa.rik = rik;
    return sa;
}

enum : int { kStatusOk = 0, kStatusTmaTimeout = 1 };

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }

// One blend of abc_for_p: a 2nd-order one-way extrapolation from the two
// previous levels along the inward direction, weighted by w against the
// current value (fdtd2D_modelling.c:843-849).  p1a..p1c = p1 at 0,1,2 steps
// inward; p0a..p0e = p0 at 0..4 steps inward.  The extrapolation is float;
// the final mix is the double expression w*ext + (1.0-w)*q, reproduced
// exactly by blend_mix.
__device__ __forceinline__ float abc_blend(float q, float t11, float t12, float t13, float p1a,
                                           float p1b, float p1c, float p0a, float p0b, float p0c,
                                           float p0d, float p0e, const BlendCoef &c, int fp32_ok)
{
    const float a2 = fm(2.0f, t11), b2 = fm(2.0f, t12), e2 = fm(2.0f, t13);
    float ext = fa(fa(fm(a2, p1a), fm(b2, p1b)), fm(e2, p1c));
    ext = fs(ext, fm(fm(t11, t11), p0a));
    ext = fs(ext, fm(fm(a2, t12), p0b));
    ext = fs(ext, fm(fa(fm(t12, t12), fm(a2, t13)), p0c));
    ext = fs(ext, fm(fm(b2, t13), p0d));
    ext = fs(ext, fm(fm(t13, t13), p0e));
    // The double mix by one FMA where blend_fma_ok proves it (fwi2d_exact.h),
    // the exact FP32 / FP64 evaluation otherwise.
    const float a = fm(c.w, ext);
    if (blend_fma_ok(a, q, c.khi, c.klo)) return __fmaf_rn(c.bh, q, a);
    return blend_mix(a, q, c, fp32_ok);
}

// Receiver index of padded column ix on the receiver row, or -1.
__device__ __forceinline__ int receiver_of(const Geom &g, int ix)
{
    const int off = ix - g.r_ix0;
    if (g.dr == 0) return off == 0 ? 0 : -1;
    if (off % g.dr) return -1;
    const int ir = off / g.dr;
    return (ir >= 0 && ir < g.nr) ? ir : -1;
}

// Inner velocity at padded cell (iz, ix): get_velp's edge replication
// (fdtd2D_modelling.c:1187-1238) is a clamp of both coordinates.
__device__ __forceinline__ float padded_velocity(const Geom &g, const float *vel, int iz, int ix)
{
    int jz = min(max(iz - g.pml, 0), g.nz - 1);
    int jx = min(max(ix - g.pml, 0), g.nx - 1);
    return vel[(long long)jz * g.nx + jx];
}

// ---------------------------------------------------------------------------
// TMA / mbarrier helpers (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// 3-D tiled TMA load into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y,
                                            int z)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// Bounded wait: true once phase `parity` completed, false after the limit
// (the caller records the timeout and skips its work).
// Programmatic dependent launch: wait for the previous grid on the stream
// (complete, its writes visible), and let the next one be scheduled.  Both
// are no-ops in a launch without the programmatic-serialization attribute.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    for (int i = 0; i < (1 << 24); ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

template <int H>
struct TileShape {
    static constexpr int kP1Rows = kTileZ + 2 * H;   // p1 rows staged
    static constexpr int kP1Floats = kP1Rows * kBoxX;
    static constexpr int kBytes = 4 * kP1Floats;     // TMA bytes per block
    static constexpr int kSmem = kBytes + 16;        // + the mbarrier
};

// Exact two-step quotients (x/d)/d for both Laplacian terms; one range test
// covers the four divisions of a cell, the rest takes div2_any.
__device__ __forceinline__ void laplacian_quotients(float lx, float lz, const Geom &g, float &ddx, float &ddz)
{
    if (g.fast_dx & g.fast_dz & in_fast_range(lx, kDiv2Lo, kDiv2Hi) & in_fast_range(lz, kDiv2Lo, kDiv2Hi)) {
        ddx = div2_fast(lx, g.dx, -g.rdx);
        ddz = div2_fast(lz, g.dz, -g.rdz);
    } else {
        ddx = div2_any(lx, g.dx, g.rdx, g.fast_dx);
        ddz = div2_any(lz, g.dz, g.rdz, g.fast_dz);
    }
}

// Per-warp view of one step: where the warp's 16 x 32 cells live and which
// buffers they read and write.
struct WarpCtx {
    const float *s1;             // staged p1 tile (48 columns x (16 + 2H) rows)
    const float *p0;             // previous-previous level, padded field
    float *p2;                   // new level, padded field
    const float *vdt;            // v*dt, padded field
    float *ps;                   // this column's stored snapshot (interior), or null
    float *G;                    // this column's gradient accumulator (adjoint), or null
    long long c;                 // field offset of the warp's first cell of this lane
    int rr0, iz0, ix, cx, lane;  // first tile row, first padded row, column, staged column, lane
    int inst, sample, shot;
};

// One interior row of a warp whose 32 lanes are all live: the stencil, the
// exact quotients, the new level and the snapshot (forward) or gradient
// term (adjoint).  The exact-quotient range tests are warp votes, so the
// common case is one uniform branch; lanes outside the fast range (zeros
// and tiny tails, which div2_any scales inline) fix their quotients.
template <int H, bool ADJ>
__device__ __forceinline__ void lean_row(const Geom &g, const Batch &b, const float (&win)[2 * H + 1],
                                         const float *srow, float p0c, float vd, float *p2, float *ps, float *G,
                                         float psv, float gv)
{
    const float p1c = win[H];
    float lx = fm(fd_weight<H>(0), p1c);
    float lz = lx;
#pragma unroll
    for (int m = 1; m <= H; ++m) {
        lx = fa(lx, fm(fd_weight<H>(m), fa(srow[m], srow[-m])));
        lz = fa(lz, fm(fd_weight<H>(m), fa(win[H + m], win[H - m])));
    }
    // div2_fast is proved for zero and 2^-80 <= |l| <= 2^80: both second
    // differences within the range, or both zero (a field the wave has not
    // reached); anything else takes div2_any below.
    const float hi = fmaxf(fabsf(lx), fabsf(lz)), lo = fminf(fabsf(lx), fabsf(lz));
    const bool ok = (g.fast_dx & g.fast_dz) && (hi <= kDiv2Hi) && ((lo >= kDiv2Lo) || (hi == 0.0f));
    float ddx = div2_fast(lx, g.dx, -g.rdx);
    float ddz = div2_fast(lz, g.dz, -g.rdz);
    if (!__all_sync(0xffffffffu, ok) && !ok) {
        ddx = div2_any(lx, g.dx, g.rdx, g.fast_dx);
        ddz = div2_any(lz, g.dz, g.rdz, g.fast_dz);
    }
    const float q = fa(fs(fm(2.0f, p1c), p0c), fm(fm(vd, vd), fa(ddx, ddz)));
    *p2 = q;
    if (ps) {
        if (!ADJ) {
            // FWI stores p2 - 2 p1 + p0; the 1/dt^2 of d2p/dt2 is applied once,
            // in FP64, by the gradient reduction.
            *ps = b.imaging ? q : fa(fs(q, fm(2.0f, p1c)), p0c);
        } else {
            *G = fa(gv, fm(psv, q));  // psv = *ps, gv = *G, loaded ahead
        }
    }
}

// Interior sweep: every cell of the warp is inside the interior of the
// padded grid, away from the absorbing strips, the source and the receivers,
// so each row is lean_row without per-cell region tests.  Rows go in blocks
// of U (a variant parameter): the z window covers the block (2H + U values), the
// block's p0 / v*dt rows are fetched one block ahead, and the rows'
// independent dependency chains interleave.
template <int H, bool ADJ, int U>
__device__ __forceinline__ void sweep_interior(const Geom &g, const Batch &b, const StepArgs &sa, const WarpCtx &w,
                                               float p0_first, float vd_first)
{
    static_assert(kWarpRows % U == 0, "row blocks must tile the warp's rows");
    float win[2 * H + U];
#pragma unroll
    for (int m = 0; m < 2 * H; ++m) win[m] = w.s1[(w.rr0 + m) * kBoxX + w.cx];
    const long long pitch = g.pitch;
    const float *p0 = w.p0 + w.c;
    const float *vdt = w.vdt + w.c;
    float *p2 = w.p2 + w.c;
    float *ps = w.ps ? w.ps + (long long)(w.iz0 - g.pml) * g.ipitch : nullptr;
    float *G = w.G ? w.G + (long long)(w.iz0 - g.pml) * g.ipitch : nullptr;
    const float *scol = w.s1 + w.rr0 * kBoxX + w.cx;  // staged row rr0 - H of this column
    float p0n[U], vdn[U];
    p0n[0] = p0_first;
    vdn[0] = vd_first;
#pragma unroll
    for (int u = 1; u < U; ++u) {
        p0n[u] = __ldg(p0 + u * pitch);
        vdn[u] = __ldg(vdt + u * pitch);
    }
#pragma unroll 1
    for (int j0 = 0; j0 < kWarpRows; j0 += U) {
        float p0c[U], vd[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            p0c[u] = p0n[u];
            vd[u] = vdn[u];
            win[2 * H + u] = scol[(j0 + 2 * H + u) * kBoxX];
        }
        if (j0 + U < kWarpRows) {  // fetch the next block's rows (inside the grid: the warp is interior)
#pragma unroll
            for (int u = 0; u < U; ++u) {
                p0n[u] = __ldg(p0 + (j0 + U + u) * pitch);
                vdn[u] = __ldg(vdt + (j0 + U + u) * pitch);
            }
        }
        // Adjoint stored step: this block's snapshot and gradient values,
        // requested before the stencil work that hides their latency.
        float psv[U], gv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            psv[u] = gv[u] = 0.0f;
            if (ADJ && ps) {
                psv[u] = __ldg(ps + (long long)(j0 + u) * g.ipitch);
                gv[u] = G[(long long)(j0 + u) * g.ipitch];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const float(&wu)[2 * H + 1] = *reinterpret_cast<const float(*)[2 * H + 1]>(win + u);
            float *psu = ps ? ps + (long long)(j0 + u) * g.ipitch : nullptr;
            float *Gu = (ADJ && ps) ? G + (long long)(j0 + u) * g.ipitch : nullptr;
            lean_row<H, ADJ>(g, b, wu, scol + (j0 + u + H) * kBoxX, p0c[u], vd[u], p2 + (j0 + u) * pitch, psu, Gu,
                             psv[u], gv[u]);
        }
#pragma unroll
        for (int m = 0; m < 2 * H; ++m) win[m] = win[m + U];
    }
}

// General sweep for warps that touch the rim, an absorbing strip, the
// source row or the receiver row: the same arithmetic with every region
// test of the reference's loops.  (Routing this sweep's interior rows to
// lean_row was measured slower: the second copy of the row body costs more
// in instruction-cache misses and registers than the region tests save.)
template <int H, bool ADJ>
__device__ __forceinline__ void sweep_general(const Geom &g, const Batch &b, const StepArgs &sa, const WarpCtx &w,
                                              float p0_next, float vd_next)
{
    const int ix = w.ix;
    const bool sx = ix >= g.Lc && ix < g.ntx - g.Lc;
    const bool lef = ix >= g.Lc && ix < g.pml;
    const bool rig = ix >= g.ntx - g.pml && ix < g.ntx - g.Lc;
    const int wix = lef ? ix - g.Lc : g.ntx - g.Lc - ix - 1;
    const bool src_col = ix == g.s_ix0 + w.shot * g.ds;
    const int cx = w.cx;
    const float *s1 = w.s1;
    const float *p0 = w.p0;
    const float *vdt = w.vdt;

    float win[2 * H + 1];
#pragma unroll
    for (int m = 0; m < 2 * H + 1; ++m) win[m] = s1[(w.rr0 + m) * kBoxX + cx];

#pragma unroll 1
    for (int j = 0; j < kWarpRows; ++j) {
        const int rr = w.rr0 + j;
        const int iz = w.iz0 + j;
        if (iz >= g.ntz) break;
        const long long c = w.c + (long long)j * g.pitch;
        const float p0c = p0_next;
        const float vd = vd_next;
        if (j + 1 < kWarpRows && iz + 1 < g.ntz) {  // prefetch the next row
            p0_next = __ldg(p0 + c + g.pitch);
            vd_next = __ldg(vdt + c + g.pitch);
        }
        // Adjoint stored step: request the snapshot and gradient values early.
        float psv = 0.0f, gv = 0.0f;
        if (ADJ && w.ps && iz >= g.pml && iz < g.ntz - g.pml) {
            const long long pc = (long long)(iz - g.pml) * g.ipitch;
            psv = __ldg(w.ps + pc);
            gv = w.G[pc];
        }
        const float p1c = win[H];
        const int srow1 = (rr + H) * kBoxX;
        float q = p1c;  // cells the stencil skips keep the previous level
        if (sx && iz >= g.Lc && iz < g.ntz - g.Lc) {
            float lx = fm(fd_weight<H>(0), p1c);
            float lz = lx;
#pragma unroll
            for (int m = 1; m <= H; ++m) {
                lx = fa(lx, fm(fd_weight<H>(m), fa(s1[srow1 + cx + m], s1[srow1 + cx - m])));
                lz = fa(lz, fm(fd_weight<H>(m), fa(win[H + m], win[H - m])));
            }
            float ddx, ddz;
            laplacian_quotients(lx, lz, g, ddx, ddz);
            q = fa(fs(fm(2.0f, p1c), p0c), fm(fm(vd, vd), fa(ddx, ddz)));
        }
        const bool top = iz >= g.Lc && iz < g.pml;
        const bool bot = iz >= g.ntz - g.pml && iz < g.ntz - g.Lc;
        if (top || bot || lef || rig) {
            const float s = div_const(vd, g.dx, g.rdx, g.fast_dx);
            const float t11 = fm(fm(fs(2.0f, s), fs(1.0f, s)), 0.5f);
            const float t12 = fm(s, fs(2.0f, s));
            const float t13 = fm(fm(s, fs(s, 1.0f)), 0.5f);
            if (top || bot) {  // abc_for_p top / bottom passes (fdtd2D_modelling.c:837-867)
                const long long st = top ? g.pitch : -(long long)g.pitch;
                const int wi = top ? iz - g.Lc : g.ntz - g.Lc - iz - 1;
                q = abc_blend(q, t11, t12, t13, p1c, top ? win[H + 1] : win[H - 1], top ? win[H + 2] : win[H - 2],
                              p0c, __ldg(p0 + c + st), __ldg(p0 + c + 2 * st), __ldg(p0 + c + 3 * st),
                              __ldg(p0 + c + 4 * st), b.coef[wi], b.blend_fp32);
            }
            if (lef || rig) {  // left / right passes (:869-899), after top / bottom
                const int d = lef ? 1 : -1;
                q = abc_blend(q, t11, t12, t13, p1c, s1[srow1 + cx + d], s1[srow1 + cx + 2 * d], p0c,
                              __ldg(p0 + c + d), __ldg(p0 + c + 2 * d), __ldg(p0 + c + 3 * d),
                              __ldg(p0 + c + 4 * d), b.coef[wix], b.blend_fp32);
            }
        }
        if (!ADJ) {
            if (iz == g.s_iz && src_col) {  // forward_IO source injection (:910)
                const float v = padded_velocity(g, b.vel + (long long)w.sample * g.nx * g.nz, iz, ix);
                q = fa(q, fm(fm(fm(fm(sa.rik, g.dt), g.dt), v), v));
            }
        } else if (iz == g.r_iz) {  // backward_IO residual injection (:949-959)
            const int ir = receiver_of(g, ix);
            if (ir >= 0) {
                const long long rec = ((long long)w.inst * g.nt + sa.it) * g.nr + ir;
                const float o = b.obs[((long long)w.shot * g.nt + sa.it) * g.nr + ir];
                const float r = b.imaging ? o : fs(b.syn[rec], o);
                const float v = padded_velocity(g, b.vel + (long long)w.sample * g.nx * g.nz, iz, ix);
                q = fa(q, fm(fm(fm(fm(r, g.dt), g.dt), v), v));
            }
        }
        w.p2[c] = q;
        if (!ADJ && iz == g.r_iz) {  // forward_IO receiver sampling (:930-938)
            const int ir = receiver_of(g, ix);
            if (ir >= 0) b.syn[((long long)w.inst * g.nt + sa.it) * g.nr + ir] = q;
        }
        if (w.ps && iz >= g.pml && iz < g.ntz - g.pml) {
            const long long pc = (long long)(iz - g.pml) * g.ipitch;
            if (!ADJ)
                w.ps[pc] = b.imaging ? q : fa(fs(q, fm(2.0f, p1c)), p0c);
            else
                w.G[pc] = fa(gv, fm(psv, q));
        }
        if (j + 1 < kWarpRows) {  // slide the z window one row down
#pragma unroll
            for (int m = 0; m < 2 * H; ++m) win[m] = win[m + 1];
            win[2 * H] = s1[(rr + 1 + 2 * H) * kBoxX + cx];
        }
    }
}

// One time step of every solve in the wave, one block per (resident slot,
// tile).  tm_p1 views the ring as [3*resident][ntz][pitch] with a
// (48, 16+2H) box: the p1 tile and its halo are staged by one TMA load; p0
// and v*dt are read once per cell with coalesced read-only loads (the
// boundary's p0 neighbours hit L1/L2), which keeps shared memory at ~4.6 KB
// per block.  The warp then sweeps its 16 rows with the interior or the
// general row body, a warp-uniform choice.

// One time step of every solve in the wave, one block per (resident slot,
// tile): blockIdx.x = solve, blockIdx.y = tile rank.
template <int H, bool ADJ, int U, int MINB>
__global__ void __launch_bounds__(kThreads, MINB)
    k_step(const __grid_constant__ CUtensorMap tm_p1, const Geom g, const Batch b, const StepArgs sa)
{
    // Dynamic shared memory only (no static __shared__), so the tile starts
    // at the 1024-byte aligned base.
    extern __shared__ __align__(1024) float smem[];
    const CUtensorMap *tile_map = &tm_p1;
    const int solve = blockIdx.x, rank = blockIdx.y;
#include "fwi2d_step_tile.inc"
}

// Fused launches over instances of different geometry (gb_fwi2d_run_instances).
constexpr int kMaxPieces = 16;  // pieces per k_step_multi launch

// One piece: consecutive solves of one instance -- its buffers (the ring and
// stored field of these solves), acquisition and time axis, and where its
// solves and blocks start.
struct PieceArgs {
    const float *vdt, *vel, *obs, *rik;
    float *syn, *ring, *psave, *gacc;
    int s_iz, r_iz, r_ix0, dr, nr, ds, s_ix0, ns, nt, nti, nt_save;
    int inst0;        // its first solve within the instance
    int tm_slot0;     // its first ring slot among the tensor map's fields
    int nres;         // its solves
    int first_block;  // its first block in the launch
};

// Everything a k_step_multi launch reads about its pieces, passed by value
// as the kernel's parameter: the pieces share their grid (every Geom field
// but the acquisition and the time axis) and their rings lie back to back
// under one tensor map.  NP: the pieces it can hold (a launch's parameter
// bytes are part of its fixed cost, so small launches take a small table).
template <int NP>
struct MultiArgsN {
    CUtensorMap tm;
    Geom gc;
    const BlendCoef *coef;
    int *status;
    int blend_fp32, imaging, store, npieces;
    int first[NP + 1];  // first blocks, ascending; first[npieces] = the blocks of all pieces
    PieceArgs piece[NP];
};
using MultiArgs = MultiArgsN<kMaxPieces>;

// One time step k of the first `nact` pieces of a launch (sorted by nt,
// longest first, so the pieces still running at step k are a prefix):
// block -> piece by binary search of first[], then (solve, tile) as in
// k_step.  All of it comes from the parameter space, as k_step's geometry
// and buffers do: the grid's fields stay constant operands of the sweeps and
// a piece's are constant-bank loads, which nothing the kernel stores can
// alias.  Each piece's time index, snapshot index and Ricker value follow
// from its own nt and nt_interval.
template <int H, bool ADJ, int U, int MINB, int NP>
__global__ void __launch_bounds__(kThreads, MINB)
    k_step_multi(const __grid_constant__ MultiArgsN<NP> a, int nact, int k)
{
    extern __shared__ __align__(1024) float smem[];
    int lo = 0, hi = nact - 1;  // the last piece whose first block is <= blockIdx.x
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.first[mid] <= (int)blockIdx.x)
            lo = mid;
        else
            hi = mid - 1;
    }
    const PieceArgs &pc = a.piece[lo];
    Geom g = a.gc;
    g.s_iz = pc.s_iz;
    g.r_iz = pc.r_iz;
    g.r_ix0 = pc.r_ix0;
    g.dr = pc.dr;
    g.nr = pc.nr;
    g.ds = pc.ds;
    g.s_ix0 = pc.s_ix0;
    g.ns = pc.ns;
    g.nt = pc.nt;
    g.nti = pc.nti;
    g.nt_save = pc.nt_save;
    Batch b;
    b.vdt = pc.vdt;
    b.vel = pc.vel;
    b.obs = pc.obs;
    b.syn = pc.syn;
    b.ring = pc.ring;
    b.psave = pc.psave;
    b.gacc = pc.gacc;
    b.coef = a.coef;
    b.blend_fp32 = a.blend_fp32;
    b.status = a.status;
    b.inst0 = pc.inst0;
    b.slot0 = 0;
    b.levels = 3;
    b.tm_slot0 = pc.tm_slot0;
    b.imaging = a.imaging;
    b.store = a.store;
    b.spec = nullptr;
    b.kk = nullptr;
    b.spec_resident = 0;
    const int it = ADJ ? g.nt - 1 - k : k;
    const StepArgs sa = ring_step(k, it, (it % g.nti) == 0 ? it / g.nti : -1, ADJ ? 0.0f : __ldg(pc.rik + it));
    const int local = (int)blockIdx.x - pc.first_block;
    const int rank = local / pc.nres;
    const int solve = local - rank * pc.nres;
    const CUtensorMap *tile_map = &a.tm;
#include "fwi2d_step_tile.inc"
}

}  // namespace gbfwi

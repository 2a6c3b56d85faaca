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
// Data movement: one block owns a 64-column x 64-row tile of one solve.  An
// elected thread stages the previous time level with its stencil halo into
// shared memory with one TMA tensor load completing on an mbarrier; each
// warp then sweeps 16 rows of the 64 columns, two adjacent columns per
// thread, keeping the z-stencil windows in registers, reading x-neighbours
// as 8-byte shared-memory pairs, the level before (p0) and v*dt with
// coalesced 8-byte loads, and writing the new level, the stored snapshot
// (forward) or the gradient accumulator (adjoint) with coalesced 8-byte
// stores.
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

#include "fwi2d_exact.h"

namespace gbfwi {

constexpr int kColsPerThread = 2;  // adjacent columns per thread
constexpr int kTileX = 32 * kColsPerThread;  // columns per tile: one warp wide
constexpr int kWarpRows = 16; // rows each warp sweeps
constexpr int kWarps = 4;     // warps per block, stacked in z
constexpr int kTileZ = kWarpRows * kWarps;  // 64 rows per tile
constexpr int kHaloX = 8;     // x halo of the staged tiles (TMA x offsets stay 16-byte aligned)
constexpr int kBoxX = kTileX + 2 * kHaloX;  // 80 staged columns
constexpr int kThreads = 32 * kWarps;       // 128
constexpr int kAlignX = 32;   // the interior's first column sits on a 128-byte line

// Second-derivative weights of fd_coefficient (fdtd2D_modelling.c:1292-1325)
// for half-width H = Lc-1: the reference's double literals rounded to float,
// as compile-time constants (with m known at compile time they become
// instruction immediates).
template <int H>
__host__ __device__ constexpr float fd_weight(int m)
{
    if (H == 3) {
        return m == 0 ? (float)(-49.0 / 18) : m == 1 ? 1.5f : m == 2 ? (float)(-3.0 / 20) : (float)(1.0 / 90);
    } else if (H == 4) {
        return m == 0 ? (float)(-205.0 / 72) : m == 1 ? (float)(8.0 / 5) : m == 2 ? (float)(-1.0 / 5)
               : m == 3 ? (float)(8.0 / 315) : (float)(-1.0 / 560);
    } else if (H == 5) {
        return m == 0 ? (float)(-73766.0 / 25200) : m == 1 ? (float)(42000.0 / 25200)
               : m == 2 ? (float)(-6000.0 / 25200) : m == 3 ? (float)(1000.0 / 25200)
               : m == 4 ? (float)(-125.0 / 25200) : (float)(8.0 / 25200);
    } else {
        return m == 0 ? (float)(-2.332705821577166e+45 / 7.820582005659452e+44)
               : m == 1 ? (float)(1.3406712009703548e+45 / 7.820582005659452e+44)
               : m == 2 ? (float)(-2.0947987515168676e+44 / 7.820582005659452e+44)
               : m == 3 ? (float)(4.13787407707198e+43 / 7.820582005659452e+44)
               : m == 4 ? (float)(-6.982662505061379e+42 / 7.820582005659452e+44)
               : m == 5 ? (float)(8.12528000589218e+41 / 7.820582005659452e+44)
                        : (float)(-4.702129633040854e+40 / 7.820582005659452e+44);
    }
}

// Geometry shared by every solve of one launch (one parameter set).
struct Geom {
    int ntx, ntz;        // padded grid (fdtd2D_modelling.c:86-87)
    int pitch, xoff;     // row pitch in floats; memory column of padded ix = 0
    int nx, nz, ipitch;  // interior grid and the row pitch of interior arrays
    int pml, Lc, pml0;   // Lc here is the reference's Lc after Lc += 1
    int s_iz, r_iz, r_ix0, dr, nr;
    int ds, s_ix0;       // source column of shot is: s_ix0 + is*ds
    int ns, nt, nti, nt_save;
    int tiles_x, tiles_z;
    int fast_dx, fast_dz, fast_dt;  // the host proved div_const exact for this divisor
    long long fstride;   // floats per padded field (ntz * pitch)
    long long pstride;   // floats per interior snapshot (nz * ipitch)
    float dx, dz, dt;
    float rdx, rdz, rdt; // RN(1/dx), RN(1/dz), RN(1/dt)
    float fd[8];
};

// Where the solves of a wave live.  Solve `inst` = sample * ns + shot.
struct Batch {
    const float *vdt;    // [nsamples][fstride]   padded v*dt per sample
    const float *vel;    // [nsamples][nz*nx]      inner velocity per sample
    const float *obs;    // [ns][nt][nr]
    float *syn;          // [nsamples*ns][nt][nr]
    float *ring;         // [resident][3][fstride]
    float *psave;        // [resident][nt_save][pstride]
    float *gacc;         // [nsamples*ns][pstride]
    const BlendCoef *coef;  // [pml0] boundary weight w, 1 - w split in floats and as double
    int blend_fp32;      // the host proved (1 - w) * q exact in double for every weight
    int *status;         // device error word (0 = ok)
    int inst0;           // first solve of this wave
    int imaging;         // run_fwi == 0
    int store;           // forward pass stores the wavefield for the adjoint
};

// Per-launch step data.
struct StepArgs {
    int k;        // step within the pass: ring buffers (k%3, (k+1)%3, (k+2)%3) = (p0, p1, p2)
    int it;       // time index
    int snap;     // snapshot index it/nt_interval, or -1 when it % nt_interval != 0
    float rik;    // Ricker value at it (forward)
};

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
    return blend_mix(fm(c.w, ext), q, c, fp32_ok);
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
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity)
{
    for (int i = 0; i < (1 << 24); ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}


// Exact two-step quotients (x/d)/d for both Laplacian terms; one range test
// covers the four divisions of a cell, the rare rest takes div_const2.
__device__ __forceinline__ void laplacian_quotients(float lx, float lz, const Geom &g, float &ddx, float &ddz)
{
    if (g.fast_dx & g.fast_dz & in_fast_range(lx, kDiv2Lo, kDiv2Hi) & in_fast_range(lz, kDiv2Lo, kDiv2Hi)) {
        ddx = div_fast(div_fast(lx, g.dx, g.rdx), g.dx, g.rdx);
        ddz = div_fast(div_fast(lz, g.dz, g.rdz), g.dz, g.rdz);
    } else {
        ddx = div_const2(lx, g.dx, g.rdx, g.fast_dx);
        ddz = div_const2(lz, g.dz, g.rdz, g.fast_dz);
    }
}

// Per-thread view of one step: where the thread's two columns of 16 rows
// live and which buffers they read and write.
struct WarpCtx {
    const float *s1;             // staged p1 tile (80 columns x (64 + 2H) rows)
    const float *p0;             // previous-previous level, padded field
    float *p2;                   // new level, padded field
    const float *vdt;            // v*dt, padded field
    float *ps;                   // this thread's stored snapshot (first column), or null
    float *G;                    // this thread's gradient accumulator (adjoint), or null
    long long c;                 // field offset of the thread's first cell
    int rr0, iz0, ix, cx, lane;  // first tile row, first padded row, first column, staged column, lane
    int inst, sample, shot;
};

__device__ __forceinline__ float2 ld2_shared(const float *p) { return *reinterpret_cast<const float2 *>(p); }
__device__ __forceinline__ float2 ld2_global(const float *p) { return __ldg(reinterpret_cast<const float2 *>(p)); }
__device__ __forceinline__ void st2(float *p, float a, float b) { *reinterpret_cast<float2 *>(p) = make_float2(a, b); }

// Laplacian numerator of one cell: fd0*p + sum fd[m]*(p[+m] + p[-m]) per
// axis, accumulated in the reference's order (fdtd2D_modelling.c:768-774).
// xs[H + d] holds the row value at x offset d; z offsets come from win.
template <int H>
__device__ __forceinline__ void laplacian_terms(const float *xs, const float (&win)[2 * H + 1], float &lx, float &lz)
{
    const float p = win[H];
    lx = fm(fd_weight<H>(0), p);
    lz = lx;
#pragma unroll
    for (int m = 1; m <= H; ++m) {
        lx = fa(lx, fm(fd_weight<H>(m), fa(xs[H + m], xs[H - m])));
        lz = fa(lz, fm(fd_weight<H>(m), fa(win[H + m], win[H - m])));
    }
}

// Two interior cells of a row (columns c and c+1), for a warp whose lanes
// are all live and whose cells are all interior: the stencil, the exact
// quotients, the new level and the snapshot (forward) or gradient term
// (adjoint).  The exact-quotient range tests are warp votes, so the common
// case is one uniform branch.
template <int H, bool ADJ>
__device__ __forceinline__ void lean_row2(const Geom &g, const Batch &b, const float (&wa)[2 * H + 1],
                                          const float (&wb)[2 * H + 1], const float *srow, float2 p0c, float2 vd,
                                          float *p2, float *ps, float *G)
{
    constexpr int HP = (H + 1) / 2;  // x pairs on each side
    float xr[2 * (2 * HP + 1)];      // row values at x offsets -2HP .. 2HP+1
#pragma unroll
    for (int k = -HP; k <= HP; ++k) {
        const float2 v = ld2_shared(srow + 2 * k);
        xr[2 * (k + HP)] = v.x;
        xr[2 * (k + HP) + 1] = v.y;
    }
    float lxa, lza, lxb, lzb;
    laplacian_terms<H>(xr + 2 * HP - H, wa, lxa, lza);      // column c: offset d at xr[2HP + d]
    laplacian_terms<H>(xr + 2 * HP + 1 - H, wb, lxb, lzb);  // column c+1
    const bool ok = (g.fast_dx & g.fast_dz) && in_fast_range(lxa, kDiv2Lo, kDiv2Hi) &&
                    in_fast_range(lza, kDiv2Lo, kDiv2Hi) && in_fast_range(lxb, kDiv2Lo, kDiv2Hi) &&
                    in_fast_range(lzb, kDiv2Lo, kDiv2Hi);
    float dxa = div_fast(div_fast(lxa, g.dx, g.rdx), g.dx, g.rdx);
    float dza = div_fast(div_fast(lza, g.dz, g.rdz), g.dz, g.rdz);
    float dxb = div_fast(div_fast(lxb, g.dx, g.rdx), g.dx, g.rdx);
    float dzb = div_fast(div_fast(lzb, g.dz, g.rdz), g.dz, g.rdz);
    if (!__all_sync(0xffffffffu, ok) && !ok) {
        dxa = div_const2(lxa, g.dx, g.rdx, g.fast_dx);
        dza = div_const2(lza, g.dz, g.rdz, g.fast_dz);
        dxb = div_const2(lxb, g.dx, g.rdx, g.fast_dx);
        dzb = div_const2(lzb, g.dz, g.rdz, g.fast_dz);
    }
    const float pa = wa[H], pb = wb[H];
    const float qa = fa(fs(fm(2.0f, pa), p0c.x), fm(fm(vd.x, vd.x), fa(dxa, dza)));
    const float qb = fa(fs(fm(2.0f, pb), p0c.y), fm(fm(vd.y, vd.y), fa(dxb, dzb)));
    st2(p2, qa, qb);
    if (ps) {
        if (!ADJ) {
            float va = qa, vb = qb;
            if (!b.imaging) {
                const float xa = fa(fs(qa, fm(2.0f, pa)), p0c.x);
                const float xb = fa(fs(qb, fm(2.0f, pb)), p0c.y);
                const bool okt = g.fast_dt && in_fast_range(xa, kDiv2Lo, kDiv2Hi) && in_fast_range(xb, kDiv2Lo, kDiv2Hi);
                va = div_fast(div_fast(xa, g.dt, g.rdt), g.dt, g.rdt);
                vb = div_fast(div_fast(xb, g.dt, g.rdt), g.dt, g.rdt);
                if (!__all_sync(0xffffffffu, okt) && !okt) {
                    va = div_const2(xa, g.dt, g.rdt, g.fast_dt);
                    vb = div_const2(xb, g.dt, g.rdt, g.fast_dt);
                }
            }
            st2(ps, va, vb);
        } else {
            const float2 gv = *reinterpret_cast<const float2 *>(G);
            const float2 sv = *reinterpret_cast<const float2 *>(ps);
            st2(G, fa(gv.x, fm(sv.x, qa)), fa(gv.y, fm(sv.y, qb)));
        }
    }
}

// One general cell: every region test of the reference's loops, the
// absorbing-boundary blends, source injection, receiver sampling and
// residual injection.  z-neighbours are read from the staged tile.
template <int H, bool ADJ>
__device__ __forceinline__ void general_cell(const Geom &g, const Batch &b, const StepArgs &sa, const WarpCtx &w,
                                             int iz, int rr, int ix, int cx, long long c, float p0c, float vd)
{
    const float *s1 = w.s1;
    const float *p0 = w.p0;
    const int srow1 = (rr + H) * kBoxX;
    const float p1c = s1[srow1 + cx];
    float q = p1c;  // cells the stencil skips keep the previous level
    if (ix >= g.Lc && ix < g.ntx - g.Lc && iz >= g.Lc && iz < g.ntz - g.Lc) {
        float lx = fm(fd_weight<H>(0), p1c);
        float lz = lx;
#pragma unroll
        for (int m = 1; m <= H; ++m) {
            lx = fa(lx, fm(fd_weight<H>(m), fa(s1[srow1 + cx + m], s1[srow1 + cx - m])));
            lz = fa(lz, fm(fd_weight<H>(m), fa(s1[srow1 + m * kBoxX + cx], s1[srow1 - m * kBoxX + cx])));
        }
        const float ddx = div_const2(lx, g.dx, g.rdx, g.fast_dx);
        const float ddz = div_const2(lz, g.dz, g.rdz, g.fast_dz);
        q = fa(fs(fm(2.0f, p1c), p0c), fm(fm(vd, vd), fa(ddx, ddz)));
    }
    const bool top = iz >= g.Lc && iz < g.pml;
    const bool bot = iz >= g.ntz - g.pml && iz < g.ntz - g.Lc;
    const bool lef = ix >= g.Lc && ix < g.pml;
    const bool rig = ix >= g.ntx - g.pml && ix < g.ntx - g.Lc;
    if (top || bot || lef || rig) {
        const float s = div_const(vd, g.dx, g.rdx, g.fast_dx);
        const float t11 = fm(fm(fs(2.0f, s), fs(1.0f, s)), 0.5f);
        const float t12 = fm(s, fs(2.0f, s));
        const float t13 = fm(fm(s, fs(s, 1.0f)), 0.5f);
        if (top || bot) {  // abc_for_p top / bottom passes (fdtd2D_modelling.c:837-867)
            const int d = top ? 1 : -1;
            const long long st = top ? g.pitch : -(long long)g.pitch;
            const int wi = top ? iz - g.Lc : g.ntz - g.Lc - iz - 1;
            q = abc_blend(q, t11, t12, t13, p1c, s1[srow1 + d * kBoxX + cx], s1[srow1 + 2 * d * kBoxX + cx], p0c,
                          __ldg(p0 + c + st), __ldg(p0 + c + 2 * st), __ldg(p0 + c + 3 * st),
                          __ldg(p0 + c + 4 * st), b.coef[wi], b.blend_fp32);
        }
        if (lef || rig) {  // left / right passes (:869-899), after top / bottom
            const int d = lef ? 1 : -1;
            const int wi = lef ? ix - g.Lc : g.ntx - g.Lc - ix - 1;
            q = abc_blend(q, t11, t12, t13, p1c, s1[srow1 + cx + d], s1[srow1 + cx + 2 * d], p0c,
                          __ldg(p0 + c + d), __ldg(p0 + c + 2 * d), __ldg(p0 + c + 3 * d), __ldg(p0 + c + 4 * d),
                          b.coef[wi], b.blend_fp32);
        }
    }
    if (!ADJ) {
        if (iz == g.s_iz && ix == g.s_ix0 + w.shot * g.ds) {  // forward_IO source injection (:910)
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
    const bool inner = ix >= g.pml && ix < g.ntx - g.pml && iz >= g.pml && iz < g.ntz - g.pml;
    if (inner && sa.snap >= 0 && (ADJ || b.store)) {
        const long long pc = (long long)(iz - g.pml) * g.ipitch + (ix - g.pml);
        float *ps = b.psave + ((long long)blockIdx.y * g.nt_save + sa.snap) * g.pstride + pc;
        if (!ADJ) {
            *ps = b.imaging ? q : div_const2(fa(fs(q, fm(2.0f, p1c)), p0c), g.dt, g.rdt, g.fast_dt);
        } else {
            float *G = b.gacc + (long long)w.inst * g.pstride + pc;
            *G = fa(*G, fm(*ps, q));
        }
    }
}

// Interior sweep: both columns of every lane of the warp are inside the
// interior, away from the absorbing strips, the source and the receivers,
// so each row is lean_row2 without per-cell region tests.  z windows for the
// two columns slide down the staged tile in registers.
template <int H, bool ADJ>
__device__ __forceinline__ void sweep_interior(const Geom &g, const Batch &b, const WarpCtx &w, float2 p0_next,
                                               float2 vd_next)
{
    float wa[2 * H + 1], wb[2 * H + 1];
#pragma unroll
    for (int m = 0; m < 2 * H + 1; ++m) {
        const float2 v = ld2_shared(w.s1 + (w.rr0 + m) * kBoxX + w.cx);
        wa[m] = v.x;
        wb[m] = v.y;
    }
    const float *p0 = w.p0 + w.c;
    const float *vdt = w.vdt + w.c;
    float *p2 = w.p2 + w.c;
    float *ps = w.ps ? w.ps + (long long)(w.iz0 - g.pml) * g.ipitch : nullptr;
    float *G = w.G ? w.G + (long long)(w.iz0 - g.pml) * g.ipitch : nullptr;
    const float *srow = w.s1 + (w.rr0 + H) * kBoxX + w.cx;
#pragma unroll 1
    for (int j = 0; j < kWarpRows; ++j) {
        const float2 p0c = p0_next, vd = vd_next;
        p0 += g.pitch;
        vdt += g.pitch;
        if (j + 1 < kWarpRows) {  // rows stay inside the grid: the warp is interior
            p0_next = ld2_global(p0);
            vd_next = ld2_global(vdt);
        }
        lean_row2<H, ADJ>(g, b, wa, wb, srow, p0c, vd, p2, ps, G);
        p2 += g.pitch;
        if (ps) {
            ps += g.ipitch;
            if (ADJ) G += g.ipitch;
        }
#pragma unroll
        for (int m = 0; m < 2 * H; ++m) {
            wa[m] = wa[m + 1];
            wb[m] = wb[m + 1];
        }
        srow += kBoxX;
        if (j + 1 < kWarpRows) {
            const float2 v = ld2_shared(srow + H * kBoxX);
            wa[2 * H] = v.x;
            wb[2 * H] = v.y;
        }
    }
}

// General sweep for warps that touch the rim, an absorbing strip, the
// source row or the receiver row.  Rows whose cells are all interior (the
// warp's columns are interior and the row is neither the source nor the
// receiver row) still take lean_row2; other rows run general_cell on each
// live column.
template <int H, bool ADJ>
__device__ __forceinline__ void sweep_general(const Geom &g, const Batch &b, const StepArgs &sa, const WarpCtx &w,
                                              bool cols_interior, bool live0, bool live1)
{
#pragma unroll 1
    for (int j = 0; j < kWarpRows; ++j) {
        const int rr = w.rr0 + j;
        const int iz = w.iz0 + j;
        if (iz >= g.ntz) break;
        const long long c = w.c + (long long)j * g.pitch;
        if (cols_interior && iz >= g.pml && iz < g.ntz - g.pml && iz != g.s_iz && iz != g.r_iz) {
            float wa[2 * H + 1], wb[2 * H + 1];
#pragma unroll
            for (int m = 0; m < 2 * H + 1; ++m) {
                const float2 v = ld2_shared(w.s1 + (rr + m) * kBoxX + w.cx);
                wa[m] = v.x;
                wb[m] = v.y;
            }
            float *ps = w.ps ? w.ps + (long long)(iz - g.pml) * g.ipitch : nullptr;
            float *G = w.G ? w.G + (long long)(iz - g.pml) * g.ipitch : nullptr;
            lean_row2<H, ADJ>(g, b, wa, wb, w.s1 + (rr + H) * kBoxX + w.cx, ld2_global(w.p0 + c),
                              ld2_global(w.vdt + c), w.p2 + c, ps, G);
            continue;
        }
        if (live0)
            general_cell<H, ADJ>(g, b, sa, w, iz, rr, w.ix, w.cx, c, __ldg(w.p0 + c), __ldg(w.vdt + c));
        if (live1)
            general_cell<H, ADJ>(g, b, sa, w, iz, rr, w.ix + 1, w.cx + 1, c + 1, __ldg(w.p0 + c + 1),
                                 __ldg(w.vdt + c + 1));
    }
}

template <int H>
struct TileShape {
    static constexpr int kP1Rows = kTileZ + 2 * H;   // p1 rows staged
    static constexpr int kP1Floats = kP1Rows * kBoxX;
    static constexpr int kBytes = 4 * kP1Floats;     // TMA bytes per block
    static constexpr int kSmem = kBytes + 16;        // + the mbarrier
};

// One time step of every solve in the wave.  blockIdx.x = tile, blockIdx.y =
// resident slot.  tm_p1 views the ring as [3*resident][ntz][pitch] with an
// (80, 64+2H) box: the p1 tile and its halo are staged by one TMA load; p0
// and v*dt are read once per cell with coalesced read-only loads (the
// boundary's p0 neighbours hit L1/L2), which keeps shared memory at ~23 KB
// per block.  Each warp then sweeps its 16 rows with the interior or the
// general row body, a warp-uniform choice.
template <int H, bool ADJ>
__global__ void __launch_bounds__(kThreads, 5)
    k_step(const __grid_constant__ CUtensorMap tm_p1, const Geom g, const Batch b, const StepArgs sa)
{
    using TS = TileShape<H>;
    // Dynamic shared memory only (no static __shared__), so the tile starts
    // at the 1024-byte aligned base.
    extern __shared__ __align__(1024) float smem[];
    float *s1 = smem;
    uint64_t &bar = *reinterpret_cast<uint64_t *>(s1 + TS::kP1Floats);

    const int slot = blockIdx.y;
    const int tcol = blockIdx.x % g.tiles_x;
    const int trow = blockIdx.x / g.tiles_x;
    const int col0 = tcol * kTileX;
    const int row0 = trow * kTileZ;
    const int b0 = sa.k % 3, b1 = (sa.k + 1) % 3, b2 = (sa.k + 2) % 3;

    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&bar, TS::kBytes);
        tma_load_3d(s1, &tm_p1, &bar, col0 - kHaloX, row0 - H, slot * 3 + b1);
    }

    WarpCtx w;
    w.inst = b.inst0 + slot;
    w.sample = w.inst / g.ns;
    w.shot = w.inst - w.sample * g.ns;
    w.lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int col = col0 + kColsPerThread * w.lane;
    w.ix = col - g.xoff;
    w.cx = kColsPerThread * w.lane + kHaloX;
    w.rr0 = warp * kWarpRows;
    w.iz0 = row0 + w.rr0;
    w.s1 = s1;
    const bool live0 = w.ix >= 0 && w.ix < g.ntx;
    const bool live1 = w.ix + 1 >= 0 && w.ix + 1 < g.ntx;
    float *ring = b.ring + (long long)slot * 3 * g.fstride;
    w.p0 = ring + (long long)b0 * g.fstride;
    w.p2 = ring + (long long)b2 * g.fstride;
    w.vdt = b.vdt + (long long)w.sample * g.fstride;
    w.c = (long long)w.iz0 * g.pitch + col;

    // Warp-uniform: all 16 rows and 64 columns interior, no source or receiver row.
    const int ix0 = col0 - g.xoff;
    const bool cols_interior = ix0 >= g.pml && ix0 + kTileX <= g.ntx - g.pml;
    const bool interior = cols_interior && w.iz0 >= g.pml && w.iz0 + kWarpRows <= g.ntz - g.pml &&
                          (g.s_iz < w.iz0 || g.s_iz >= w.iz0 + kWarpRows) &&
                          (g.r_iz < w.iz0 || g.r_iz >= w.iz0 + kWarpRows);

    // Interior warps issue their first p0 / v*dt loads while the tile is in flight.
    float2 p0_next = make_float2(0.0f, 0.0f), vd_next = p0_next;
    if (interior) {
        p0_next = ld2_global(w.p0 + w.c);
        vd_next = ld2_global(w.vdt + w.c);
    }

    if (!mbar_wait_bounded(&bar, 0)) {
        if (threadIdx.x == 0) atomicOr(b.status, kStatusTmaTimeout);
        // The copy may still land in this block's shared memory: wait for it
        // a second time (bounded) before the block retires.
        mbar_wait_bounded(&bar, 0);
        return;
    }
    if (!(live0 || live1) || w.iz0 >= g.ntz) return;

    // Snapshot and gradient columns (interior columns only; a pair is either
    // both interior or handled cell by cell in general_cell).
    w.ps = nullptr;
    w.G = nullptr;
    if (sa.snap >= 0 && cols_interior && (ADJ || b.store)) {
        w.ps = b.psave + ((long long)slot * g.nt_save + sa.snap) * g.pstride + (w.ix - g.pml);
        if (ADJ) w.G = b.gacc + (long long)w.inst * g.pstride + (w.ix - g.pml);
    }
    if (interior)
        sweep_interior<H, ADJ>(g, b, w, p0_next, vd_next);
    else
        sweep_general<H, ADJ>(g, b, sa, w, cols_interior, live0, live1);
}

}  // namespace gbfwi

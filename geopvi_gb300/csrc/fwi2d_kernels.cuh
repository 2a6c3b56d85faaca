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
// Arithmetic follows the reference operation by operation: __fmul_rn /
// __fadd_rn / __fsub_rn / __fdiv_rn never contract into FMA, and the
// boundary blend is carried out in double exactly as the C expression
// promotes it.  The forward data therefore match the reference bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gbfwi {

constexpr int kTileX = 32;   // cells per tile along x: one warp
constexpr int kTileZ = 32;   // cells per tile along z
constexpr int kBlockZ = 8;   // threads along z; each owns kTileZ / kBlockZ rows
constexpr int kMaxHalf = 6;  // stencil half-width Lc-1 for Lc = 4..7

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
    long long fstride;   // floats per padded field (ntz * pitch)
    long long pstride;   // floats per interior snapshot (nz * ipitch)
    float dx, dz, dt;
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
    const float *wtab;   // [pml0]   boundary weights w
    const double *omw;   // [pml0]   1 - w in double
    int inst0;           // first solve of this wave
    int imaging;         // run_fwi == 0
    int store;           // forward pass stores the wavefield for the adjoint
};

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fq(float a, float b) { return __fdiv_rn(a, b); }

// One blend of abc_for_p: a 2nd-order one-way extrapolation from the two
// previous levels along the inward direction, weighted by w against the
// current value.  p1a..p1c = p1 at 0,1,2 steps inward; p0a..p0e = p0 at
// 0..4 steps inward.  The final mix is double, as (1.0-w)*p2 promotes it.
__device__ __forceinline__ float abc_blend(float q, float t11, float t12, float t13, float p1a,
                                           float p1b, float p1c, float p0a, float p0b, float p0c,
                                           float p0d, float p0e, float w, double omw)
{
    const float a2 = fm(2.0f, t11), b2 = fm(2.0f, t12), e2 = fm(2.0f, t13);
    float ext = fa(fa(fm(a2, p1a), fm(b2, p1b)), fm(e2, p1c));
    ext = fs(ext, fm(fm(t11, t11), p0a));
    ext = fs(ext, fm(fm(a2, t12), p0b));
    ext = fs(ext, fm(fa(fm(t12, t12), fm(a2, t13)), p0c));
    ext = fs(ext, fm(fm(b2, t13), p0d));
    ext = fs(ext, fm(fm(t13, t13), p0e));
    return __double2float_rn(__dadd_rn((double)fm(w, ext), __dmul_rn(omw, (double)q)));
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

// One time step of every solve in the wave.  blockIdx.x = tile, blockIdx.y =
// resident slot.  `k` counts steps within the current pass (ring position),
// `it` is the time index (forward: k, adjoint: nt-1-k).
template <int H, bool ADJ>
__global__ void __launch_bounds__(kTileX *kBlockZ)
    k_step(const Geom g, const Batch b, int k, int it, float rik_it)
{
    constexpr int SW = kTileX + 2 * H;
    constexpr int SH = kTileZ + 2 * H;
    __shared__ float s1[SH][SW + 1];

    const int slot = blockIdx.y;
    const int inst = b.inst0 + slot;
    const int sample = inst / g.ns;
    const int shot = inst - sample * g.ns;
    const int tile = blockIdx.x;
    const int tcol = tile % g.tiles_x;
    const int trow = tile / g.tiles_x;
    const int col0 = tcol * kTileX;   // memory column
    const int row0 = trow * kTileZ;   // padded row

    float *ring = b.ring + (long long)slot * 3 * g.fstride;
    const float *p0 = ring + (long long)(k % 3) * g.fstride;
    const float *p1 = ring + (long long)((k + 1) % 3) * g.fstride;
    float *p2 = ring + (long long)((k + 2) % 3) * g.fstride;
    const float *vdt = b.vdt + (long long)sample * g.fstride;

    // Stage p1 with a halo of H cells; cells outside the padded grid read 0.
    const int tid = threadIdx.y * kTileX + threadIdx.x;
    for (int e = tid; e < SH * SW; e += kTileX * kBlockZ) {
        const int r = e / SW, c = e - r * SW;
        const int gz = row0 - H + r;
        const int gc = col0 - H + c;
        const int gx = gc - g.xoff;
        float v = 0.0f;
        if (gz >= 0 && gz < g.ntz && gx >= 0 && gx < g.ntx) v = p1[(long long)gz * g.pitch + gc];
        s1[r][c] = v;
    }
    __syncthreads();

    const int tx = threadIdx.x;
    const int col = col0 + tx;
    const int ix = col - g.xoff;
    if (ix < 0 || ix >= g.ntx) return;
    const bool snap = (it % g.nti) == 0;
    const int s_ix = g.s_ix0 + shot * g.ds;

#pragma unroll
    for (int j = 0; j < kTileZ / kBlockZ; ++j) {
        const int rr = threadIdx.y + j * kBlockZ;  // row within tile
        const int iz = row0 + rr;
        if (iz >= g.ntz) break;
        const long long c = (long long)iz * g.pitch + col;
        const int sr = rr + H, sc = tx + H;
        const float p1c = s1[sr][sc];
        const float p0c = p0[c];
        const float vd = vdt[c];
        float q = p1c;  // cells the stencil skips keep the previous level
        if (iz >= g.Lc && iz < g.ntz - g.Lc && ix >= g.Lc && ix < g.ntx - g.Lc) {
            float lx = fm(g.fd[0], p1c);
            float lz = lx;
#pragma unroll
            for (int m = 1; m <= H; ++m) {
                lx = fa(lx, fm(g.fd[m], fa(s1[sr][sc + m], s1[sr][sc - m])));
                lz = fa(lz, fm(g.fd[m], fa(s1[sr + m][sc], s1[sr - m][sc])));
            }
            const float lap = fa(fq(fq(lx, g.dx), g.dx), fq(fq(lz, g.dz), g.dz));
            q = fa(fs(fm(2.0f, p1c), p0c), fm(fm(vd, vd), lap));
        }
        const bool top = iz >= g.Lc && iz < g.pml;
        const bool bot = iz >= g.ntz - g.pml && iz < g.ntz - g.Lc;
        const bool lef = ix >= g.Lc && ix < g.pml;
        const bool rig = ix >= g.ntx - g.pml && ix < g.ntx - g.Lc;
        if (top || bot || lef || rig) {
            const float s = fq(vd, g.dx);
            const float t11 = fm(fm(fs(2.0f, s), fs(1.0f, s)), 0.5f);
            const float t12 = fm(s, fs(2.0f, s));
            const float t13 = fm(fm(s, fs(s, 1.0f)), 0.5f);
            if (top || bot) {
                const int d = top ? 1 : -1;
                const long long st = top ? g.pitch : -(long long)g.pitch;
                const int wi = top ? iz - g.Lc : g.ntz - g.Lc - iz - 1;
                q = abc_blend(q, t11, t12, t13, p1c, s1[sr + d][sc], s1[sr + 2 * d][sc], p0c,
                              p0[c + st], p0[c + 2 * st], p0[c + 3 * st], p0[c + 4 * st],
                              b.wtab[wi], b.omw[wi]);
            }
            if (lef || rig) {
                const int d = lef ? 1 : -1;
                const int wi = lef ? ix - g.Lc : g.ntx - g.Lc - ix - 1;
                q = abc_blend(q, t11, t12, t13, p1c, s1[sr][sc + d], s1[sr][sc + 2 * d], p0c,
                              p0[c + d], p0[c + 2 * d], p0[c + 3 * d], p0[c + 4 * d], b.wtab[wi],
                              b.omw[wi]);
            }
        }
        const long long rec = (long long)inst * g.nt * g.nr + (long long)it * g.nr;
        if (!ADJ) {
            if (iz == g.s_iz && ix == s_ix) {
                const float v = padded_velocity(g, b.vel + (long long)sample * g.nx * g.nz, iz, ix);
                q = fa(q, fm(fm(fm(fm(rik_it, g.dt), g.dt), v), v));
            }
        } else if (iz == g.r_iz) {
            const int ir = receiver_of(g, ix);
            if (ir >= 0) {
                const float o = b.obs[(long long)shot * g.nt * g.nr + (long long)it * g.nr + ir];
                const float r = b.imaging ? o : fs(b.syn[rec + ir], o);
                const float v = padded_velocity(g, b.vel + (long long)sample * g.nx * g.nz, iz, ix);
                q = fa(q, fm(fm(fm(fm(r, g.dt), g.dt), v), v));
            }
        }
        p2[c] = q;
        if (!ADJ && iz == g.r_iz) {
            const int ir = receiver_of(g, ix);
            if (ir >= 0) b.syn[rec + ir] = q;
        }
        const bool inner = iz >= g.pml && iz < g.ntz - g.pml && ix >= g.pml && ix < g.ntx - g.pml;
        if (snap && inner && (ADJ || b.store)) {
            const long long pc = (long long)(iz - g.pml) * g.ipitch + (ix - g.pml);
            float *ps = b.psave + ((long long)slot * g.nt_save + it / g.nti) * g.pstride;
            if (!ADJ) {
                ps[pc] = b.imaging ? q : fq(fq(fa(fs(q, fm(2.0f, p1c)), p0c), g.dt), g.dt);
            } else {
                float *G = b.gacc + (long long)inst * g.pstride;
                G[pc] = fa(G[pc], fm(ps[pc], q));
            }
        }
    }
}

}  // namespace gbfwi

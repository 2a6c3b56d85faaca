// fwi2d_pstd.cuh -- pseudo-spectral Laplacian mode (laplace_solver = 1).
//
// pstd_2d_calculate_p (geopvi/forward/fwi2d/fdtd2D_modelling.c:783-830)
// replaces the FD stencil by a double-precision 2-D DFT of the whole padded
// field: spec = IDFT(-|k|^2 DFT(p1)), and
//   p2 = 2 p1 - p0 + powf(v dt, 2) * re(spec) / (ntx ntz)
// over every cell (the float part in float, the rest in double as the C
// expression promotes it).  The absorbing blends, source or residual
// injection, receivers and the snapshot / gradient term then follow as in
// the FD mode (forward_aco_2D :692-700, backward_aco_2D :732-740).
//
// On the GPU: k_pstd_pack copies p1 of every resident solve into a dense
// [resident][ntz][ntx] real double array; a batched cuFFT D2Z transform
// gives the half spectrum [ntz][ntx/2 + 1] (the input is real, so the
// reference's complex transform's other half is its mirror image and the
// imaginary part of the result is zero); k_pstd_scale multiplies by -|k|^2
// (the wavenumber table of wavenumber() :1127-1184, symmetric under
// k -> -k); a Z2D transform returns the real part; k_step_pstd applies the
// update and the rest of the step per cell.  The transforms dominate; they
// run on the FP64 units, as the reference's FFTW does in double.
#pragma once

#include "fwi2d_kernels.cuh"

namespace gbfwi {

// real[slot][iz][ix] = p1 for the wave's resident solves.
__global__ void k_pstd_pack(const Geom g, const float *__restrict__ ring, int b1, double *__restrict__ real)
{
    const int slot = blockIdx.y;
    const long long n = (long long)g.ntz * g.ntx;
    const float *p1 = ring + ((long long)slot * 3 + b1) * g.fstride;
    double *out = real + (long long)slot * n;
    for (long long d = blockIdx.x * (long long)blockDim.x + threadIdx.x; d < n;
         d += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(d / g.ntx), ix = (int)(d - (long long)iz * g.ntx);
        out[d] = (double)p1[(long long)iz * g.pitch + ix + g.xoff];
    }
}

// half[slot][iz][jx] *= -k[iz][jx], jx <= ntx/2 (k float, the product in
// double: indata = -k[..] * indata).
__global__ void k_pstd_scale(const Geom g, const float *__restrict__ kk, double2 *__restrict__ half)
{
    const int slot = blockIdx.y;
    const int nh = g.ntx / 2 + 1;
    const long long n = (long long)g.ntz * nh;
    double2 *s = half + (long long)slot * n;
    for (long long d = blockIdx.x * (long long)blockDim.x + threadIdx.x; d < n;
         d += (long long)gridDim.x * blockDim.x) {
        const int iz = (int)(d / nh), jx = (int)(d - (long long)iz * nh);
        const double mk = -(double)kk[(long long)iz * g.ntx + jx];
        const double2 v = s[d];
        s[d] = make_double2(__dmul_rn(mk, v.x), __dmul_rn(mk, v.y));
    }
}

// One time step of every resident solve in the pseudo-spectral mode, one
// thread per padded cell: the spectral update, then abc_for_p's blends
// (top / bottom, then left / right) from the previous levels in global
// memory, the injection, receivers and snapshot / gradient term exactly as
// the FD kernel's general sweep does them.
template <bool ADJ>
__global__ void __launch_bounds__(256) k_step_pstd(const Geom g, const Batch b, const StepArgs sa,
                                                   const double *__restrict__ real)
{
    const int slot = blockIdx.y;
    const int inst = b.inst0 + slot;
    const int sample = inst / g.ns, shot = inst - sample * g.ns;
    const long long n = (long long)g.ntz * g.ntx;
    const long long d = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (d >= n) return;
    const int iz = (int)(d / g.ntx), ix = (int)(d - (long long)iz * g.ntx);
    const long long c = (long long)iz * g.pitch + ix + g.xoff;
    const float *ring = b.ring + (long long)slot * 3 * g.fstride;
    const float *p0 = ring + (long long)(sa.k % 3) * g.fstride;
    const float *p1 = ring + (long long)((sa.k + 1) % 3) * g.fstride;
    float *p2 = const_cast<float *>(ring) + (long long)((sa.k + 2) % 3) * g.fstride;
    const float *vdt = b.vdt + (long long)sample * g.fstride;
    const float p1c = p1[c], p0c = p0[c], vd = vdt[c];

    // 2*p1 - p0 + powf(v*dt, 2) * re / (ntx*ntz)
    const double re = real[(long long)slot * n + d];
    const double lap = __ddiv_rn(__dmul_rn((double)fm(vd, vd), re), (double)(g.ntx * g.ntz));
    float q = __double2float_rn(__dadd_rn((double)fs(fm(2.0f, p1c), p0c), lap));

    const bool top = iz >= g.Lc && iz < g.pml;
    const bool bot = iz >= g.ntz - g.pml && iz < g.ntz - g.Lc;
    const bool lef = ix >= g.Lc && ix < g.pml;
    const bool rig = ix >= g.ntx - g.pml && ix < g.ntx - g.Lc;
    if (top || bot || lef || rig) {
        const float s = div_const(vd, g.dx, g.rdx, g.fast_dx);
        const float t11 = fm(fm(fs(2.0f, s), fs(1.0f, s)), 0.5f);
        const float t12 = fm(s, fs(2.0f, s));
        const float t13 = fm(fm(s, fs(s, 1.0f)), 0.5f);
        if (top || bot) {  // abc_for_p top / bottom passes (:837-867)
            const long long st = top ? (long long)g.pitch : -(long long)g.pitch;
            const int wi = top ? iz - g.Lc : g.ntz - g.Lc - iz - 1;
            q = abc_blend(q, t11, t12, t13, p1c, p1[c + st], p1[c + 2 * st], p0c, p0[c + st], p0[c + 2 * st],
                          p0[c + 3 * st], p0[c + 4 * st], b.coef[wi], b.blend_fp32);
        }
        if (lef || rig) {  // left / right passes (:869-899), after top / bottom
            const int dd = lef ? 1 : -1;
            const int wi = lef ? ix - g.Lc : g.ntx - g.Lc - ix - 1;
            q = abc_blend(q, t11, t12, t13, p1c, p1[c + dd], p1[c + 2 * dd], p0c, p0[c + dd], p0[c + 2 * dd],
                          p0[c + 3 * dd], p0[c + 4 * dd], b.coef[wi], b.blend_fp32);
        }
    }
    if (!ADJ) {
        if (iz == g.s_iz && ix == g.s_ix0 + shot * g.ds) {  // forward_IO source injection (:910)
            const float v = padded_velocity(g, b.vel + (long long)sample * g.nx * g.nz, iz, ix);
            q = fa(q, fm(fm(fm(fm(sa.rik, g.dt), g.dt), v), v));
        }
    } else if (iz == g.r_iz) {  // backward_IO residual injection (:949-959)
        const int ir = receiver_of(g, ix);
        if (ir >= 0) {
            const long long rec = ((long long)inst * g.nt + sa.it) * g.nr + ir;
            const float o = b.obs[((long long)shot * g.nt + sa.it) * g.nr + ir];
            const float r = b.imaging ? o : fs(b.syn[rec], o);
            const float v = padded_velocity(g, b.vel + (long long)sample * g.nx * g.nz, iz, ix);
            q = fa(q, fm(fm(fm(fm(r, g.dt), g.dt), v), v));
        }
    }
    p2[c] = q;
    if (!ADJ && iz == g.r_iz) {  // forward_IO receiver sampling (:930-938)
        const int ir = receiver_of(g, ix);
        if (ir >= 0) b.syn[((long long)inst * g.nt + sa.it) * g.nr + ir] = q;
    }
    if (sa.snap >= 0 && (ADJ || b.store) && iz >= g.pml && iz < g.ntz - g.pml && ix >= g.pml &&
        ix < g.ntx - g.pml) {
        const long long pc = ((long long)slot * g.nt_save + sa.snap) * g.pstride + (long long)(iz - g.pml) * g.ipitch +
                             (ix - g.pml + g.ioff);
        if (!ADJ) {
            b.psave[pc] = b.imaging ? q : fa(fs(q, fm(2.0f, p1c)), p0c);  // 1/dt^2 in the reduction
        } else {
            float *G = b.gacc + (long long)inst * g.pstride + (long long)(iz - g.pml) * g.ipitch + (ix - g.pml + g.ioff);
            *G = fa(*G, fm(b.psave[pc], q));
        }
    }
}

}  // namespace gbfwi

// fwi2d_exact.h -- exact FP32 building blocks shared by the kernels and the
// host-side unit tests.
//
// The reference solver (geopvi/forward/fwi2d/fdtd2D_modelling.c) divides by
// the grid constants dx, dz, dt and mixes its absorbing-boundary update in
// double precision.  Reproducing those results bit for bit on a GPU whose
// FP64 rate is a small fraction of its FP32 rate needs two tools:
//
//  * div_const: the correctly rounded quotient x / y for a divisor fixed per
//    launch, in one multiply and two FMAs (Markstein's correction step);
//  * blend_mix: RN_float(RN_double(a + (1 - w) * q)) -- the value the C
//    expression  w*ext + (1.0-w)*p2  produces -- from FP32 error-free
//    transformations, falling back to the double formula only when the FP32
//    evaluation cannot prove its rounding.
//
// Compiled as CUDA device code (nvcc) and as plain C++ (g++ with
// -ffp-contract=off) for the unit tests; GBX_MUL/ADD/SUB/FMA are
// IEEE-exact single operations in both.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define GBX_HD __host__ __device__ __forceinline__
// Rare paths stay out of line so the hot loops keep a small instruction footprint.
#define GBX_COLD __host__ __device__ __noinline__
#else
#define GBX_HD inline
#define GBX_COLD inline
#endif

namespace gbfwi {

#if defined(__CUDA_ARCH__)
GBX_HD float gbx_mul(float a, float b) { return __fmul_rn(a, b); }
GBX_HD float gbx_add(float a, float b) { return __fadd_rn(a, b); }
GBX_HD float gbx_sub(float a, float b) { return __fsub_rn(a, b); }
GBX_HD float gbx_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
GBX_HD float gbx_div(float a, float b) { return __fdiv_rn(a, b); }
GBX_HD double gbx_dmix(float a, double omw, float q)
{
    return __dadd_rn((double)a, __dmul_rn(omw, (double)q));
}
GBX_HD float gbx_d2f(double v) { return __double2float_rn(v); }
GBX_HD uint32_t gbx_bits(float v) { return __float_as_uint(v); }
GBX_HD float gbx_from_bits(uint32_t b) { return __uint_as_float(b); }
#else
// Host: the translation unit must be compiled without FMA contraction.
GBX_HD float gbx_mul(float a, float b) { return a * b; }
GBX_HD float gbx_add(float a, float b) { return a + b; }
GBX_HD float gbx_sub(float a, float b) { return a - b; }
GBX_HD float gbx_fma(float a, float b, float c) { return std::fma(a, b, c); }
GBX_HD float gbx_div(float a, float b) { return a / b; }
GBX_HD double gbx_dmix(float a, double omw, float q) { return (double)a + omw * (double)q; }
GBX_HD float gbx_d2f(double v) { return (float)v; }
GBX_HD uint32_t gbx_bits(float v)
{
    uint32_t b;
    std::memcpy(&b, &v, sizeof b);
    return b;
}
GBX_HD float gbx_from_bits(uint32_t b)
{
    float v;
    std::memcpy(&v, &b, sizeof v);
    return v;
}
#endif

// Magnitudes for which div_fast is proved, given a divisor in [2^-20, 2^20]
// that passed the host's exhaustive binade check: every quotient, remainder
// and corrected quotient stays normal (the remainder's granularity
// ulp(q0)*ulp(y) ~ 2^-46*|x| stays above 2^-149), so the binade [1, 2)
// scales exactly to every |x| in [kDivLo, kDivHi].
constexpr float kDivLo = 0x1p-100f;
constexpr float kDivHi = 0x1p100f;
// (x / y) / y on the fast path: the first quotient stays in [kDivLo, kDivHi].
constexpr float kDiv2Lo = 0x1p-80f;
constexpr float kDiv2Hi = 0x1p80f;

GBX_HD float gbx_copysign(float mag, float sgn)
{
    return gbx_from_bits((gbx_bits(mag) & 0x7FFFFFFFu) | (gbx_bits(sgn) & 0x80000000u));
}

// Markstein's correction step with r = RN(1/y): q0 = RN(x*r) is within an
// ulp of x/y, rem = x - q0*y is exact in one FMA, and RN(q0 + rem*r) is the
// correctly rounded quotient.  For x = +-0 the steps give +0; the sign of
// x/y (y > 0) is the sign of x, so it is copied back, which makes zeros exact
// too.  Valid for x = 0 and kDivLo <= |x| <= kDivHi.
GBX_HD float div_fast(float x, float y, float r)
{
    const float q0 = gbx_mul(x, r);
    const float rem = gbx_fma(-q0, y, x);
    return gbx_copysign(gbx_fma(rem, r, q0), x);
}

// True when v is zero or lo <= |v| <= hi (NaN: false).
GBX_HD bool in_fast_range(float v, float lo, float hi)
{
    const float a = std::fabs(v);
    return (a <= hi) & ((a >= lo) | (a == 0.0f));
}

// x / y correctly rounded for every x (y > 0).  On the proved range: the
// fast path.  Below it (|x| < 2^-100, including subnormals): x * 2^64 is
// exact and lands inside the range, and scaling the quotient back by 2^-64
// is exact whenever the result is normal, |q * 2^-64| >= 2^-126; only
// quotients in the subnormal range, and huge or non-finite x, take IEEE
// division.
GBX_COLD float div_const_slow(float x, float y, float r, int fast)
{
    if (fast && std::fabs(x) < kDivLo) {
        const float qs = div_fast(gbx_mul(x, 0x1p64f), y, r);
        if (std::fabs(qs) >= 0x1p-62f) return gbx_mul(qs, 0x1p-64f);
    }
    return gbx_div(x, y);
}

GBX_HD float div_const(float x, float y, float r, int fast)
{
    if (fast && in_fast_range(x, kDivLo, kDivHi)) return div_fast(x, y, r);
    return div_const_slow(x, y, r, fast);
}

// (x / y) / y correctly rounded at each division.
GBX_COLD float div_const2_slow(float x, float y, float r, int fast)
{
    const float q = (fast && in_fast_range(x, kDivLo, kDivHi)) ? div_fast(x, y, r) : div_const_slow(x, y, r, fast);
    return (fast && in_fast_range(q, kDivLo, kDivHi)) ? div_fast(q, y, r) : div_const_slow(q, y, r, fast);
}

GBX_HD float div_const2(float x, float y, float r, int fast)
{
    if (fast && in_fast_range(x, kDiv2Lo, kDiv2Hi)) return div_fast(div_fast(x, y, r), y, r);
    return div_const2_slow(x, y, r, fast);
}

// Split of 1 - w into floats bh + bl (exact) for the boundary blend, with
// omw = 1 - w in double.  The host precomputes one per boundary weight and
// enables the FP32 path only when (1 - w) * q is exact in double for every
// float q, i.e. 1 - w has at most 29 significant bits.
struct BlendCoef {
    float w;
    float bh, bl;
    double omw;
};

// RN_f(RN_d(a + omw * q)) for a = RN_f(w * ext), computed in FP32.
//   ph + pl = bh*q and qh + ql = bl*q exactly (FMA two-products);
//   s + e = a + ph exactly (two-sum); t ~ e + pl + qh + ql;  r = RN(s + t).
// With T the exact tail and D = X - r the exact distance of the true sum X
// from r: |t - T| <= 3u*S (S = |e|+|pl|+|qh|+|ql|, u = 2^-24); when
// |t| <= |s|/4, s - r is exact (Sterbenz), so d = RN((s - r) + t) is within
// 3u*S + u*|d| of D.  The double rounding moves X by at most 2^-52*|r|.  If
// |d| plus those bounds stays below half an ulp of r (the smaller one when r
// is a power of two), every value between X and RN_d(X) rounds to r, which
// is then the reference's result.  Otherwise -- zeros aside -- the double
// formula is evaluated (rare: near-ties, cancellation, extreme magnitudes).
GBX_COLD float blend_mix_double(float a, float q, double omw) { return gbx_d2f(gbx_dmix(a, omw, q)); }

GBX_HD float blend_mix(float a, float q, const BlendCoef &c, int fp32_ok)
{
    if (q == 0.0f) return gbx_add(a, gbx_mul(c.bh, q));  // a + (+-0), signs as in double
    const float aq = std::fabs(q), aa = std::fabs(a);
    if (fp32_ok && aq >= 0x1p-60f && aq <= 0x1p60f && aa <= 0x1p60f) {
        const float ph = gbx_mul(c.bh, q);
        const float pl = gbx_fma(c.bh, q, -ph);
        const float qh = gbx_mul(c.bl, q);
        const float ql = gbx_fma(c.bl, q, -qh);
        const float s = gbx_add(a, ph);
        const float bv = gbx_sub(s, a);
        const float av = gbx_sub(s, bv);
        const float e = gbx_add(gbx_sub(a, av), gbx_sub(ph, bv));
        const float t = gbx_add(gbx_add(gbx_add(e, pl), qh), ql);
        const float r = gbx_add(s, t);
        const float ar = std::fabs(r);
        if (ar >= 0x1p-90f && ar <= 0x1p90f && std::fabs(t) <= 0.25f * std::fabs(s)) {
            const float d = gbx_add(gbx_sub(s, r), t);
            const float S = gbx_add(gbx_add(std::fabs(e), std::fabs(pl)), gbx_add(std::fabs(qh), std::fabs(ql)));
            const float err = gbx_add(gbx_add(gbx_mul(S, 0x1p-21f), gbx_mul(std::fabs(d), 0x1p-23f)),
                                      gbx_mul(ar, 0x1p-51f));
            const uint32_t rb = gbx_bits(r);
            const uint32_t ex = (rb >> 23) & 0xFFu;
            const uint32_t hu_ex = ex - ((rb & 0x7FFFFFu) ? 24u : 25u);  // half ulp (below, if r = 2^k)
            const float hu = gbx_from_bits(hu_ex << 23);
            if (gbx_add(std::fabs(d), err) < gbx_mul(hu, 0.99f)) return r;
        }
    }
    return blend_mix_double(a, q, c.omw);
}

}  // namespace gbfwi

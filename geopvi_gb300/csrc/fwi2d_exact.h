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

// -(x / y) correctly rounded, from div_fast's three operations with r
// negated (nr = -r): n0 = RN(x*nr) = -q0, RN(n0*y + x) is Markstein's
// remainder, and RN(rem*nr + n0) = -RN(q0 + rem*r) since rounding to nearest
// is symmetric.  For x = +-0 the steps give the zero of the opposite sign,
// which is the negated quotient, so no sign fix-up is needed.
GBX_HD float div_fast_neg(float x, float y, float nr)
{
    const float n0 = gbx_mul(x, nr);
    return gbx_fma(gbx_fma(n0, y, x), nr, n0);
}

// (x / y) / y with both divisions on the fast path: two negated quotients
// give the quotient with its sign (zeros included).  Valid for x = 0 and
// kDiv2Lo <= |x| <= kDiv2Hi.
GBX_HD float div2_fast(float x, float y, float nr) { return div_fast_neg(div_fast_neg(x, y, nr), y, nr); }

// True when v is zero or lo <= |v| <= hi (NaN: false).
GBX_HD bool in_fast_range(float v, float lo, float hi)
{
    const float a = std::fabs(v);
    return (a <= hi) & ((a >= lo) | (a == 0.0f));
}

// The quotient Q = qs + rs / y (y > 0) -- qs = RN(xs / y) normal with
// |qs| < 2^-62, rs = xs - qs*y its exact remainder -- rounded to nearest
// even on the grid G = 2^-85, returned as the float Q * 2^-64 (a subnormal,
// or the smallest normal 2^-126).  With |qs| = m * 2^(e-150) (m the 24-bit
// significand, e the biased exponent <= 64), Q / G = m / 2^s + rs/(y G),
// s = 65 - e >= 1.  The G/2 midpoints lie on qs's own grid, so Q and qs are
// on the same side of every midpoint, and when qs is a midpoint the sign of
// rs tells on which side Q lies (rs = 0: an exact tie, to even).  The
// result's bit pattern is sign | N, N = the rounded multiple of G.
GBX_HD float round_scaled_to_subnormal(float qs, float rs)
{
    const uint32_t b = gbx_bits(qs);
    const uint32_t sign = b & 0x80000000u;
    const int s = 65 - (int)((b >> 23) & 0xFFu);
    if (s > 25) return gbx_from_bits(sign);  // |Q| < G/4: rounds to zero
    const uint32_t m = (b & 0x7FFFFFu) | 0x800000u;
    const uint32_t qint = m >> s, rem = m & ((1u << s) - 1u), half = 1u << (s - 1);
    uint32_t n = qint;
    if (rem > half) {
        n += 1u;
    } else if (rem == half) {
        if (rs == 0.0f)
            n += qint & 1u;
        else if (((gbx_bits(rs) ^ b) & 0x80000000u) == 0u)  // |Q| > |qs|
            n += 1u;
    }
    return gbx_from_bits(sign | n);
}

// x / y correctly rounded for every x (y > 0).  On the proved range: the
// fast path.  Below it (|x| < 2^-100, including subnormals): xs = x * 2^64 is
// exact and lands inside the range; scaling the quotient back by 2^-64 is
// exact whenever the result is normal, |q * 2^-64| >= 2^-126, and a quotient
// in the subnormal range is rounded on the subnormal grid from the scaled
// quotient and its exact remainder.  Only huge or non-finite x (and divisors
// the host could not prove) take IEEE division.
GBX_COLD float div_const_slow(float x, float y, float r, int fast)
{
    if (fast && std::fabs(x) < kDivLo) {
        const float xs = gbx_mul(x, 0x1p64f);
        const float qs = div_fast(xs, y, r);
        if (std::fabs(qs) >= 0x1p-62f) return gbx_mul(qs, 0x1p-64f);
        return round_scaled_to_subnormal(qs, gbx_fma(-qs, y, xs));
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
    if (fast && in_fast_range(x, kDiv2Lo, kDiv2Hi)) return div2_fast(x, y, -r);
    return div_const2_slow(x, y, r, fast);
}

// x / y for 0 < |x| < 2^-80 (y in the proved divisor range), correctly
// rounded including quotients in the subnormal range: xs = x * 2^64 is exact
// and inside div_fast's range; a normal quotient is the scaled one times
// 2^-64 (exact), a subnormal one is rounded on the subnormal grid from the
// scaled quotient and its exact remainder.  nr = -RN(1/y).
GBX_HD float div_tiny(float x, float y, float nr)
{
    const float xs = gbx_mul(x, 0x1p64f);
    const float n = div_fast_neg(xs, y, nr);  // -RN(xs / y)
    if (std::fabs(n) >= 0x1p-62f) return gbx_mul(n, -0x1p-64f);
    return round_scaled_to_subnormal(-n, gbx_fma(n, y, xs));
}

// (x / y) / y for the lanes that miss div2_fast's range, inline for every
// nonzero |x| < 2^-80 (the decaying tails ahead of a wavefront, down to
// subnormals); huge and non-finite x take div_const2's slow path.
GBX_HD float div2_any(float x, float y, float r, int fast)
{
    const float ax = std::fabs(x);
    if (fast && ax < kDiv2Lo && ax != 0.0f) {
        const float nr = -r;
        const float q1 = div_tiny(x, y, nr);
        if (q1 == 0.0f) return q1;  // +-0 / y
        return std::fabs(q1) < kDiv2Lo ? div_tiny(q1, y, nr) : gbx_mul(div_fast_neg(q1, y, nr), -1.0f);
    }
    return div_const2(x, y, r, fast);
}

// Split of 1 - w into floats bh + bl (exact) for the boundary blend, with
// omw = 1 - w in double.  The host precomputes one per boundary weight and
// enables the FP32 path only when (1 - w) * q is exact in double for every
// float q, i.e. 1 - w has at most 29 significant bits.  khi and klo are the
// bounds of blend_fast's one-FMA path (blend_coef_init).
struct BlendCoef {
    float w;
    float bh, bl;
    float khi, klo;
    double omw;
};

#if defined(__CUDA_ARCH__)
GBX_HD uint64_t gbx_dbits(double v) { return (uint64_t)__double_as_longlong(v); }
#else
GBX_HD uint64_t gbx_dbits(double v)
{
    uint64_t b;
    std::memcpy(&b, &v, sizeof b);
    return b;
}
#endif

// 2^k as a float, -126 <= k <= 127.
GBX_HD float gbx_pow2(int k) { return gbx_from_bits((uint32_t)(127 + k) << 23); }

// Boundary weight i of pml0: w = 1 - i/pml0 in double stored as float
// (fdtd2D_modelling.c:227-230), 1 - w in double and as floats bh + bl, and
// the constants of blend_fast.  Every operation is a correctly rounded IEEE
// operation, so host and device produce the same table.
//
// blend_fast's one-FMA path: when bl = 0, omw = bh = B * 2^lam with B odd of
// kb bits.  For normal a, q (a float, q in [2^-60, 2^60]) with biased
// exponents ea, eq, X = a + bh*q is an integer multiple of 2^(min(ea, lam+eq)
// - 150) below 2^(max(ea, kb+lam+eq) - 125), so X is a double whenever
// max(ea, kb+lam+eq) - min(ea, lam+eq) <= 28, i.e. kb - 28 <= ea - eq - lam
// <= 28.  |a| < 2^(28+lam) |q| implies ea - eq <= 28 + lam, and
// |a| >= 2^(kb-28+lam) |q| implies ea - eq >= kb - 28 + lam; a = 0 gives
// X = bh*q (at most 48 bits).  X a double means RN_d(X) = X, so the
// reference's RN_f(RN_d(X)) is RN_f(X): one FMA.  khi = 2^(28+lam) and
// klo = 2^(kb-28+lam); bh = 0 (w = 1) always qualifies (khi = inf, klo = 0);
// weights with bl != 0 never do (khi = 0).
GBX_HD void blend_coef_init(BlendCoef &c, int i, int pml0)
{
    c.w = (float)(1.0 - 1.0 * i / pml0);
    c.omw = 1.0 - (double)c.w;
    c.bh = (float)c.omw;
    c.bl = (float)(c.omw - (double)c.bh);
    c.khi = 0.0f;
    c.klo = 0.0f;
    if (c.omw == 0.0) {
        c.khi = gbx_from_bits(0x7F800000u);  // +inf
    } else if (c.bl == 0.0f) {
        const uint64_t b = gbx_dbits(c.omw);
        const int e = (int)((b >> 52) & 0x7FF);  // omw is a normal double in (0, 1]
        uint64_t m = (b & ((1ull << 52) - 1)) | (1ull << 52);
        int lam = e - 1075;
        while (!(m & 1u)) {
            m >>= 1;
            ++lam;
        }
        int kb = 0;
        while (m) {
            m >>= 1;
            ++kb;
        }
        c.khi = gbx_pow2(28 + lam);
        c.klo = gbx_pow2(kb - 28 + lam);
    }
}

// RN_f(RN_d(a + omw * q)) for a = RN_f(w * ext), computed in FP32.
//   ph + pl = bh*q and qh + ql = bl*q exactly (FMA two-products);
//   s + e = a + ph exactly (two-sum); t ~ e + pl + qh + ql;  r = RN(s + t).
// With T the exact tail and D = X - r the exact distance of the true sum X
// from r: |t - T| <= 3u*S (S = |e|+|pl|+|qh|+|ql|, u = 2^-24); when
// |t| <= |s|/4, s - r is exact (Sterbenz), so d = RN((s - r) + t) is within
// 3u*S + u*|d| of D.  The double rounding moves X by at most 2^-52*|r|.  If
// |d| plus those bounds stays below half an ulp of r (the smaller one when r
// is a power of two) -- tested against hu * (1 - 2^-16), which absorbs the
// rounding of the test's own three additions -- every value between X and
// RN_d(X) rounds to r, which is then the reference's result.  Otherwise --
// zeros aside -- the double formula is evaluated (rare: X within ~2^-16 of a
// half ulp from a midpoint, cancellation, extreme magnitudes).
GBX_COLD float blend_mix_double(float a, float q, double omw) { return gbx_d2f(gbx_dmix(a, omw, q)); }

// The FP32 evaluation below for 2^-60 <= |q| <= 2^60, |a| <= 2^60: true and
// the result in *out when its rounding is proved, false otherwise.
GBX_HD bool blend_mix_fp32(float a, float q, const BlendCoef &c, float *out)
{
    {
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
            if (gbx_add(std::fabs(d), err) < gbx_mul(hu, 0x1.fffep-1f)) {  // hu * (1 - 2^-16)
                *out = r;
                return true;
            }
            // Exact ties.  When 1 - w has few significant bits (w = 0.5, 0.75,
            // ...), X often sits exactly on the midpoint M = r + sign(d)*hu.
            // With bl*q = 0, X = a + ph + pl exactly and X - M = e + pl + k,
            // k = (s - r) - sign(d)*hu exact (r is s or a neighbour of s when
            // |t| <= 2^-20 |s|, so k is a sum of two nearby powers of two).
            // Two-sums decide whether that is zero; an exact midpoint is a
            // double, so the reference rounds it half to even.
            if (qh == 0.0f && ql == 0.0f && std::fabs(t) <= gbx_mul(0x1p-20f, std::fabs(s))) {
                const float k = gbx_sub(gbx_sub(s, r), d > 0.0f ? hu : -hu);
                const float u = gbx_add(e, pl);
                const float ub = gbx_sub(u, e), ue = gbx_add(gbx_sub(e, gbx_sub(u, ub)), gbx_sub(pl, ub));
                const float v = gbx_add(u, k);
                const float vb = gbx_sub(v, u), ve = gbx_add(gbx_sub(u, gbx_sub(v, vb)), gbx_sub(k, vb));
                if (ve == 0.0f && v == -ue) {
                    if ((rb & 1u) == 0u) {
                        *out = r;  // r is the even neighbour
                    } else {       // the neighbour of r toward X
                        const bool grows = (d > 0.0f) == (r > 0.0f);
                        *out = gbx_from_bits(grows ? rb + 1u : rb - 1u);
                    }
                    return true;
                }
            }
        }
    }
    return false;
}

GBX_HD float blend_mix(float a, float q, const BlendCoef &c, int fp32_ok);

// True when blend_fast's one-FMA path gives the reference's value (see
// blend_coef_init); q = 0 always qualifies (X = a exactly).
GBX_HD bool blend_fma_ok(float a, float q, float khi, float klo)
{
    const float aq = std::fabs(q), aa = std::fabs(a);
    return (q == 0.0f) |
           ((aq >= 0x1p-60f) & (aq <= 0x1p60f) & (aa < gbx_mul(aq, khi)) & ((aa >= gbx_mul(aq, klo)) | (a == 0.0f)));
}

// blend_mix by reference to a table entry, out of line: the kernels' rare path.
GBX_COLD float blend_mix_at(float a, float q, const BlendCoef *c, int fp32_ok) { return blend_mix(a, q, *c, fp32_ok); }

// RN_f(RN_d(a + (1 - w) q)): one FMA where blend_fma_ok proves it, blend_mix
// otherwise.  bh, khi, klo are the entry's fields, held in registers by the caller.
GBX_HD float blend_fast(float a, float q, float bh, float khi, float klo, const BlendCoef *c, int fp32_ok)
{
    if (blend_fma_ok(a, q, khi, klo)) return gbx_fma(bh, q, a);
    return blend_mix_at(a, q, c, fp32_ok);
}

GBX_HD float blend_mix(float a, float q, const BlendCoef &c, int fp32_ok)
{
    if (q == 0.0f) return gbx_add(a, gbx_mul(c.bh, q));  // a + (+-0), signs as in double
    // Tiny operands (|q| < 2^-60, |a| < 2^-40: the tails ahead of a
    // wavefront) are scaled by 2^100 first.  a * 2^100 and q * 2^100 are exact
    // and inside the FP32 evaluation's range, and RN_f(RN_d(X * 2^100)) =
    // RN_f(RN_d(X)) * 2^100 whenever the unscaled result is normal (|r| >=
    // 2^-26 scaled), so scaling back is exact.  Subnormal results, and
    // anything else unproved, take the double formula.
    const bool tiny = std::fabs(q) < 0x1p-60f && std::fabs(a) < 0x1p-40f;
    const float up = tiny ? 0x1p100f : 1.0f, lo = tiny ? 0x1p-26f : 0.0f;
    const float as = gbx_mul(a, up), qs = gbx_mul(q, up);
    const float aq = std::fabs(qs);
    float r;
    if (fp32_ok && aq >= 0x1p-60f && aq <= 0x1p60f && std::fabs(as) <= 0x1p60f && blend_mix_fp32(as, qs, c, &r) &&
        std::fabs(r) >= lo)
        return gbx_mul(r, tiny ? 0x1p-100f : 1.0f);
    return blend_mix_double(a, q, c.omw);
}

}  // namespace gbfwi

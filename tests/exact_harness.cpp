// Host-side harness for the exact FP32 helpers of the GPU kernels
// (geopvi_gb300/csrc/fwi2d_exact.h).  Built by tests/test_exact_math.py with
// g++ -ffp-contract=off; every helper is compared with the arithmetic it
// must reproduce: IEEE float division and the reference's double-precision
// boundary mix  (float)((double)a + (1.0 - w) * (double)q).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>

#include "../geopvi_gb300/csrc/fwi2d_exact.h"

using namespace gbfwi;

extern "C" {

// Number of x (all significands of [1,2) times 2^k for k in [klo, khi]) where
// div_const differs from x / y.
long long harness_div_mismatches(float y, int klo, int khi)
{
    const float r = 1.0f / y;
    long long bad = 0;
    for (int k = klo; k <= khi; ++k)
        for (uint32_t m = 0; m < (1u << 23); m += 97) {
            const uint32_t bits = ((uint32_t)(127 + k) << 23) | m;
            float x;
            std::memcpy(&x, &bits, 4);
            for (float xs : {x, -x}) {
                if (div_const(xs, y, r, 1) != xs / y) ++bad;
                if (div_const2(xs, y, r, 1) != (xs / y) / y) ++bad;
            }
        }
    // zeros keep their sign; subnormals and huge values take the slow path
    // tiny magnitudes: every significand of binades near and below 2^-100
    for (int k = -126; k <= -100; k += 2)
        for (uint32_t m = 0; m < (1u << 23); m += 61) {
            const uint32_t bits = ((uint32_t)(127 + k) << 23) | m;
            float x;
            std::memcpy(&x, &bits, 4);
            for (float xs : {x, -x}) {
                const float a = div_const(xs, y, r, 1), b = xs / y;
                const float a2 = div_const2(xs, y, r, 1), b2 = (xs / y) / y;
                if (std::memcmp(&a, &b, 4) != 0) ++bad;
                if (std::memcmp(&a2, &b2, 4) != 0) ++bad;
            }
        }
    for (uint32_t sub = 1; sub < (1u << 23); sub += 37) {  // subnormals
        float x;
        std::memcpy(&x, &sub, 4);
        const float a = div_const(x, y, r, 1), b = x / y;
        if (std::memcmp(&a, &b, 4) != 0) ++bad;
    }
    for (float xs : {0.0f, -0.0f, 1e-40f, -3e-39f, 1e-31f, 1e30f, 3e38f}) {
        const float a = div_const(xs, y, r, 1), b = xs / y;
        const float a2 = div_const2(xs, y, r, 1), b2 = (xs / y) / y;
        if (std::memcmp(&a, &b, 4) != 0) ++bad;
        if (std::memcmp(&a2, &b2, 4) != 0) ++bad;
    }
    return bad;
}

// Every significand of the binades 2^k, k in [klo, khi], through div_fast
// directly (the proof's range ends), both signs.
long long harness_div_fast_binades(float y, int klo, int khi)
{
    const float r = 1.0f / y;
    long long bad = 0;
    for (int k = klo; k <= khi; ++k)
        for (uint32_t m = 0; m < (1u << 23); ++m) {
            const uint32_t bits = ((uint32_t)(127 + k) << 23) | m;
            float x;
            std::memcpy(&x, &bits, 4);
            if (div_fast(x, y, r) != x / y) ++bad;
            if (div_fast(-x, y, r) != -x / y) ++bad;
        }
    return bad;
}

// div2_any against (x / y) / y bit for bit: every 7th significand of each
// binade from the subnormals up to 2^-79 and of a few normal binades, both
// signs, plus zeros, every 37th subnormal and huge values.
long long harness_div2_any(float y)
{
    const float r = 1.0f / y;
    long long bad = 0;
    auto check = [&](float x) {
        const float a = div2_any(x, y, r, 1), b = (x / y) / y;
        if (std::memcmp(&a, &b, 4) != 0) ++bad;
    };
    for (int k = -126; k <= -79; ++k)
        for (uint32_t m = 0; m < (1u << 23); m += 7) {
            const uint32_t bits = ((uint32_t)(127 + k) << 23) | m;
            float x;
            std::memcpy(&x, &bits, 4);
            check(x);
            check(-x);
        }
    for (uint32_t sub = 1; sub < (1u << 23); sub += 37) {
        float x;
        std::memcpy(&x, &sub, 4);
        check(x);
        check(-x);
    }
    for (float x : {0.0f, -0.0f, 1.0f, -3.5f, 1e30f, -3e38f, 0x1p81f})
        check(x);
    return bad;
}

// div2_fast (two negated quotients, no sign fix-up) against (x / y) / y bit
// for bit, every significand of the binades 2^k, k in [klo, khi], both
// signs, and both zeros.
long long harness_div2_fast_binades(float y, int klo, int khi)
{
    const float nr = -(1.0f / y);
    long long bad = 0;
    auto check = [&](float x) {
        const float a = div2_fast(x, y, nr), b = (x / y) / y;
        if (std::memcmp(&a, &b, 4) != 0) ++bad;
    };
    for (int k = klo; k <= khi; ++k)
        for (uint32_t m = 0; m < (1u << 23); ++m) {
            const uint32_t bits = ((uint32_t)(127 + k) << 23) | m;
            float x;
            std::memcpy(&x, &bits, 4);
            check(x);
            check(-x);
        }
    check(0.0f);
    check(-0.0f);
    return bad;
}

static float ref_mix(float a, double omw, float q) { return (float)((double)a + omw * (double)q); }

// Ties: operands with short significands, so that a + (1 - w) * q often
// lands exactly on a float midpoint (weights 1/2, 3/4, 1/4, ... of pml0 = 4,
// 8, 20).  Returns mismatches against the double formula; *fp32 counts the
// trials the FP32 evaluation settled itself.
long long harness_blend_ties(int pml0, long long trials, unsigned seed, long long *fp32)
{
    std::mt19937_64 rng(seed);
    std::uniform_int_distribution<int> M(-(1 << 20), 1 << 20), E(-30, 10), B(20, 24);
    long long bad = 0, ok32 = 0;
    for (int i = 0; i < pml0; ++i) {
        BlendCoef c;
        c.w = (float)(1.0 - 1.0 * i / pml0);
        c.omw = 1.0 - (double)c.w;
        c.bh = (float)c.omw;
        c.bl = (float)(c.omw - (double)c.bh);
        for (long long t = 0; t < trials; ++t) {
            const int e = E(rng);
            const float q = std::ldexp((float)(M(rng) | 1) * (float)(1 << (24 - B(rng))), e - 20);
            const float ext = std::ldexp((float)M(rng), e - 20 + (int)(t % 3) - 1);
            const float a = c.w * ext;
            float r32;
            if (q != 0.0f && blend_mix_fp32(a, q, c, &r32)) ++ok32;
            const float got = blend_mix(a, q, c, 1);
            const float want = ref_mix(a, c.omw, q);
            if (std::memcmp(&got, &want, 4) != 0) ++bad;
        }
    }
    *fp32 = ok32;
    return bad;
}

// Random and adversarial trials of blend_mix against the double formula.
// Returns the number of bitwise mismatches; *fallbacks counts trials that took
// the double path.
long long harness_blend_mismatches(int pml0, long long trials, unsigned seed, long long *fallbacks)
{
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    std::uniform_int_distribution<int> E(-40, 40);
    long long bad = 0, fb = 0;
    for (int i = 0; i < pml0; ++i) {
        BlendCoef c;
        c.w = (float)(1.0 - 1.0 * i / pml0);
        c.omw = 1.0 - (double)c.w;
        c.bh = (float)c.omw;
        c.bl = (float)(c.omw - (double)c.bh);
        const bool ok = ((double)c.bh + (double)c.bl) == c.omw;
        for (long long t = 0; t < trials; ++t) {
            float q = (float)(U(rng) * std::ldexp(1.0, E(rng)));
            float ext = (float)(U(rng) * std::ldexp(1.0, E(rng) / 8));
            if (t % 4 == 1) ext = (float)(-(c.omw * q) / (c.w > 0 ? c.w : 1.0f) * (1.0 + 1e-6 * U(rng)));  // cancellation
            if (t % 4 == 2) q = std::nextafter(q, 0.0f);
            if (t % 97 == 3) q = 0.0f;
            if (t % 89 == 4) q = -0.0f;
            if (t % 83 == 5) ext = 0.0f;
            if (t % 79 == 6) q = 1e-41f;  // subnormal
            if (t % 7 == 5) {  // tiny tails: the scaled FP32 path
                q = std::ldexp(q, -95);
                ext = std::ldexp(ext, -95);
            }
            if (t % 13 == 9) {  // results near and below the normal range
                q = std::ldexp(q, -118);
                ext = std::ldexp(ext, -118);
            }
            const float a = c.w * ext;
            // near-tie construction: choose q so that a + omw*q sits near a float midpoint
            if (t % 4 == 3 && c.omw > 0) {
                const float target = (float)(U(rng) * 4.0);
                const float next = std::nextafter(target, 10.0f);
                const double mid = 0.5 * ((double)target + (double)next);
                q = (float)((mid - (double)a) / c.omw);
            }
            const float got = blend_mix(a, q, c, ok ? 1 : 0);
            const float want = ref_mix(a, c.omw, q);
            if (std::memcmp(&got, &want, 4) != 0) ++bad;
            // count the double fallbacks the same way the kernel takes them
            const float aq = std::fabs(q);
            if (q != 0.0f && !(aq >= 0x1p-60f && aq <= 0x1p60f)) ++fb;
        }
    }
    if (fallbacks) *fallbacks = fb;
    return bad;
}

// blend_fast (one FMA where its exponent test proves the result, blend_mix
// otherwise) against the double formula, on realistic blends (a near w*q),
// cancellation, near-midpoint sums, zeros, tiny, huge and subnormal operands.
// Returns mismatches; *fast counts the trials the FMA path settled.
long long harness_blend_fast(int pml0, long long trials, unsigned seed, long long *fast)
{
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    std::uniform_int_distribution<int> E(-70, 70);
    long long bad = 0, nfast = 0;
    for (int i = 0; i < pml0; ++i) {
        BlendCoef c;
        blend_coef_init(c, i, pml0);
        const bool ok = ((double)c.bh + (double)c.bl) == c.omw;
        for (long long t = 0; t < trials; ++t) {
            float q = (float)(U(rng) * std::ldexp(1.0, E(rng)));
            float ext = q * (float)(1.0 + 0.3 * U(rng));  // smooth field: extrapolation near the value
            switch (t % 11) {
            case 1: ext = (float)(U(rng) * std::ldexp(1.0, E(rng))); break;   // unrelated magnitudes
            case 2: ext = (float)(-(c.omw * q) / (c.w > 0 ? c.w : 1.0f) * (1.0 + 1e-7 * U(rng))); break;  // cancellation
            case 3: q = 0.0f; break;
            case 4: ext = 0.0f; break;
            case 5: q = std::ldexp(q, -80); ext = std::ldexp(ext, -80); break;  // tails
            case 6: q = 1e-41f * (float)U(rng); break;  // subnormal
            case 7: q = std::ldexp(q, 55); ext = std::ldexp(ext, 60); break;  // huge
            default: break;
            }
            const float a = c.w * ext;
            if (t % 11 == 8 && c.omw > 0) {  // sum near a float midpoint
                const float target = (float)(U(rng) * 4.0);
                const double mid = 0.5 * ((double)target + (double)std::nextafter(target, 10.0f));
                q = (float)((mid - (double)a) / c.omw);
            }
            if (blend_fma_ok(a, q, c.khi, c.klo)) ++nfast;
            const float got = blend_fast(a, q, c.bh, c.khi, c.klo, &c, ok ? 1 : 0);
            const float want = ref_mix(a, c.omw, q);
            if (std::memcmp(&got, &want, 4) != 0) ++bad;
        }
    }
    if (fast) *fast = nfast;
    return bad;
}

}  // extern "C"

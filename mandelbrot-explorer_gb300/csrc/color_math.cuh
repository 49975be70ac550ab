// Correctly rounded single-precision log and pow for the colour epilogue,
// computed in pairs of floats (hi + lo, ~48-bit significand) on the FP32 pipe.
//
// The reference's palette coordinate powf(logf(v+2), logf(v+2)^2*d/3600)
// (src/tools/render.cpp:31-33) is a float; at deep zooms v reaches 1e4..1e6 and
// the coordinate times 2048 reaches 2^15..2^23, so a one-ulp difference in
// either function moves a sample to the neighbouring palette entry. Both libm
// functions it calls are correctly rounded on all but a few inputs in 10^4, so
// the epilogue computes the exact rounding: a pair-of-floats evaluation with a
// known error bound, and, when the pair lies within that bound of a rounding
// midpoint (about one sample in 10^5), the FP64 library functions.
//
// Methods (all standard): error-free sum and product of floats (Knuth's
// TwoSum, Dekker's FastTwoSum, the FMA product error), pair-of-floats
// arithmetic after Dekker (1971); log via m = x / 2^k in [1/sqrt2, sqrt2] and
// the series log m = 2 atanh(s), s = (m-1)/(m+1); exp via Tang's table method
// (1989): y = (32k + j) ln2/32 + r, e^y = 2^k 2^(j/32) e^r, |r| <= ln2/64,
// with e^r by its Taylor series.
//
// The same header compiles for the host (g++ with -ffp-contract=off, std::fmaf)
// and the device (explicit round-to-nearest intrinsics that the compiler never
// contracts), so both execute the identical sequence of IEEE operations and the
// host build can check the error bounds exhaustively.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define CM_HD __host__ __device__ __forceinline__
#else
#define CM_HD inline
#endif

namespace mbx {
namespace cm {

#if defined(__CUDA_ARCH__)
CM_HD float add(float a, float b) { return __fadd_rn(a, b); }
CM_HD float sub(float a, float b) { return __fsub_rn(a, b); }
CM_HD float mul(float a, float b) { return __fmul_rn(a, b); }
CM_HD float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
CM_HD float div(float a, float b) { return __fdiv_rn(a, b); }
CM_HD uint32_t bits(float x) { return __float_as_uint(x); }
CM_HD float from_bits(uint32_t u) { return __uint_as_float(u); }
#else
CM_HD float add(float a, float b) { return a + b; }
CM_HD float sub(float a, float b) { return a - b; }
CM_HD float mul(float a, float b) { return a * b; }
CM_HD float fma(float a, float b, float c) { return std::fmaf(a, b, c); }
CM_HD float div(float a, float b) { return a / b; }
CM_HD uint32_t bits(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
}
CM_HD float from_bits(uint32_t u) {
    float x;
    memcpy(&x, &u, 4);
    return x;
}
#endif

struct ff {
    float hi, lo;
};

CM_HD ff two_sum(float a, float b) {
    const float s = add(a, b);
    const float bb = sub(s, a);
    return {s, add(sub(a, sub(s, bb)), sub(b, bb))};
}
CM_HD ff fast_two_sum(float a, float b) { // |a| >= |b| or a == 0
    const float s = add(a, b);
    return {s, sub(b, sub(s, a))};
}
CM_HD ff ff_add(ff x, ff y) {
    const ff s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, add(s.lo, add(x.lo, y.lo)));
}
CM_HD ff ff_add_f(ff x, float y) {
    const ff s = two_sum(x.hi, y);
    return fast_two_sum(s.hi, add(s.lo, x.lo));
}
CM_HD ff ff_mul(ff x, ff y) {
    const float p = mul(x.hi, y.hi);
    float e = fma(x.hi, y.hi, -p);
    e = fma(x.hi, y.lo, e);
    e = fma(x.lo, y.hi, e);
    return fast_two_sum(p, e);
}
CM_HD ff ff_mul_f(ff x, float y) {
    const float p = mul(x.hi, y);
    const float e = fma(x.lo, y, fma(x.hi, y, -p));
    return fast_two_sum(p, e);
}
// x / y with two correction steps of the float quotient.
CM_HD ff ff_div(ff x, ff y) {
    const float q1 = div(x.hi, y.hi);
    ff r = ff_add(x, ff_mul_f(y, -q1));
    const float q2 = div(r.hi, y.hi);
    r = ff_add(r, ff_mul_f(y, -q2));
    const float q3 = div(r.hi, y.hi);
    const ff q = fast_two_sum(q1, q2);
    return ff_add_f(q, q3);
}

// ln 2 and ln 2 / 32 as pairs (hi = RN(v), lo = RN(v - hi)); 1/3, 1/5, 1/7 likewise.
constexpr float kLn2Hi = 0x1.62e430p-1f, kLn2Lo = -0x1.05c610p-29f;
constexpr float kLn2_32Hi = 0x1.62e430p-6f, kLn2_32Lo = -0x1.05c610p-34f;
constexpr float kThirdHi = 0x1.555556p-2f, kThirdLo = -0x1.555556p-27f;
constexpr float kFifthHi = 0x1.99999ap-3f, kFifthLo = -0x1.99999ap-29f;
constexpr float kSeventhHi = 0x1.24924ap-3f, kSeventhLo = -0x1.b6db6ep-28f;

// Natural log of a positive normal float; relative error below 2^-45 over the
// colour epilogue's ranges (checked by the host build in the tests).
CM_HD ff log_ff(float x) {
    const uint32_t u = bits(x);
    int k = (int)((u >> 23) & 0xff) - 127;
    float m = from_bits((u & 0x007fffffu) | 0x3f800000u); // [1, 2)
    if (m > 1.41421356f) {
        m = mul(m, 0.5f);
        k += 1;
    }
    const float f = sub(m, 1.0f); // exact (Sterbenz)
    const ff s = ff_div(ff{f, 0.0f}, two_sum(m, 1.0f));
    const ff s2 = ff_mul(s, s);
    const float t = s2.hi;
    // Q(t) = 1/3 + t/5 + t^2/7 + ... + t^7/17, leading three terms in pairs
    // (the float tail's rounding reaches log m scaled by t^3 <= 2^-15)
    float r3 = fma(t, 1.0f / 17.0f, 1.0f / 15.0f);
    r3 = fma(t, r3, 1.0f / 13.0f);
    r3 = fma(t, r3, 1.0f / 11.0f);
    r3 = fma(t, r3, 1.0f / 9.0f);
    const ff r2 = ff_add(ff{kSeventhHi, kSeventhLo}, ff_mul_f(s2, r3));
    const ff r = ff_add(ff{kFifthHi, kFifthLo}, ff_mul(s2, r2));
    const ff q = ff_add(ff{kThirdHi, kThirdLo}, ff_mul(s2, r));
    ff lm = ff_add(s, ff_mul(s, ff_mul(s2, q))); // atanh(s)
    lm = ff{mul(lm.hi, 2.0f), mul(lm.lo, 2.0f)};
    if (k == 0) return lm;
    return ff_add(ff_mul_f(ff{kLn2Hi, kLn2Lo}, (float)k), lm);
}

// 2^(j/32), j = 0..31, as pairs (hi = RN(v), lo = RN(v - hi)).
struct Exp2Table {
    float hi[32], lo[32];
};
inline void make_exp2_table(Exp2Table& t) { // host: from the FP64 exp2
    for (int j = 0; j < 32; ++j) {
        const double v = std::exp2(j / 32.0);
        t.hi[j] = (float)v;
        t.lo[j] = (float)(v - (double)t.hi[j]);
    }
}

// e^y for |y| < 80; relative error below 2^-46 beyond the error already in y.
CM_HD ff exp_ff(ff y, const Exp2Table& tab) {
    const float n = ::rintf(mul(y.hi, 0x1.715476p+5f)); // y * 32 / ln2
    const int ni = (int)n;
    const int k = ni >> 5, j = ni & 31;
    const ff r = ff_add(y, ff_mul_f(ff{-kLn2_32Hi, -kLn2_32Lo}, n)); // |r| <= ln2/64 (+)
    // e^r - 1 = r + r^2/2 + r^3/6 + r^4/24 + r^5/120
    const float rh = r.hi;
    float c = fma(rh, 1.0f / 120.0f, 1.0f / 24.0f);
    c = fma(rh, c, 1.0f / 6.0f);
    c = mul(c, mul(rh, mul(rh, rh)));
    const ff r2h = ff_mul(r, r);
    ff em = ff_add(r, ff{mul(r2h.hi, 0.5f), mul(r2h.lo, 0.5f)});
    em = ff_add_f(em, c);
    const ff t{tab.hi[j], tab.lo[j]};
    const ff e = ff_add(t, ff_mul(t, em)); // 2^(j/32) e^r
    // scale by 2^k (exact while the result stays normal)
    const float sc = from_bits((uint32_t)(k + 127) << 23);
    return ff{mul(e.hi, sc), mul(e.lo, sc)};
}

// The float nearest to a pair whose relative error is at most rel, or false
// when that error could put the exact value on the other side of a rounding
// midpoint. v must be positive and normal with |lo| <= ulp(hi)/2.
CM_HD bool round_checked(ff v, float rel, float& out) {
    const uint32_t u = bits(v.hi);
    const float ulp = from_bits((u & 0x7f800000u) - (23u << 23));
    const bool pow2 = (u & 0x007fffffu) == 0;
    const float half = (v.lo < 0.0f && pow2) ? mul(ulp, 0.25f) : mul(ulp, 0.5f);
    const float err = mul(v.hi, rel);
    out = v.hi;
    return add(fabsf(v.lo), err) < half;
}

constexpr float kLogRel = 0x1p-44f;  // bound used for log_ff (measured below 2^-45)
constexpr float kExpRel = 0x1p-44f;  // bound used for exp_ff's own rounding

// RN(log x) for x >= 2^-126; falls back to the FP64 library function
// (counted in fallbacks) near a rounding midpoint.
CM_HD float logf_cr(float x, int& fallbacks) {
    float out;
    if (round_checked(log_ff(x), kLogRel, out)) return out;
    ++fallbacks;
    return (float)::log((double)x);
}

// RN(L^e) for L > 0, e >= 0 with L^e finite and normal.
CM_HD float powf_cr(float L, float e, const Exp2Table& tab, int& fallbacks) {
    const ff y = ff_mul_f(log_ff(L), e);
    const float ay = fabsf(y.hi);
    if (ay < 80.0f) {
        float out;
        // error of y (relative kLogRel) scales the result by |y| kLogRel
        if (round_checked(exp_ff(y, tab), add(mul(ay, kLogRel), kExpRel), out)) return out;
    }
    ++fallbacks;
    return (float)::pow((double)L, (double)e);
}

} // namespace cm
} // namespace mbx

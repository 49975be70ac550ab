// Double-float arithmetic: a value is hi + lo with two floats, |lo| <= ulp(hi)/2,
// giving about 48 significant bits on the FP32 pipe. On GB300 FP64 issues at
// 1/64 of the FP32 rate and a single warp's FP64 dependency chain is long, so
// the lane that reruns the samples the FP32 pass cannot vouch for computes in
// this type. The error-free transformations are the published ones (Knuth's
// TwoSum, Dekker's Fast2Sum, the FMA-based TwoProd); addition is the "sloppy"
// variant (error bounded relative to |a| + |b|), multiplication and division
// follow the usual double-double construction reduced to float pairs.
#pragma once
#include <math.h>

#include "floatexp.h"

namespace mbx {

struct df32 {
    float hi, lo;
    df32() = default;
    MBX_HD constexpr df32(float h, float l) : hi(h), lo(l) {}
    MBX_HD constexpr df32(float x) : hi(x), lo(0.0f) {}
    MBX_HD constexpr df32(int x) : hi((float)x), lo(0.0f) {}
    MBX_HD df32(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    MBX_HD explicit operator double() const { return (double)hi + (double)lo; }
    MBX_HD explicit operator float() const { return hi + lo; }
};

struct df2 {
    df32 x, y;
};

MBX_HD float df_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
// s + e = a + b exactly (Knuth).
MBX_HD df32 df_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return df32(s, e);
}
// s + e = a + b exactly for |a| >= |b| (Dekker).
MBX_HD df32 df_fast_two_sum(float a, float b) {
    const float s = a + b;
    return df32(s, b - (s - a));
}
MBX_HD df32 operator+(df32 a, df32 b) {
    const df32 s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
MBX_HD df32 operator-(df32 a) { return df32(-a.hi, -a.lo); }
MBX_HD df32 operator-(df32 a, df32 b) { return a + (-b); }
MBX_HD df32 operator*(df32 a, df32 b) {
    const float p = a.hi * b.hi;
    float e = df_fma(a.hi, b.hi, -p);
    e = df_fma(a.hi, b.lo, df_fma(a.lo, b.hi, e));
    return df_fast_two_sum(p, e);
}
MBX_HD df32 operator/(df32 a, df32 b) {
    const float q1 = a.hi / b.hi;
    const df32 r = a - b * df32(q1);
    const float q2 = (r.hi + r.lo) / b.hi;
    return df_fast_two_sum(q1, q2);
}
MBX_HD df32& operator+=(df32& a, df32 b) { return a = a + b; }
MBX_HD df32& operator-=(df32& a, df32 b) { return a = a - b; }
MBX_HD df32& operator*=(df32& a, df32 b) { return a = a * b; }
MBX_HD bool operator<(df32 a, df32 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
MBX_HD bool operator>(df32 a, df32 b) { return b < a; }
MBX_HD bool operator<=(df32 a, df32 b) { return !(b < a); }
MBX_HD bool operator>=(df32 a, df32 b) { return !(a < b); }
MBX_HD bool operator==(df32 a, df32 b) { return a.hi == b.hi && a.lo == b.lo; }
MBX_HD bool operator!=(df32 a, df32 b) { return !(a == b); }

MBX_HD df32 tsqrt(df32 a) {
    if (!(a.hi > 0.0f)) return df32(0.0f);
    const float x = sqrtf(a.hi);
    const df32 r = a - df32(x) * df32(x);
    return df_fast_two_sum(x, (r.hi + r.lo) / (2.0f * x));
}
MBX_HD df32 tabs(df32 a) { return a.hi < 0.0f ? -a : a; }
MBX_HD df32 tmin(df32 a, df32 b) { return a < b ? a : b; }

} // namespace mbx

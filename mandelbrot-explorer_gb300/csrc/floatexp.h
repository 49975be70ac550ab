// Extended-exponent float (m * 2^e, 0.5 <= |m| < 1) and the complex helpers of
// the perturbation path, usable from host C++ and CUDA device code alike.
//
// Semantics follow the reference's src/engine/floatexp.h:17-107 operation by
// operation; frexp/ldexp are implemented on the IEEE bit patterns so that host
// and device produce identical bits (ldexp rounds to nearest-even in the
// subnormal range exactly like libm's). Everything here must be compiled
// without FMA contraction (-ffp-contract=off / -fmad=false).
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define MBX_HD __host__ __device__ __forceinline__
#else
#define MBX_HD inline
#endif

namespace mbx {

MBX_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}
MBX_HD double bitsd(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}
MBX_HD double dabs(double x) { return bitsd(dbits(x) & 0x7fffffffffffffffull); }

// Comparisons on the bit patterns, with exactly the IEEE results (NaN
// included): integer compares, where an FP64 compare costs the latency of an
// FP64 add (64 cycles on GB300, against 4 for an FP32 FMA).
// x == 0.0 (either sign)
MBX_HD bool d_is_zero(double x) { return (dbits(x) << 1) == 0; }
// |a| < |b|; for a and b +0, positive or NaN (a sum of squares, a squared
// radius) this is a < b
MBX_HD bool d_abs_less(double a, double b) {
    const uint64_t ua = dbits(a) & 0x7fffffffffffffffull, ub = dbits(b) & 0x7fffffffffffffffull;
    return ua < ub && ub <= 0x7ff0000000000000ull;
}
// a == b (+0 equals -0, NaN equals nothing)
MBX_HD bool d_eq(double a, double b) {
    const uint64_t ua = dbits(a), ub = dbits(b);
    return (ua == ub && (ua & 0x7fffffffffffffffull) <= 0x7ff0000000000000ull) || ((ua | ub) << 1) == 0;
}
// x <= 0.0
MBX_HD bool d_le_zero(double x) {
    const uint64_t u = dbits(x);
    return (u << 1) == 0 || ((u >> 63) != 0 && (u & 0x7fffffffffffffffull) <= 0x7ff0000000000000ull);
}
// x + x, exactly as the FP64 add rounds it, on the bit pattern for finite x
MBX_HD double d_twice(double x) {
    const uint64_t b = dbits(x);
    const uint64_t e = (b >> 52) & 0x7ff;
    if (e - 1 < 0x7fd) return bitsd(b + (1ull << 52)); // normal, result normal
    if (e == 0) // zero or subnormal: the magnitude shifts (a carry into the exponent gives the normal result)
        return bitsd((b & 0x8000000000000000ull) | ((b & 0x7fffffffffffffffull) << 1));
    if (e == 0x7fe) return bitsd((b & 0x8000000000000000ull) | 0x7ff0000000000000ull); // overflows to infinity
    return x + x; // infinity, NaN
}

// frexp: x = r * 2^e with 0.5 <= |r| < 1; zero, inf and nan return x with e = 0.
MBX_HD double xfrexp(double x, int* e) {
    uint64_t b = dbits(x);
    int ex = (int)((b >> 52) & 0x7ff);
    int adj = 0;
    if (ex == 0) {
        if ((b << 1) == 0) {
            *e = 0;
            return x;
        }
        x = x * 18014398509481984.0; // 2^54, exact
        b = dbits(x);
        ex = (int)((b >> 52) & 0x7ff);
        adj = -54;
    } else if (ex == 0x7ff) {
        *e = 0;
        return x;
    }
    *e = ex - 1022 + adj;
    return bitsd((b & 0x800fffffffffffffull) | (1022ull << 52));
}

// Exact power of two 2^k for -1074 <= k <= 1023 (subnormal below -1022).
MBX_HD double pow2i(int k) {
    if (k >= -1022) return bitsd((uint64_t)(k + 1023) << 52);
    return bitsd(1ull << (k + 1074));
}

// ldexp for finite x, correctly rounded (one rounding in the subnormal range).
MBX_HD double xldexp(double x, int k) {
    if (d_is_zero(x)) return x;
    uint64_t b = dbits(x);
    if (((b >> 52) & 0x7ff) == 0x7ff) return x;
    int e;
    double m = xfrexp(x, &e); // |m| in [0.5,1)
    long long ne = (long long)e + k;   // value = m * 2^ne
    if (ne > 1024) return bitsd((b & 0x8000000000000000ull) | 0x7ff0000000000000ull);
    if (ne >= -1021) {                 // normal result, exact
        uint64_t mb = dbits(m);
        return bitsd((mb & 0x800fffffffffffffull) | ((uint64_t)(ne + 1022) << 52));
    }
    if (ne < -1074) return bitsd(b & 0x8000000000000000ull); // below half the smallest subnormal
    // 2^ne is exactly representable here; one multiply gives the one rounding.
    return m * pow2i((int)ne);
}

struct FE {
    double m;
    int64_t e;
};

MBX_HD FE fe_make(double m, int64_t e) {
    FE r;
    r.m = m;
    r.e = e;
    return r;
}
MBX_HD FE fe_from(double x) {
    if (d_is_zero(x)) return fe_make(0.0, 0);
    int ex;
    double mm = xfrexp(x, &ex);
    return fe_make(mm, (int64_t)ex);
}
MBX_HD double fe_to_double(FE a) {
    if (d_is_zero(a.m)) return 0.0;
    if (a.e > 1100) return bitsd(a.m > 0 ? 0x7ff0000000000000ull : 0xfff0000000000000ull);
    if (a.e < -1100) return 0.0;
    return xldexp(a.m, (int)a.e);
}
MBX_HD FE fe_renorm(double m, int64_t e) {
    if (d_is_zero(m)) return fe_make(0.0, 0);
    int ex;
    double mm = xfrexp(m, &ex);
    return fe_make(mm, e + ex);
}
MBX_HD FE fe_mul(FE a, FE b) {
    if (d_is_zero(a.m) || d_is_zero(b.m)) return fe_make(0.0, 0);
    return fe_renorm(a.m * b.m, a.e + b.e);
}
MBX_HD FE fe_mul_d(FE a, double b) {
    if (d_is_zero(a.m) || d_is_zero(b)) return fe_make(0.0, 0);
    return fe_renorm(a.m * b, a.e);
}
MBX_HD FE fe_scale2(FE a, int64_t k) { return d_is_zero(a.m) ? a : fe_make(a.m, a.e + k); }
MBX_HD FE fe_add(FE a, FE b) {
    if (d_is_zero(a.m)) return b;
    if (d_is_zero(b.m)) return a;
    int64_t d = a.e - b.e;
    if (d > 54) return a;
    if (d < -54) return b;
    if (d >= 0) return fe_renorm(a.m + xldexp(b.m, -(int)d), a.e);
    return fe_renorm(b.m + xldexp(a.m, (int)d), b.e);
}
MBX_HD FE fe_neg(FE a) { return fe_make(-a.m, a.e); }
MBX_HD FE fe_sub(FE a, FE b) { return fe_add(a, fe_neg(b)); }
MBX_HD FE fe_div(FE a, FE b) {
    if (d_is_zero(a.m)) return fe_make(0.0, 0);
    return fe_renorm(a.m / b.m, a.e - b.e);
}
MBX_HD bool fe_abs_less(FE a, FE b) {
    if (d_is_zero(a.m)) return !d_is_zero(b.m);
    if (d_is_zero(b.m)) return false;
    if (a.e != b.e) return a.e < b.e;
    return d_abs_less(a.m, b.m);
}
MBX_HD double xsqrt(double x) {
#ifdef __CUDA_ARCH__
    return __dsqrt_rn(x);
#else
    return __builtin_sqrt(x);
#endif
}
MBX_HD FE fe_sqrt(FE a) {
    if (a.m <= 0.0) return fe_make(0.0, 0);
    int64_t e = a.e;
    double m = a.m;
    if (e & 1) {
        m *= 2.0;
        --e;
    }
    return fe_renorm(xsqrt(m), e / 2);
}

// Complex arithmetic as GCC evaluates std::complex<double> for finite operands
// (inline multiply; division through libgcc's scaled Smith algorithm, restated).
struct C2 {
    double re, im;
};
MBX_HD C2 c2(double r, double i) {
    C2 z;
    z.re = r;
    z.im = i;
    return z;
}
MBX_HD C2 c_add(C2 a, C2 b) { return c2(a.re + b.re, a.im + b.im); }
MBX_HD C2 c_mul(C2 x, C2 y) { return c2(x.re * y.re - x.im * y.im, x.re * y.im + x.im * y.re); }
MBX_HD C2 c_div(C2 num, C2 den) {
    double a = num.re, b = num.im, c = den.re, d = den.im;
    const double RBIG = 8.98846567431157953865e307; // DBL_MAX / 2
    const double RMIN = 2.2250738585072013831e-308;  // DBL_MIN
    const double RMIN2 = 2.2204460492503130808e-16;  // DBL_EPSILON
    const double RMINSCAL = 4503599627370496.0;      // 1 / DBL_EPSILON
    const double RMAX2 = RBIG * RMIN2;
    double ratio, denom, x, y;
    if (dabs(c) < dabs(d)) {
        if (dabs(d) >= RBIG) { a = a / 2; b = b / 2; c = c / 2; d = d / 2; }
        if (dabs(d) < RMIN2) {
            a = a * RMINSCAL; b = b * RMINSCAL; c = c * RMINSCAL; d = d * RMINSCAL;
        } else if ((dabs(a) < RMIN && dabs(b) < RMAX2 && dabs(d) < RMAX2) || (dabs(b) < RMIN && dabs(a) < RMAX2 && dabs(d) < RMAX2)) {
            a = a * RMINSCAL; b = b * RMINSCAL; c = c * RMINSCAL; d = d * RMINSCAL;
        }
        ratio = c / d;
        denom = (c * ratio) + d;
        if (dabs(ratio) > RMIN) {
            x = ((a * ratio) + b) / denom;
            y = ((b * ratio) - a) / denom;
        } else {
            x = ((c * (a / d)) + b) / denom;
            y = ((c * (b / d)) - a) / denom;
        }
    } else {
        if (dabs(c) >= RBIG) { a = a / 2; b = b / 2; c = c / 2; d = d / 2; }
        if (dabs(c) < RMIN2) {
            a = a * RMINSCAL; b = b * RMINSCAL; c = c * RMINSCAL; d = d * RMINSCAL;
        } else if ((dabs(a) < RMIN && dabs(b) < RMAX2 && dabs(c) < RMAX2) || (dabs(b) < RMIN && dabs(a) < RMAX2 && dabs(c) < RMAX2)) {
            a = a * RMINSCAL; b = b * RMINSCAL; c = c * RMINSCAL; d = d * RMINSCAL;
        }
        ratio = d / c;
        denom = (d * ratio) + c;
        if (dabs(ratio) > RMIN) {
            x = ((b * ratio) + a) / denom;
            y = (b - (a * ratio)) / denom;
        } else {
            x = (a + (d * (b / c))) / denom;
            y = (b - (d * (a / c))) / denom;
        }
    }
    return c2(x, y);
}

} // namespace mbx

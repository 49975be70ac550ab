// Per-sample logic of the lane passes: floatexp helpers with a T mantissa
// (float or double), the exact floatexp step, the floatexp BLA skip and the
// lane state machine (setup, iterate, escape / interior / rebase decisions).
//
// Two instantiations run on the device (kernels_mixed.cu):
//   * T = float: the mixed-precision pass. A running error estimate decides
//     which FP32 results it may keep; it queues the other samples for the
//     double-float tier.
//   * T = df32: that tier, the same lane in double-float on the FP32 pipe; what
//     its own estimate cannot vouch for goes to the exact form (the
//     reference's FP64 floatexp loop, kernels_exact.cu).
// T = double compiles as well (the lane in FP64 with its own estimate), for
// host builds. Host-and-device code: the same source compiles as plain C++ so
// a host build can step one sample for inspection. Semantics follow the reference's
// rescaled loop (src/engine/mandel_perturbation.cpp:3287-3618, "mp.cpp").
#pragma once
#include <math.h>
#include <string.h>

#include <climits>
#include <type_traits>

#include "dfloat.cuh"
#include "kernels.h"

#ifdef __CUDACC__
#define MBX_HDF __host__ __device__
#else
#define MBX_HDF inline
#endif

namespace mbx {

MBX_HD unsigned fbits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    unsigned u;
    memcpy(&u, &x, 4);
    return u;
#endif
}
MBX_HD float bitsf(unsigned u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}
// a / b where a relative error of a few ulp is acceptable (screens only).
MBX_HD float fdiv_approx(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdividef(a, b);
#else
    return a / b;
#endif
}
MBX_HD double fdiv_approx(double a, double b) { return a / b; }
MBX_HD float tsqrt(float x) { return sqrtf(x); }
MBX_HD double tsqrt(double x) { return sqrt(x); }
MBX_HD float tabs(float x) { return fabsf(x); }
MBX_HD double tabs(double x) { return fabs(x); }
MBX_HD float tmin(float a, float b) { return fminf(a, b); }
MBX_HD double tmin(double a, double b) { return fmin(a, b); }
// Position of the least significant set bit, 1-based; 0 for x == 0.
MBX_HD int ffs32(int x) {
#ifdef __CUDA_ARCH__
    return __ffs(x);
#else
    return __builtin_ffs(x);
#endif
}
MBX_HD int imax(int a, int b) { return a > b ? a : b; }
MBX_HD int imin(int a, int b) { return a < b ? a : b; }
MBX_HD int64_t lmax(int64_t a, int64_t b) { return a > b ? a : b; }

// ---- floatexp with a T mantissa: m in [0.5,1) (or 0), e int ---------------
template <class T>
struct TE {
    T m;
    int e;
};
using F32E = TE<float>;
using F64E = TE<double>;

MBX_HD F32E te_norm(float m, int e) {
    if (m == 0.0f) return F32E{0.0f, 0};
    unsigned b = fbits(m);
    int ex = (int)((b >> 23) & 0xff);
    if (ex == 0) { // subnormal mantissa: scale up exactly
        m *= 16777216.0f;
        b = fbits(m);
        ex = (int)((b >> 23) & 0xff) - 24;
    }
    return F32E{bitsf((b & 0x807fffffu) | (126u << 23)), e + ex - 126};
}
MBX_HD F64E te_norm(double m, int e) {
    if (m == 0.0) return F64E{0.0, 0};
    uint64_t b = dbits(m);
    int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0) {
        m *= 18014398509481984.0; // 2^54, exact
        b = dbits(m);
        ex = (int)((b >> 52) & 0x7ff) - 54;
    }
    return F64E{bitsd((b & 0x800fffffffffffffull) | (1022ull << 52)), e + ex - 1022};
}
// a * 2^k for a normal (or zero) a, flushing below the type's normal range to
// zero and saturating above it.
MBX_HD float ldexp_ftz(float a, int k) {
    if (a == 0.0f) return 0.0f;
    unsigned b = fbits(a);
    int ex = (int)((b >> 23) & 0xff) + k;
    if (ex <= 0) return 0.0f;
    if (ex >= 255) return bitsf((b & 0x80000000u) | 0x7f7fffffu);
    return bitsf((b & 0x807fffffu) | ((unsigned)ex << 23));
}
MBX_HD double ldexp_ftz(double a, int k) {
    if (a == 0.0) return 0.0;
    uint64_t b = dbits(a);
    int ex = (int)((b >> 52) & 0x7ff) + k;
    if (ex <= 0) return 0.0;
    if (ex >= 2047) return bitsd((b & 0x8000000000000000ull) | 0x7fefffffffffffffull);
    return bitsd((b & 0x800fffffffffffffull) | ((uint64_t)ex << 52));
}
// Double-float forms: the exponent is the high part's.
MBX_HD df32 ldexp_ftz(df32 a, int k) { return df32(ldexp_ftz(a.hi, k), ldexp_ftz(a.lo, k)); }
MBX_HD TE<df32> te_norm(df32 m, int e) {
    if (m.hi == 0.0f) return TE<df32>{df32(0.0f), 0};
    const F32E h = te_norm(m.hi, e); // h.m = m.hi 2^(e - h.e)
    return TE<df32>{df32(h.m, ldexp_ftz(m.lo, e - h.e)), h.e};
}
MBX_HD df32 fdiv_approx(df32 a, df32 b) { return a / b; }
template <class T>
MBX_HD T te_to_real(TE<T> a) { return ldexp_ftz(a.m, a.e); }
template <class T>
MBX_HD TE<T> te_mulr(TE<T> a, T b) { return te_norm(a.m * b, a.e); }
template <class T>
MBX_HD TE<T> te_from_fe(FE a) {
    if (a.m == 0.0) return TE<T>{T(0), 0};
    return te_norm((T)a.m, (int)a.e);
}
template <class T>
MBX_HD FE fe_from_te(TE<T> a) { return a.m == T(0) ? fe_make(0.0, 0) : fe_make((double)a.m, (int64_t)a.e); }

// Per-type constants of the lane.
template <class T>
struct LaneReal;
template <>
struct LaneReal<float> {
    using V2 = float2;
    static constexpr float kTinyX = 1e-30f;         // orbit entries below: exact floatexp step
    static constexpr float kMinS = 8.881784e-16f;  // 2^-50: first step after a rebase needs s above this (|w'| ~ s stays normal)
    static constexpr float kWFloor = 1e-30f;       // |w|^2 floor of the error estimate (err2 ~ 2^-47 |w|^2 stays normal)
    static constexpr float kEscLo = 0.999998f;     // escape screen margins around R^2
    static constexpr float kEscHi = 1.000002f;
    static constexpr int kExpClamp = 120;
    static constexpr bool kTrackError = true;
    using E = float;                              // the error estimate's type
    static constexpr E kEps2 = 7.105427e-15f;     // 2 * (2^-24)^2: per-step rounding variance
    static constexpr E kErrMax = 3e38f;           // saturation of the estimate
    static constexpr int kRatioClamp = 300;       // exponent clamp of (S_old / S_new)^2
    using Z = float;                              // screens (|z|^2, |w|^2 and the like)
    MBX_HD static V2 make2(float a, float b) { return make_float2(a, b); }
    MBX_HD static float tof(float x) { return x; }
    MBX_HD static float toe(float x) { return x; }
    MBX_HD static float z(float x) { return x; }
    MBX_HD static float zabs2(float a, float b) { return fmaf(a, a, b * b); }
};
template <>
struct LaneReal<double> {
    using V2 = double2;
    static constexpr double kTinyX = 1e-290;
    static constexpr double kMinS = 9.332636185032189e-302; // 2^-1000
    static constexpr double kWFloor = 1e-290;
    static constexpr double kEscLo = 1.0;
    static constexpr double kEscHi = 1.0;
    static constexpr int kExpClamp = 1000;
    static constexpr bool kTrackError = true;
    // The estimate in double: its absolute form (units of S^2) reaches
    // 2^-105 |w|^2, below FP32's range.
    using E = double;
    static constexpr E kEps2 = 2.465190328815662e-32; // 2 * (2^-53)^2
    static constexpr E kErrMax = 1e300;
    static constexpr int kRatioClamp = 2000;
    using Z = double;
    MBX_HD static V2 make2(double a, double b) { return make_double2(a, b); }
    MBX_HD static float tof(double x) { return (float)x; }
    MBX_HD static double toe(double x) { return x; }
    MBX_HD static double z(double x) { return x; }
    MBX_HD static double zabs2(double a, double b) { return a * a + b * b; }
};
template <>
struct LaneReal<df32> {
    using V2 = df2;
    static constexpr float kTinyX = 1e-30f;         // as the FP32 lane: both parts must stay normal
    static constexpr float kMinS = 8.673617e-19f;   // 2^-60
    static constexpr float kWFloor = 1e-30f;
    static constexpr float kEscLo = 0.999998f;     // screens run on the high parts, as in the FP32 lane
    static constexpr float kEscHi = 1.000002f;
    static constexpr int kExpClamp = 120;
    static constexpr bool kTrackError = true;
    using E = float;
    static constexpr E kEps2 = 2.524355e-29f;   // 2 * (2^-48)^2
    static constexpr E kErrMax = 3e38f;
    static constexpr int kRatioClamp = 300;
    using Z = float;
    MBX_HD static V2 make2(df32 a, df32 b) { return df2{a, b}; }
    MBX_HD static float tof(df32 x) { return x.hi; }
    MBX_HD static float toe(df32 x) { return x.hi; }
    MBX_HD static float z(df32 x) { return x.hi; }
    MBX_HD static float zabs2(df32 a, df32 b) { return a.hi * a.hi + b.hi * b.hi; }
};

// Exact floatexp step for orbit entries below the lane type's range
// (mp.cpp:2794-2835).
MBX_HDF void exact_step(FE Xr, FE Xi, FE dcr, FE dci, FE& S, double& wr, double& wi) {
    const double sm = S.m, sm2 = sm * sm;
    const int64_t se = S.e;
    const int64_t NONE = (int64_t)0x8000000000000000ll;
    int64_t e = NONE;
    const bool has_w = wr != 0.0 || wi != 0.0;
    if (has_w && Xr.m != 0.0) e = lmax(e, Xr.e + se);
    if (has_w && Xi.m != 0.0) e = lmax(e, Xi.e + se);
    if (has_w) e = lmax(e, se + se);
    if (dcr.m != 0.0) e = lmax(e, dcr.e);
    if (dci.m != 0.0) e = lmax(e, dci.e);
    if (e == NONE) {
        S = fe_make(1.0, 0);
        wr = wi = 0.0;
        return;
    }
    auto align = [e](double m, int64_t te) -> double {
        int64_t d = te - e;
        if (m == 0.0 || d < -54) return 0.0;
        return m * pow2i((int)d);
    };
    const double xs_r = align(Xr.m * sm, Xr.e + se);
    const double xs_i = align(Xi.m * sm, Xi.e + se);
    const double s2 = align(sm2, se + se);
    const double cr = align(dcr.m, dcr.e);
    const double ci = align(dci.m, dci.e);
    const double nr = 2.0 * (xs_r * wr - xs_i * wi) + s2 * (wr * wr - wi * wi) + cr;
    const double ni = 2.0 * (xs_r * wi + xs_i * wr) + 2.0 * s2 * wr * wi + ci;
    const double mag = sqrt(nr * nr + ni * ni);
    if (mag == 0.0) {
        S = fe_make(1.0, 0);
        wr = wi = 0.0;
        return;
    }
    S = fe_renorm(mag, e);
    wr = nr / mag;
    wi = ni / mag;
}

// The FP32 lane's rare steps in FP32 floatexp (float mantissa, int exponent):
// the floatexp step of exact_step with one shared exponent, and the sum
// X + S w with the components kept as mantissa/exponent pairs. The FP32 lane's
// error estimate covers their float roundings like any other step's, so they
// need no FP64 (whose warp instructions cost ~60 FP32 ones on this part).
MBX_HD F32E te_from_fe_f(FE a) { return a.m == 0.0 ? F32E{0.0f, 0} : te_norm((float)a.m, (int)a.e); }
MBX_HD float te_align_f(float m, int me, int e) { // m 2^me in units of 2^e (e >= me - 30 assumed)
    const int d = me - e;
    if (m == 0.0f || d < -30) return 0.0f;
    return ldexp_ftz(m, d);
}
MBX_HD void exact_step_f(F32E Xr, F32E Xi, F32E dcr, F32E dci, F32E& S, float& wr, float& wi) {
    const float sm = S.m, sm2 = sm * sm;
    const int se = S.e;
    int e = INT_MIN;
    const bool has_w = wr != 0.0f || wi != 0.0f;
    if (has_w && Xr.m != 0.0f) e = imax(e, Xr.e + se);
    if (has_w && Xi.m != 0.0f) e = imax(e, Xi.e + se);
    if (has_w) e = imax(e, se + se);
    if (dcr.m != 0.0f) e = imax(e, dcr.e);
    if (dci.m != 0.0f) e = imax(e, dci.e);
    if (e == INT_MIN) {
        S = F32E{0.5f, 1};
        wr = wi = 0.0f;
        return;
    }
    const float xs_r = te_align_f(Xr.m * sm, Xr.e + se, e);
    const float xs_i = te_align_f(Xi.m * sm, Xi.e + se, e);
    const float s2 = te_align_f(sm2, se + se, e);
    const float cr = te_align_f(dcr.m, dcr.e, e);
    const float ci = te_align_f(dci.m, dci.e, e);
    const float nr = 2.0f * (xs_r * wr - xs_i * wi) + s2 * (wr * wr - wi * wi) + cr;
    const float ni = 2.0f * (xs_r * wi + xs_i * wr) + 2.0f * s2 * wr * wi + ci;
    const float mag = sqrtf(nr * nr + ni * ni);
    if (mag == 0.0f) {
        S = F32E{0.5f, 1};
        wr = wi = 0.0f;
        return;
    }
    S = te_norm(mag, e);
    wr = nr / mag;
    wi = ni / mag;
}
// z = X + S w per component as F32E.
MBX_HD F32E te_add_f(F32E a, F32E b) {
    if (a.m == 0.0f) return b;
    if (b.m == 0.0f) return a;
    const int e = imax(a.e, b.e);
    return te_norm(te_align_f(a.m, a.e, e) + te_align_f(b.m, b.e, e), e);
}

// The double-float lane's orbit-entry steps in double-float floatexp (df32
// mantissa, int exponent), the same operations as the FP32 lane's above at
// about 48 bits: the lane's error estimate covers their roundings (kEps2 per
// step) like any other step's, and they take no FP64 instruction. (Its
// floatexp rebase decisions stay in FP64: in double-float floatexp their
// rounding of X + dz relative to |z| grows the estimate at every rebase, and
// the DE frames' double-float tier ran 1.3-1.8x longer.)
// FE -> double-float floatexp; the mantissa's 53 bits split on the bit
// pattern (the top 24 bits exactly, the rest rounded to float).
MBX_HD TE<df32> te_from_fe_df(FE a) {
    if (d_is_zero(a.m)) return TE<df32>{df32(0.0f), 0};
    const uint64_t b = dbits(a.m);
    const int ex = (int)((b >> 52) & 0x7ff); // 1022 for a normalised mantissa in [0.5, 1)
    const unsigned sg = (unsigned)(b >> 63) << 31;
    const float hi = bitsf(sg | (126u << 23) | (unsigned)((b >> 29) & 0x7fffffu));
    const float lo = (float)(unsigned)(b & 0x1fffffffu) * 0x1p-53f;
    const df32 m = df_fast_two_sum(hi, sg ? -lo : lo);
    return TE<df32>{m, (int)a.e + ex - 1022};
}
MBX_HD df32 te_align_df(df32 m, int me, int e) { // m 2^me in units of 2^e
    const int d = me - e;
    if (m.hi == 0.0f || d < -60) return df32(0.0f);
    return ldexp_ftz(m, d);
}
MBX_HD TE<df32> te_add_df(TE<df32> a, TE<df32> b) {
    if (a.m.hi == 0.0f) return b;
    if (b.m.hi == 0.0f) return a;
    const int e = imax(a.e, b.e);
    return te_norm(te_align_df(a.m, a.e, e) + te_align_df(b.m, b.e, e), e);
}
MBX_HD void exact_step_df(TE<df32> Xr, TE<df32> Xi, TE<df32> dcr, TE<df32> dci, TE<df32>& S, df32& wr, df32& wi) {
    const df32 sm = S.m, sm2 = sm * sm;
    const int se = S.e;
    int e = INT_MIN;
    const bool has_w = wr.hi != 0.0f || wi.hi != 0.0f;
    if (has_w && Xr.m.hi != 0.0f) e = imax(e, Xr.e + se);
    if (has_w && Xi.m.hi != 0.0f) e = imax(e, Xi.e + se);
    if (has_w) e = imax(e, se + se);
    if (dcr.m.hi != 0.0f) e = imax(e, dcr.e);
    if (dci.m.hi != 0.0f) e = imax(e, dci.e);
    if (e == INT_MIN) {
        S = TE<df32>{df32(0.5f), 1};
        wr = wi = df32(0.0f);
        return;
    }
    const df32 xs_r = te_align_df(Xr.m * sm, Xr.e + se, e);
    const df32 xs_i = te_align_df(Xi.m * sm, Xi.e + se, e);
    const df32 s2 = te_align_df(sm2, se + se, e);
    const df32 cr = te_align_df(dcr.m, dcr.e, e);
    const df32 ci = te_align_df(dci.m, dci.e, e);
    const df32 two(2.0f);
    const df32 nr = two * (xs_r * wr - xs_i * wi) + s2 * (wr * wr - wi * wi) + cr;
    const df32 ni = two * (xs_r * wi + xs_i * wr) + two * s2 * wr * wi + ci;
    const df32 mag = tsqrt(nr * nr + ni * ni);
    if (mag.hi == 0.0f) {
        S = TE<df32>{df32(0.5f), 1};
        wr = wi = df32(0.0f);
        return;
    }
    S = te_norm(mag, e);
    wr = nr / mag;
    wi = ni / mag;
}

// Floatexp copy of the FP64 BLA table: A and B as mantissa pairs with one
// exponent each, the radius^2 as mantissa + exponent. Built once per reference
// from the FP64 table (k_bla_to_lane).
MBX_HD int dexp_of(double x) { // x = m 2^e, m in [0.5,1)
    int e;
    (void)xfrexp(x, &e);
    return e;
}

template <class T>
MBX_HDF BlaEntry<T> bla_entry(double v, double4 c) {
    BlaEntry<T> b;
    double amax = fmax(fabs(c.x), fabs(c.y)), bmax = fmax(fabs(c.z), fabs(c.w));
    b.ea = amax > 0 ? dexp_of(amax) : 0;
    b.eb = bmax > 0 ? dexp_of(bmax) : 0;
    b.ar = (T)xldexp(c.x, -b.ea);
    b.ai = (T)xldexp(c.y, -b.ea);
    b.br = (T)xldexp(c.z, -b.eb);
    b.bi = (T)xldexp(c.w, -b.eb);
    if (v > 0.0) {
        int e;
        double m = xfrexp(v, &e);
        b.r2m = (T)m;
        b.r2e = e;
        if (b.r2m >= T(1)) { // mantissa rounded up to 1.0
            b.r2m = T(0.5);
            b.r2e += 1;
        }
    } else {
        b.r2m = T(0);
        b.r2e = 0;
    }
    return b;
}

// BLA skip in floatexp (mp.cpp:2883-2970 semantics; coefficients and radii
// constructed in FP64). dz = S w, dc = dcm 2^dce (shared exponent). amp2
// receives |A|^2 (S_old / S_new)^2, the factor that carries a squared error of
// w into the new units.
template <class T>
MBX_HDF int lane_bla(const BlaView& b, const BlaEntry<T>* t, const typename LaneReal<T>::V2* orb, bool periodic, int s, TE<T>& S, T& wr, T& wi,
                     typename LaneReal<T>::V2 dcm, int dce, typename LaneReal<T>::Z ESC2lo, int mx_ref_it, float& amp2, BlaEntry<T>* used = nullptr) {
    using R = LaneReal<T>;
    using Z = typename R::Z;
    int maxp = b.nlev - 1;
    int startp = (s == 1) ? maxp : ffs32(s - 1) - 1;
    if (startp > maxp) startp = maxp;
    if (startp < b.minlevel) return 0;
    const Z wm2 = R::zabs2(wr, wi);
    if (wm2 == Z(0)) return 0;
    const TE<Z> dz2 = te_norm(R::z(S.m) * R::z(S.m) * wm2, 2 * S.e);
    for (int p = startp; p >= b.minlevel; --p) {
        int i = (s - 1) >> p;
        if (i >= b.size[p]) continue;
        const BlaEntry<T> e = t[b.off[p] + i];
        if (e.r2m == T(0)) continue;
        if (!(dz2.e < e.r2e || (dz2.e == e.r2e && dz2.m < R::z(e.r2m)))) continue; // |dz|^2 < r2
        const int l = 1 << p;
        const int land = s + l;
        if (land >= mx_ref_it - 1) continue;
        // A dz + B dc = A (S.m w) 2^(ea + S.e) + B dcm 2^(eb + dce)
        const T swr = S.m * wr, swi = S.m * wi;
        T t1r = e.ar * swr - e.ai * swi, t1i = e.ar * swi + e.ai * swr;
        T t2r = e.br * dcm.x - e.bi * dcm.y, t2i = e.br * dcm.y + e.bi * dcm.x;
        const int E1 = e.ea + S.e, E2 = e.eb + dce;
        const int E = imax(E1, E2);
        const T vr = ldexp_ftz(t1r, E1 - E) + ldexp_ftz(t2r, E2 - E);
        const T vi = ldexp_ftz(t1i, E1 - E) + ldexp_ftz(t2i, E2 - E);
        const T v2 = vr * vr + vi * vi;
        // Never skip past an escape: z = X_land + dz' (conservative test).
        const typename LaneReal<T>::V2 zl = orb[land];
        const T zr = zl.x + ldexp_ftz(vr, E), zi = zl.y + ldexp_ftz(vi, E);
        if (R::zabs2(zr, zi) > ESC2lo) return 0;
        if (v2 == T(0)) {
            if (!periodic) return 0;
            S = TE<T>{T(0.5), 1};
            wr = wi = T(0);
            amp2 = 0.0f;
        } else {
            const T vm = tsqrt(v2), inv = T(1) / vm;
            {
                const float ar = R::tof(e.ar), ai = R::tof(e.ai), sm = R::tof(S.m);
                amp2 = ldexp_ftz(fminf((ar * ar + ai * ai) * (sm * sm) / R::tof(v2), 1e38f), 2 * (E1 - E));
            }
            S = te_norm(vm, E);
            wr = vr * inv;
            wi = vi * inv;
        }
        if (used) *used = e;
        return l;
    }
    return 0;
}

// Error model of the FP32 iteration: each FP32 step adds an independent
// relative rounding error to the delta (variance 2 u^2, u = 2^-24: the RMS of
// the step's roundings, measured against arbitrary-precision orbits), and an
// existing error is carried by the map's derivative |2 z|. A rebase divides the
// delta by |z| / |dz|, so it scales the relative error up by |dz| / |z|.
// The estimate decides which results the FP32 pass may keep; the others leave
// the pass for the FP64 rerun pass:
//   * an escape whose iteration count the error could move: |z_N|^2 or
//     |z_(N-1)|^2 within twice the estimated error of the bailout radius^2;
//   * an interior decision (cycle found, or maxiter reached) with an estimated
//     relative error above 1e-2;
//   * any sample whose estimate exceeds 1/2 (its orbit is no longer known).
// The double-float lane runs the same model with its own rounding variance and
// sends what it cannot vouch for on to the FP64 lane. The estimate itself is
// kept in float for every lane type.
constexpr float kLaneInteriorTol2 = 1e-4f; // (1e-2)^2
constexpr float kLaneCap2 = 0.25f;         // (1/2)^2
// DE colourings: the derivative J follows the orbit, so its relative error is
// of the order of the delta's; an escape's distance (or normal angle) is kept
// only when the estimated relative error of dz is below 1e-4.
constexpr float kLaneDeTol2 = 1e-8f;

// Squared relative error estimate of the delta.
template <class T>
MBX_HD typename LaneReal<T>::E lane_rel_err2(typename LaneReal<T>::E err2, T wr, T wi) {
    using E = typename LaneReal<T>::E;
    const E a = LaneReal<T>::toe(wr), b = LaneReal<T>::toe(wi);
    const E wm2 = a * a + b * b;
    return wm2 > E(0) ? err2 / wm2 : E(0);
}
template <class V2>
MBX_HD float lane_abs2f(V2 v) {
    const float a = (float)v.x, b = (float)v.y;
    return a * a + b * b;
}

// Per-lane state of a lane pass.
template <class T>
struct Lane {
    using V2 = typename LaneReal<T>::V2;
    int i, oidx;         // pass entry, output index
    double dpx, dpy;     // sample offset from the reference in pixels (for rare exact steps)
    TE<T> S;             // delta scale
    T wr, wi, s, dr, di;
    V2 dcm;              // dc mantissas with shared exponent dce
    int dce;
    int m, iter, rm;
    V2 Xc;               // X_m
    // running rounding-error estimate: err2 = (error of w)^2 in units of S^2,
    // g2 = |2 z|^2 at the current iterate (the step's error amplification)
    typename LaneReal<T>::E err2, g2;
    // interior detection
    float zsr_f, zsi_f, conf_D2;
    T swr, swi;
    double zsr, zsi, conf_zr, conf_zi;
    TE<T> sS;
    int save_iter, period_win, conf_P, conf_next, conf_count, conf_giveup, sidx, save_iter2, twin2;
    // derivative J = dz/dc of the DE colourings: J = SJ (jr, ji) with invSJ =
    // 1 / SJ in the lane type (0 below its range); ezr, ezi: z at the escape
    TE<T> SJ;
    T jr, ji, invSJ, ezr, ezi;
};

template <class T>
MBX_HD void lane_refresh(Lane<T>& L) {
    L.s = te_to_real(L.S);
    const T inv = fdiv_approx(T(1), L.S.m);
    L.dr = ldexp_ftz(L.dcm.x * inv, L.dce - L.S.e);
    L.di = ldexp_ftz(L.dcm.y * inv, L.dce - L.S.e);
}

// 2^k as a float, |k| <= 126.
MBX_HD float pow2f(int k) { return bitsf((unsigned)(127 + k) << 23); }

// Rescale of the FP32 lane by the power of two nearest |w|: with |w|^2 =
// m 2^E (m in [1, 2)) and k = floor(E / 2), S.e += k, w and d scale by 2^-k,
// s by 2^k and the error estimate (in units of S^2) by 2^-2k, all exactly, and
// |w| lands in [1, 2 sqrt 2). Needs |w|^2 normal (the caller sends |w|^2 below
// kWFloor on instead); k stays within [-50, 27] for the windows in use.
MBX_HD void lane_rescale_pow2(Lane<float>& L, float wm2) {
    const int k = ((int)((fbits(wm2) >> 23) & 0xffu) - 127) >> 1;
    L.S.e += k;
    const float sc = pow2f(-k);
    L.wr *= sc;
    L.wi *= sc;
    L.err2 *= pow2f(-2 * k);
    lane_refresh(L);
}

// ---- the derivative J = dz/dc (DE colourings) ------------------------------
// As in the reference's rescaled loop (mp.cpp:3348-3360, 3478-3511), J is
// carried like the delta: a floatexp scale SJ and a unit-scale vector (jr, ji)
// in the lane type, advancing as J' = 2 z J + 1 per step (z the pre-step
// value; the "+1" is invSJ in the units of SJ) and as J' = A J + B through a
// BLA skip. A rebase leaves J alone: it is the derivative of the reconstructed
// z. The DE value is formed once per sample, in FP64 floatexp.
MBX_HD double pow2d(int k) { return bitsd((uint64_t)(1023 + k) << 52); }
template <class T>
MBX_HD T lane_mul2k(T x, int k); // x 2^k, |k| <= 250 (exact unless the result leaves the normal range)
template <>
MBX_HD float lane_mul2k<float>(float x, int k) {
    const int h = k / 2;
    return (x * pow2f(h)) * pow2f(k - h);
}
template <>
MBX_HD double lane_mul2k<double>(double x, int k) { return x * pow2d(k); }
template <>
MBX_HD df32 lane_mul2k<df32>(df32 x, int k) { return df32(lane_mul2k<float>(x.hi, k), lane_mul2k<float>(x.lo, k)); }

template <class T>
MBX_HD void lane_j_inv(Lane<T>& L) { L.invSJ = ldexp_ftz(T(1) / L.SJ.m, -L.SJ.e); }

template <class T>
MBX_HD void lane_j_init(Lane<T>& L) { // J_1 = d(dc)/dc = 1
    L.SJ = TE<T>{T(0.5), 1};
    L.jr = T(1);
    L.ji = T(0);
    L.invSJ = T(1);
}

// |j| back to [0.5, 1.5) when |j|^2 leaves [1e-16, 1e16]: SJ.e += k and j scaled
// by 2^-k, with 2^k the binade of the larger component (exact).
template <class T>
MBX_HD void lane_j_window(Lane<T>& L) {
    using R = LaneReal<T>;
    using Z = typename R::Z;
    const Z jm2 = R::zabs2(L.jr, L.ji);
    if (jm2 <= Z(1e16) && jm2 >= Z(1e-16)) return;
    const Z ar = tabs(R::z(L.jr)), ai = tabs(R::z(L.ji));
    const Z amax = ar > ai ? ar : ai;
    if (!(amax > Z(0))) { // the derivative vanished (or is not a number)
        L.SJ = TE<T>{T(0.5), 1};
        L.jr = L.ji = T(0);
        lane_j_inv(L);
        return;
    }
    const int k = te_norm(amax, 0).e; // amax = m 2^k, m in [0.5, 1)
    L.SJ.e += k;
    L.jr = lane_mul2k(L.jr, -k);
    L.ji = lane_mul2k(L.ji, -k);
    lane_j_inv(L);
}

// J' = 2 z J + 1 with z at unit scale in the lane type.
template <class T>
MBX_HD void lane_j_step(Lane<T>& L, T zr, T zi) {
    const T a = T(2) * (zr * L.jr - zi * L.ji) + L.invSJ;
    const T b = T(2) * (zr * L.ji + zi * L.jr);
    L.jr = a;
    L.ji = b;
    lane_j_window(L);
}
// The FP32 lane's form, from 2 z = 2 X + 2 s w as the common-step loop forms it.
MBX_HD void lane_j_step_2z(Lane<float>& L, float z2r, float z2i) {
    const float a = fmaf(z2r, L.jr, fmaf(-z2i, L.ji, L.invSJ));
    const float b = fmaf(z2r, L.ji, z2i * L.jr);
    L.jr = a;
    L.ji = b;
    lane_j_window(L);
}

// J = (nr, ni) given in floatexp.
template <class T>
MBX_HDF void lane_j_set_fe(Lane<T>& L, FE nr, FE ni) {
    const FE mag = fe_sqrt(fe_add(fe_mul(nr, nr), fe_mul(ni, ni)));
    if (mag.m == 0.0) {
        L.SJ = TE<T>{T(0.5), 1};
        L.jr = L.ji = T(0);
    } else {
        L.SJ = te_from_fe<T>(mag);
        L.jr = (T)fe_to_double(fe_div(nr, mag));
        L.ji = (T)fe_to_double(fe_div(ni, mag));
    }
    lane_j_inv(L);
}
// J' = 2 z J + 1 with z in floatexp: the steps where z lies outside the lane
// type's range (the exact floatexp steps; rare).
template <class T>
MBX_HDF void lane_j_step_fe(Lane<T>& L, FE zr, FE zi) {
    const FE sj = fe_from_te(L.SJ);
    const FE Jr = fe_mul_d(sj, (double)L.jr), Ji = fe_mul_d(sj, (double)L.ji);
    const FE nr = fe_add(fe_scale2(fe_sub(fe_mul(zr, Jr), fe_mul(zi, Ji)), 1), fe_make(0.5, 1));
    const FE ni = fe_scale2(fe_add(fe_mul(zr, Ji), fe_mul(zi, Jr)), 1);
    lane_j_set_fe(L, nr, ni);
}
// J' = A J + B through a BLA skip, with the entry's floatexp coefficients.
template <class T>
MBX_HDF void lane_j_bla(Lane<T>& L, const BlaEntry<T>& e) {
    const FE sj = fe_from_te(L.SJ);
    const FE Jr = fe_mul_d(sj, (double)L.jr), Ji = fe_mul_d(sj, (double)L.ji);
    const FE Ar = fe_renorm((double)e.ar, e.ea), Ai = fe_renorm((double)e.ai, e.ea);
    const FE Br = fe_renorm((double)e.br, e.eb), Bi = fe_renorm((double)e.bi, e.eb);
    const FE nr = fe_add(fe_sub(fe_mul(Ar, Jr), fe_mul(Ai, Ji)), Br);
    const FE ni = fe_add(fe_add(fe_mul(Ar, Ji), fe_mul(Ai, Jr)), Bi);
    lane_j_set_fe(L, nr, ni);
}
// |J| in floatexp.
template <class T>
MBX_HDF FE lane_j_mag(const Lane<T>& L) {
    const double jr = (double)L.jr, ji = (double)L.ji;
    return fe_mul_d(fe_from_te(L.SJ), xsqrt(jr * jr + ji * ji));
}

// dz = S w with S <- |v| 2^e and w <- v / |v| for a vector v scaled by 2^e.
template <class T>
MBX_HD void lane_set_delta(Lane<T>& L, T vr, T vi, int e) {
    const T v2 = vr * vr + vi * vi;
    if (v2 == T(0)) {
        L.S = TE<T>{T(0.5), 1};
        L.wr = L.wi = T(0);
        return;
    }
    const T vm = tsqrt(v2), inv = T(1) / vm;
    L.S = te_norm(vm, e);
    L.wr = vr * inv;
    L.wi = vi * inv;
}

template <class T>
MBX_HD FE lane_dc_re(const MixedParams& p, const Lane<T>& L) { return fe_mul_d(p.dxfe, L.dpx); }
template <class T>
MBX_HD FE lane_dc_im(const MixedParams& p, const Lane<T>& L) { return fe_mul_d(p.dyfe, L.dpy); }

// A sample offset in the lane type: the float table's entry for FP32 lanes
// (no FP64 conversion), else the double value converted.
template <class T>
MBX_HD T lane_offset(const float* tabf, int k, double d) { return (T)d; }
template <>
MBX_HD float lane_offset<float>(const float* tabf, int k, double d) { return tabf ? tabf[k] : (float)d; }

// Start sample arr = {row, col, subrow, subcol} as pass entry i.
template <class T>
MBX_HDF void lane_setup_at(Lane<T>& L, int i, const int* arr, const MixedParams& p, const TE<T> dxf, const TE<T> dyf, const typename LaneReal<T>::V2* orb) {
    const FrameGeom& g = p.g;
    L.i = i;
    const int cy = arr[0] * g.sub + g.sub / 2 + arr[2], cx = arr[1] * g.sub + g.sub / 2 + arr[3];
    L.oidx = cy * g.W * g.sub + cx;
    T ox, oy;
    if (p.dpx_tab) {
        L.dpx = p.dpx_tab[cx];
        L.dpy = p.dpy_tab[cy];
        ox = lane_offset<T>(p.dpx_tabf, cx, L.dpx);
        oy = lane_offset<T>(p.dpy_tabf, cy, L.dpy);
    } else {
        L.dpx = arr[1] + (double)arr[3] / g.sub - p.ref_x;
        L.dpy = arr[0] + (double)arr[2] / g.sub - p.ref_y;
        ox = (T)L.dpx;
        oy = (T)L.dpy;
    }
    // dc in floatexp with one shared exponent.
    const TE<T> cr = te_mulr(dxf, ox), ci = te_mulr(dyf, oy);
    int e = (cr.m != T(0)) ? cr.e : ((ci.m != T(0)) ? ci.e : 0);
    if (cr.m != T(0) && ci.m != T(0)) e = imax(cr.e, ci.e);
    L.dce = e;
    L.dcm = LaneReal<T>::make2(ldexp_ftz(cr.m, cr.e - e), ldexp_ftz(ci.m, ci.e - e));
    lane_set_delta(L, L.dcm.x, L.dcm.y, e);
    lane_refresh(L);
    L.m = 1;
    L.iter = 1;
    L.rm = 0;
    L.Xc = orb[0];
    L.zsr = L.zsi = 1e30;
    L.zsr_f = L.zsi_f = 1e30f;
    L.conf_zr = L.conf_zi = 0.0;
    L.conf_D2 = 0.0f;
    L.save_iter = 1;
    L.period_win = 1;
    L.conf_P = L.conf_next = L.conf_count = L.conf_giveup = 0;
    L.swr = L.swi = T(3e38);
    L.sS = TE<T>{T(2), 0};
    L.sidx = -2;
    L.save_iter2 = 1;
    L.twin2 = 1;
    L.err2 = LaneReal<T>::kEps2;
    L.g2 = 4.0f * lane_abs2f(L.Xc);
    lane_j_init(L);
}

template <class T>
MBX_HDF void lane_setup(Lane<T>& L, int i, const DeviceFrame& f, const MixedParams& p, const TE<T> dxf, const TE<T> dyf, const typename LaneReal<T>::V2* orb) {
    int arr[4];
    entry_coords(f.px, i, arr);
    lane_setup_at(L, i, arr, p, dxf, dyf, orb);
}

// (a / b)^2 in the estimate's type, saturating: converts err2 from units of
// a^2 to b^2.
template <class T>
MBX_HD typename LaneReal<T>::E lane_scale_ratio2(TE<T> a, TE<T> b) {
    using E = typename LaneReal<T>::E;
    constexpr int c = LaneReal<T>::kRatioClamp;
    const E bm = LaneReal<T>::toe(b.m);
    if (bm == E(0)) return E(0);
    const E r = LaneReal<T>::toe(a.m) / bm;
    return ldexp_ftz(r * r, imax(-c, imin(c, 2 * (a.e - b.e))));
}

// z = X_m + S w in FP64 (rare decisions).
template <class T>
MBX_HD void lane_z_double(const Lane<T>& L, const double2* Zd, double& zr, double& zi) {
    const double2 Xd = L.m ? Zd[L.rm] : make_double2(0.0, 0.0);
    const double sd = xldexp((double)L.S.m, L.S.e);
    zr = Xd.x + sd * (double)L.wr;
    zi = Xd.y + sd * (double)L.wi;
}

// The lane's step w' = (2 X + s w) w + d and its error update (one rounding
// variance added, the existing error carried by g2 = |2 z|^2).
template <class T>
MBX_HD void lane_step(typename LaneReal<T>::V2 X, T s, T wr, T wi, T dr, T di, typename LaneReal<T>::E err2, typename LaneReal<T>::E g2, T& nwr, T& nwi,
                      typename LaneReal<T>::E& nerr2) {
    using R = LaneReal<T>;
    const T fR = T(2) * X.x + s * wr;
    const T fI = T(2) * X.y + s * wi;
    nwr = fR * wr - fI * wi + dr;
    nwi = fR * wi + fI * wr + di;
    const typename R::E a = R::toe(nwr), c = R::toe(nwi);
    nerr2 = err2 * g2 + R::kEps2 * (a * a + c * c);
}

// The FP32 step with its operations spelled out: f = 2 X + s w as one paired
// FMA (f32x2), w' = f w + d as four FMAs, |w'|^2 and the error update as
// FMAs. The common-step loop (lane_fast_f32) performs exactly these, so a
// sample's result does not depend on which of the two paths took a step.
template <>
MBX_HD void lane_step<float>(float2 X, float s, float wr, float wi, float dr, float di, float err2, float g2, float& nwr, float& nwi, float& nerr2) {
    const float2 X2 = make_float2(X.x + X.x, X.y + X.y); // exact
#ifdef __CUDA_ARCH__
    const float2 f = __ffma2_rn(make_float2(s, s), make_float2(wr, wi), X2);
#else
    const float2 f = make_float2(fmaf(s, wr, X2.x), fmaf(s, wi, X2.y));
#endif
    nwr = fmaf(f.x, wr, fmaf(-f.y, wi, dr));
    nwi = fmaf(f.x, wi, fmaf(f.y, wr, di));
    const float wm2 = fmaf(nwr, nwr, nwi * nwi);
    nerr2 = fmaf(err2, g2, LaneReal<float>::kEps2 * wm2);
}

// z = X + s w (per component); as one FMA in the FP32 lane.
template <class T>
MBX_HD T lane_zc(T x, T s, T w) { return x + s * w; }
template <>
MBX_HD float lane_zc<float>(float x, float s, float w) { return fmaf(s, w, x); }

// J' = 2 z J + 1 with z = X + s w of the lane's current (pre-step) state, in
// the form both of the FP32 lane's paths use.
template <class T>
MBX_HD void lane_j_advance(Lane<T>& L) {
    if constexpr (std::is_same<T, float>::value)
        lane_j_step_2z(L, fmaf(L.s + L.s, L.wr, L.Xc.x + L.Xc.x), fmaf(L.s + L.s, L.wi, L.Xc.y + L.Xc.y));
    else
        lane_j_step(L, lane_zc<T>(L.Xc.x, L.s, L.wr), lane_zc<T>(L.Xc.y, L.s, L.wi));
}


// The general code's rebase decision on a post-step state (mp.cpp:3584-3615):
// 0 none, 1 rebase in the lane type, 2 the floatexp decision. |z|^2 < |dz|^2 is
// decided on floatexp with a 1e-4 margin; inside the margin, for strong
// cancellation in X + dz, and at the end of the reference it is left to
// floatexp. Screen: |dz|^2 < |X|^2 / 5 means |z| > |dz| (no rebase); s = 0 when
// S is below the type's range, where |dz|^2 <= 2^-252 wmax2 is far below any
// |X|^2 above kTinyX^2.
template <class T>
MBX_HD int lane_rebase_decision(const TE<T>& S, T s, T wr, T wi, typename LaneReal<T>::V2 Xc, int m, typename LaneReal<T>::Z zrad, int per, int reflen) {
    using R = LaneReal<T>;
    using Z = typename R::Z;
    if (!per && m >= reflen) return 2;
    const Z w2 = R::zabs2(wr, wi);
    const Z xr2 = R::zabs2(Xc.x, Xc.y);
    const Z sz = R::z(s);
    if (xr2 > Z(R::kTinyX) * Z(R::kTinyX) && sz * sz * w2 < Z(0.2) * xr2) return 0;
    const TE<Z> dz2 = te_norm(R::z(S.m) * R::z(S.m) * w2, 2 * S.e);
    if (dz2.m == Z(0)) return 0;
    if (zrad == Z(0)) return 2;
    // q = |z|^2 / |dz|^2 against 1 -/+ 1e-4 without a division:
    // z2.m 2^(z2.e - dz2.e) against dz2.m (1 -/+ 1e-4)
    const TE<Z> z2 = te_norm(zrad, 0);
    const Z zq = ldexp_ftz(z2.m, imax(-R::kExpClamp, imin(R::kExpClamp, z2.e - dz2.e)));
    if (zq < Z(0.9999) * dz2.m) return (zrad > Z(0.25) * xr2 && s != T(0)) ? 1 : 2;
    if (zq < Z(1.0001) * dz2.m) return 2;
    return 0;
}

// Decision 1: the delta restarts as dz = z from the start of the reference;
// the error estimate changes units (S_old / S_new)^2 and gains one rounding.
template <class T>
MBX_HD void lane_rebase_to(Lane<T>& L, T zr, T zi) {
    using R = LaneReal<T>;
    const TE<T> S0 = L.S;
    lane_set_delta(L, zr, zi, 0);
    lane_refresh(L);
    if (R::kTrackError) L.err2 = L.err2 * lane_scale_ratio2(S0, L.S) + R::kEps2;
    L.m = 0;
    L.rm = -1;
    L.Xc = R::make2(T(0), T(0));
}

// Common iterations of the FP32 lane without interior detection. The
// iterations that take none of the general code's rare branches (orbit entry
// below range, escape screen, precision cap, the floatexp rebase decision, end
// of the reference) run here, and so do its two frequent ones — a BLA skip at a
// BLA position and a rebase the general code takes in the lane type — through
// the same helpers (lane_bla, lane_rebase_decision, lane_rebase_to), so that a
// sample's result does not depend on which of the two paths took an
// iteration. The first iteration that could take another branch is left
// uncommitted for the general code, which redoes it from the same state.
//
// Steps run in runs of at most kRun whose length is fixed once per run (up to
// the next BLA position, the wrap of a periodic orbit, maxiter or the end of
// the reference, and the call's budget). A full run is computed speculatively
// — kRun steps from the run's start state, unrolled, with one flag for "every
// step common" — and committed at once; a rare step in it (about one in fifty)
// sends the run to the careful loop, which redoes it one step at a time.
// Rescales (|w|^2 out of its window) are exact powers of two
// (lane_rescale_pow2), which commute with the step's roundings (every term of
// w' = (2 X + s w) w + d scales by the same power of two, as do 2 z, the error
// estimate and the BLA and rebase decisions), so they are taken between runs, a
// step only guarding |w|^2 against leaving FP32's range. Per step: one 16-byte
// load of {2 X, |X|^2 or 0} (MixedParams::Zq), the step, 2 z = 2 X + 2 s w' as
// one paired FMA (so |2 z|^2 is the next error amplification g2 = 4 |z|^2
// exactly) and four compares. At a BLA position the per-position radius
// maximum screens: |dz|^2 not below it fails every level. Returns the budget
// used (a step or a BLA skip counts one); the counters are the lane pass's.
constexpr int kRun = 8;
constexpr float kWGuard = 1e30f; // |w|^2 bound of a step between rescales (FP32 range with margin)

template <bool DERIV>
MBX_HDF int lane_fast_f32(Lane<float>& L, int budget, const FrameGeom& g, const MixedParams& p, const BlaView& bv, const Bla32* blat, const float2* orb, int reflen,
                          unsigned& n_steps, unsigned& n_bla, unsigned long long& n_skip, unsigned& n_rebase) {
    using R = LaneReal<float>;
    const float4* q = p.Zq;
    const int per = p.per;
    const BlaMaxR2* bmax = p.blamax;
    const int minlevel = bv.minlevel;
    const bool bla_on = blat != nullptr;
    int left = budget;
    const float e4 = 4.0f * p.esc2lo; // |2 z|^2 > 4 ESC2lo: the escape screen on 4 |z|^2 (exact scaling)
    const float wmax2 = p.wmax2, wmin2 = p.wmin2;
    const int blamask = (1 << minlevel) - 1;
    float s = L.s, dr = L.dr, di = L.di;
    float s2x5 = 5.0001f * (s * s); // |dz|^2 < |X|^2 / 5 as 5.0001 s^2 |w|^2 < |X|^2 (implies the general code's rebase screen)
    float wr = L.wr, wi = L.wi;
    float err2 = L.err2, g2 = L.g2;
    float2 X2 = make_float2(L.Xc.x + L.Xc.x, L.Xc.y + L.Xc.y);
    int m = L.m, rm = L.rm, it = L.iter; // it: the iteration count (a rebase restarts m, not it)
#ifdef __CUDA_ARCH__
    float2 ss = make_float2(s, s), ss2 = make_float2(s + s, s + s);
#endif
    // DE: 2 z before the step, for J' = 2 z J + 1 (the general code's form)
    float z2pr = 0.0f, z2pi = 0.0f;
    float wm2 = fmaf(wr, wr, wi * wi);
    // the lane's state into L and back (around the shared helpers)
    auto sync_out = [&]() {
        L.wr = wr;
        L.wi = wi;
        L.err2 = err2;
        L.g2 = g2;
        L.m = m;
        L.iter = it;
        L.rm = rm;
        L.Xc = make_float2(0.5f * X2.x, 0.5f * X2.y); // exact
    };
    auto sync_in = [&]() {
        wr = L.wr;
        wi = L.wi;
        err2 = L.err2;
        g2 = L.g2;
        m = L.m;
        rm = L.rm;
        it = L.iter;
        X2 = make_float2(L.Xc.x + L.Xc.x, L.Xc.y + L.Xc.y);
        s = L.s;
        dr = L.dr;
        di = L.di;
        s2x5 = 5.0001f * (s * s);
        wm2 = fmaf(wr, wr, wi * wi);
#ifdef __CUDA_ARCH__
        ss = make_float2(s, s);
        ss2 = make_float2(s + s, s + s);
#endif
        if (DERIV) {
            z2pr = fmaf(s + s, wr, X2.x);
            z2pi = fmaf(s + s, wi, X2.y);
        }
    };
    if (DERIV) {
        z2pr = fmaf(s + s, wr, X2.x);
        z2pi = fmaf(s + s, wi, X2.y);
    }
    for (;;) {
        // the window, between runs (a power-of-two rescale commutes with the
        // steps' roundings)
        if (!(wm2 <= wmax2 && wm2 >= wmin2) && wm2 >= R::kWFloor) {
            sync_out();
            lane_rescale_pow2(L, wm2);
            sync_in();
        }
        // maxiter, or the end of a non-periodic reference (where the general
        // code forces the rebase)
        int seg = g.mxit - it;
        if (!per && reflen - 1 - m < seg) seg = reflen - 1 - m;
        if (seg <= 0 || left <= 0) break;
        // (the budget is a soft bound: a run is not cut by it, so that runs stay
        // full and aligned to the BLA positions; a call overshoots by < kRun)
        // the current orbit entry below the lane's range (X = 0 after a rebase
        // takes a common step when s is a normal number well above FP32's floor)
        if (m == 0 ? !(s >= R::kMinS) : (fabsf(X2.x) < 2.0f * R::kTinyX && fabsf(X2.y) < 2.0f * R::kTinyX)) break;
        if (seg > kRun) seg = kRun;
        int nidx = rm + 1;
        if (per) {
            if (nidx == per) nidx = 0;
            if (per - nidx < seg) seg = per - nidx; // the run ends at the wrap
        }
        if (bla_on) {
            const int u = (rm - 1) & blamask;
            if (u == 0 && m >= 2) {
                if (!bmax) break;
                const BlaMaxR2 r = bmax[(rm - 1) >> minlevel];
                if (r.m != 0.0f) {
                    if (wm2 == 0.0f) break;
                    const F32E dz2 = te_norm(L.S.m * L.S.m * wm2, 2 * L.S.e); // as lane_bla forms it
                    if (dz2.e < r.e || (dz2.e == r.e && dz2.m < r.m)) {
                        // a level may apply: the general code's BLA attempt
                        sync_out();
                        float amp2 = 0.0f;
                        BlaEntry<float> used;
                        const int skip = lane_bla(bv, blat, orb, per > 0, rm, L.S, L.wr, L.wi, L.dcm, L.dce, p.esc2lo, per ? per : reflen, amp2, DERIV ? &used : nullptr);
                        if (skip > 0) {
                            ++n_bla;
                            n_skip += (unsigned long long)skip;
                            --left;
                            L.m += skip;
                            L.iter += skip;
                            L.rm += skip;
                            if (per && L.rm >= per) L.rm -= per;
                            lane_refresh(L);
                            L.Xc = orb[L.rm];
                            // the skip carries the error by A; |w| is 1 afterwards
                            L.err2 = L.err2 * amp2 + R::kEps2;
                            L.g2 = 4.0f * lane_abs2f(L.Xc);
                            if (DERIV) lane_j_bla(L, used);
                            sync_in();
                            continue;
                        }
                        // no level applies: a common iteration
                    }
                }
            }
            const int to_next = blamask + 1 - u; // iterations to the next BLA position
            if (to_next < seg) seg = to_next;
        }
        const float4* qp = q + nidx;
        if (!DERIV && seg == kRun) {
            // a full run, speculatively (see above)
            float tr = wr, ti = wi, te = err2, tg = g2, tw = wm2;
            float2 tX = X2;
            bool ok = true;
#pragma unroll
            for (int kk = 0; kk < kRun; ++kk) {
                const float4 Xn = qp[kk];
#ifdef __CUDA_ARCH__
                const float2 f = __ffma2_rn(ss, make_float2(tr, ti), tX);
#else
                const float2 f = make_float2(fmaf(s, tr, tX.x), fmaf(s, ti, tX.y));
#endif
                const float nwr = fmaf(f.x, tr, fmaf(-f.y, ti, dr));
                const float nwi = fmaf(f.x, ti, fmaf(f.y, tr, di));
#ifdef __CUDA_ARCH__
                const float2 z2 = __ffma2_rn(ss2, make_float2(nwr, nwi), make_float2(Xn.x, Xn.y));
#else
                const float2 z2 = make_float2(fmaf(s + s, nwr, Xn.x), fmaf(s + s, nwi, Xn.y));
#endif
                const float g2n = fmaf(z2.x, z2.x, z2.y * z2.y);
                const float nwm2 = fmaf(nwr, nwr, nwi * nwi);
                const float ne = fmaf(te, tg, R::kEps2 * nwm2);
                ok = ok & (!(g2n > e4) & (ne <= kLaneCap2 * nwm2) & (nwm2 >= R::kWFloor) & (nwm2 <= kWGuard) & (s2x5 * nwm2 < Xn.z));
                tr = nwr;
                ti = nwi;
                te = ne;
                tg = g2n;
                tw = nwm2;
                tX = make_float2(Xn.x, Xn.y);
            }
            if (ok) {
                wr = tr;
                wi = ti;
                err2 = te;
                g2 = tg;
                wm2 = tw;
                X2 = tX;
                m += kRun;
                it += kRun;
                rm = nidx + kRun - 1;
                left -= kRun;
                n_steps += kRun;
                continue;
            }
        }
        // the careful loop: one step at a time up to the run's end or its first
        // rare step; a rebase the general code would take in the lane type is
        // taken here
        bool leave = false, rebased = false;
        for (int k = 0; k < seg; ++k) {
            const float4 Xn = qp[k];
#ifdef __CUDA_ARCH__
            const float2 f = __ffma2_rn(ss, make_float2(wr, wi), X2);
#else
            const float2 f = make_float2(fmaf(s, wr, X2.x), fmaf(s, wi, X2.y));
#endif
            const float nwr = fmaf(f.x, wr, fmaf(-f.y, wi, dr));
            const float nwi = fmaf(f.x, wi, fmaf(f.y, wr, di));
#ifdef __CUDA_ARCH__
            const float2 z2 = __ffma2_rn(ss2, make_float2(nwr, nwi), make_float2(Xn.x, Xn.y));
#else
            const float2 z2 = make_float2(fmaf(s + s, nwr, Xn.x), fmaf(s + s, nwi, Xn.y));
#endif
            const float g2n = fmaf(z2.x, z2.x, z2.y * z2.y);
            const float nwm2 = fmaf(nwr, nwr, nwi * nwi);
            const float ne = fmaf(err2, g2, R::kEps2 * nwm2);
            // (|w| = 0 and the precision cap both leave through the |w|^2
            // tests; a NaN fails them too)
            const bool others = !(g2n > e4) && ne <= kLaneCap2 * nwm2 && nwm2 >= R::kWFloor && nwm2 <= kWGuard;
            if (!others) {
                leave = true;
                break;
            }
            int decide = 0;
            if (!(s2x5 * nwm2 < Xn.z)) {
                // the rebase screen: the general code's decision on the
                // post-step state (z = 2 z / 2 exactly)
                const float zr = 0.5f * z2.x, zi = 0.5f * z2.y;
                decide = lane_rebase_decision<float>(L.S, s, nwr, nwi, make_float2(0.5f * Xn.x, 0.5f * Xn.y), m + 1, fmaf(zr, zr, zi * zi), per, reflen);
                if (decide == 2) {
                    leave = true;
                    break;
                }
            }
            // commit the step
            if (DERIV) {
                lane_j_step_2z(L, z2pr, z2pi);
                z2pr = z2.x;
                z2pi = z2.y;
            }
            wr = nwr;
            wi = nwi;
            err2 = ne;
            g2 = g2n;
            wm2 = nwm2;
            X2 = make_float2(Xn.x, Xn.y);
            ++m;
            ++it;
            rm = nidx + k;
            --left;
            ++n_steps;
            if (decide == 1) {
                sync_out();
                lane_rebase_to(L, 0.5f * z2.x, 0.5f * z2.y);
                ++n_rebase;
                sync_in();
                rebased = true;
                break;
            }
        }
        if (leave) break; // a rare iteration: the general code takes it (after the window below)
        (void)rebased;
    }
    // leave with |w|^2 inside the window, as the general code keeps it
    if (!(wm2 <= wmax2 && wm2 >= wmin2) && wm2 >= R::kWFloor) {
        sync_out();
        lane_rescale_pow2(L, wm2);
        sync_in();
    }
    sync_out();
    return budget - left;
}

// Interior decision: a lane whose error estimate is too large leaves for the
// next tier (4: an interior decision it cannot vouch for) instead of reporting
// interior (2).
template <class T>
MBX_HD int lane_interior(const Lane<T>& L) {
    if (LaneReal<T>::kTrackError && !(lane_rel_err2(L.err2, L.wr, L.wi) <= kLaneInteriorTol2)) return 4;
    return 2;
}

// Advance one lane by up to `budget` iterations. Returns 0 running, 1 escaped,
// 2 interior, and for lanes with an error estimate (rerun in the next tier) 3
// precision spent, 4 an unvouched interior decision, 5 an unvouched escape
// (|z|^2 at N or N - 1 within the estimated error of the bailout); zrad_out is
// set on escape.
// INTR = false compiles the lane without its interior detectors, for passes
// whose interior detection is off (exterior frames after the probe): their
// state then takes no registers.
template <class T, bool INTR = true, bool FASTI = false, bool DE = false>
MBX_HDF int lane_run(Lane<T>& L, int budget, const DeviceFrame& f, const MixedParams& p, const BlaEntry<T>* blat, const typename LaneReal<T>::V2* orb,
                     int reflen, T ESC2f, int blamask, T& zrad_out, unsigned& n_steps, unsigned& n_bla, unsigned long long& n_skip,
                     unsigned& n_rebase, unsigned& n_exact, unsigned& n_ferebase) {
    using R = LaneReal<T>;
    using Z = typename R::Z;
    const FrameGeom& g = p.g;
    const int per = p.per;
    const double2* Zd = f.orbit.Z;
    const FE2* Zfe = f.orbit.Zfe;
    (void)ESC2f;
    // (float)ESC2 rounded on the host for the float-screen lanes: no FP64 conversion per call
    const Z ESC2z = std::is_same<Z, float>::value ? (Z)p.esc2f : (Z)g.ESC2;
    const Z ESC2hi = ESC2z * R::kEscHi, ESC2lo = ESC2z * R::kEscLo;
    // DE colourings: the derivative J advances with the delta (DE lanes only)
    const bool deriv = DE && g.deriv;
    for (int b = 0; b < budget; ++b) {
        if constexpr (std::is_same<T, float>::value && !FASTI) {
            if (!(INTR && p.use_interior) && p.Zq) {
                const int used = deriv ? lane_fast_f32<true>(L, budget - b, g, p, f.bla, blat, orb, reflen, n_steps, n_bla, n_skip, n_rebase)
                                       : lane_fast_f32<false>(L, budget - b, g, p, f.bla, blat, orb, reflen, n_steps, n_bla, n_skip, n_rebase);
                b += used;
                if (b >= budget) return 0;
            }
        }
        if constexpr (!std::is_same<T, double>::value) if (!(std::is_same<T, float>::value && !FASTI && !(INTR && p.use_interior) && p.Zq)) {
            // Common steps of a lane without interior detection: an
            // iteration that takes none of the branches below (no BLA skip,
            // orbit entry in range, no escape screen, precision cap, rescale,
            // rebase candidate or end of the reference) is the step, the error
            // update and the index advance. Such iterations run here with the
            // same operations; the first iteration that could take a branch is
            // left uncommitted and the general code redoes it from the same state.
            // At a BLA position the per-position radius maximum decides: if
            // |dz|^2 is not below it, every level fails and lane_bla would
            // return 0, so the iteration is a common one.
            // FASTI: the common-iteration loop with interior detection on
            // too (the interior gate's probe); its extra tests: no state
            // repetition, no save due, no confirmation in progress and not a
            // 16th-iteration Brent check
            const bool intr = INTR && p.use_interior;
            if (!intr || FASTI) {
                using E = typename R::E;
                const Z wmax2 = Z(p.wmax2), wmin2 = Z(p.wmin2);
                const BlaMaxR2* bmax = std::is_same<T, float>::value ? p.blamax : nullptr; // FP32 tables only
                const int minlevel = f.bla.minlevel;
                // one counter: m; iter = m + off, the steps taken and the
                // budget spent follow from m - m0 and are written back on exit.
                // m reaching mlim covers maxiter and the end of a non-periodic
                // reference (m + 1 >= reflen, where the rebase is forced).
                const int m0 = L.m, off = L.iter - L.m;
                int mlim = g.mxit - off;
                if (!per && reflen - 1 < mlim) mlim = reflen - 1;
                const int mbud = m0 + (budget - b);
                // |dz|^2 < |X|^2 / 5 (the rebase screen) as 5.0001 s^2 |w|^2 <
                // |X|^2: the margin makes it imply the general code's form
                // whatever the roundings, so a committed iteration is one the
                // general code would not rebase
                const Z s2x5 = Z(5.0001) * (R::z(L.s) * R::z(L.s));
                int m = m0;
                for (;;) {
                    if (m >= mlim) break;
                    if (FASTI && intr) {
                        const int it = m + off;
                        const int idxs = per ? L.rm : m;
                        if (idxs == L.sidx && L.wr == L.swr && L.wi == L.swi && L.S.m == L.sS.m && L.S.e == L.sS.e) break;
                        if (it - L.save_iter2 >= L.twin2 || L.conf_P > 0 || (((it + 1) & 15) == 0 && L.conf_giveup < 3)) break;
                    }
                    if (blat && m >= 2 && ((L.rm - 1) & blamask) == 0) {
                        if (!bmax) break;
                        const BlaMaxR2 r = bmax[(L.rm - 1) >> minlevel];
                        if (r.m != 0.0f) {
                            const Z wc2 = R::zabs2(L.wr, L.wi);
                            if (wc2 == Z(0)) break;
                            const TE<Z> dz2 = te_norm(R::z(L.S.m) * R::z(L.S.m) * wc2, 2 * L.S.e); // as lane_bla forms it
                            if (dz2.e < r.e || (dz2.e == r.e && dz2.m < r.m)) break;
                        }
                    }
                    if (tabs(L.Xc.x) < R::kTinyX && tabs(L.Xc.y) < R::kTinyX) break; // also m = 0 (X = 0)
                    int nrm = L.rm + 1;
                    if (per && nrm == per) nrm = 0;
                    const typename R::V2 X = orb[nrm];
                    T nwr, nwi;
                    E nerr2;
                    lane_step<T>(L.Xc, L.s, L.wr, L.wi, L.dr, L.di, L.err2, L.g2, nwr, nwi, nerr2);
                    const T zr = lane_zc<T>(X.x, L.s, nwr), zi = lane_zc<T>(X.y, L.s, nwi);
                    const Z zrad = R::zabs2(zr, zi);
                    const Z wm2 = R::zabs2(nwr, nwi);
                    const Z xr2 = R::zabs2(X.x, X.y);
                    const bool far = xr2 > Z(R::kTinyX) * Z(R::kTinyX) && s2x5 * wm2 < xr2;
                    // (|w| = 0 and the precision cap both leave through the
                    // |w|^2 tests: the general code handles them)
                    const bool rare = zrad > ESC2lo || !(nerr2 <= kLaneCap2 * (E)wm2) || wm2 > wmax2 || wm2 < wmin2 || !far;
                    if (rare) break;
                    if (deriv) lane_j_advance(L); // (from the pre-step state)
                    L.wr = nwr;
                    L.wi = nwi;
                    L.err2 = nerr2;
                    L.g2 = 4.0f * (E)zrad;
                    ++m;
                    L.rm = nrm;
                    L.Xc = X;
                    if (m >= mbud) break;
                }
                L.m = m;
                L.iter = m + off;
                n_steps += (unsigned)(m - m0);
                b += m - m0;
                if (b >= budget) return 0;
            }
        }
        if (L.iter >= g.mxit) return lane_interior(L);
        if (INTR && p.use_interior) {
            const int idxs = per ? L.rm : L.m;
            if (idxs == L.sidx && L.wr == L.swr && L.wi == L.swi && L.S.m == L.sS.m && L.S.e == L.sS.e) return lane_interior(L);
            if (L.iter - L.save_iter2 >= L.twin2) {
                L.swr = L.wr;
                L.swi = L.wi;
                L.sS = L.S;
                L.sidx = idxs;
                L.save_iter2 = L.iter;
                L.twin2 += L.twin2;
            }
        }
        if (blat && L.m >= 2 && ((L.rm - 1) & blamask) == 0) {
            float amp2 = 0.0f;
            BlaEntry<T> used;
            const int skip = lane_bla(f.bla, blat, orb, per > 0, L.rm, L.S, L.wr, L.wi, L.dcm, L.dce, ESC2lo, per ? per : reflen, amp2, deriv ? &used : nullptr);
            if (skip > 0) {
                if (deriv) lane_j_bla(L, used);
                ++n_bla;
                n_skip += skip;
                L.m += skip;
                L.iter += skip;
                L.rm += skip;
                if (per && L.rm >= per) L.rm -= per;
                lane_refresh(L);
                L.Xc = orb[L.rm];
                if (R::kTrackError) {
                    // the skip carries the error by A; |w| is 1 afterwards
                    L.err2 = L.err2 * amp2 + R::kEps2;
                    L.g2 = 4.0f * lane_abs2f(L.Xc);
                }
                L.zsr = L.zsi = 1e30;
                L.zsr_f = L.zsi_f = 1e30f;
                L.save_iter = L.iter;
                L.period_win = 1;
                L.conf_P = 0;
                L.conf_giveup = 0;
                continue;
            }
        }
        ++n_steps;
        // w' = (2 X_m + s w) w + d. Exact floatexp step where the lane type
        // would lose a term: the orbit entry below its range, or the first
        // step after a rebase (X = 0, |w| = 1) when s = |dz| is too small a
        // normal number, where dz^2 can be as large as dc (z ~ sqrt(minibrot
        // size) at a nucleus pass).
        const bool tiny = (L.m == 0 && !(L.s >= R::kMinS)) ||
                          (L.m != 0 && tabs(L.Xc.x) < R::kTinyX && tabs(L.Xc.y) < R::kTinyX && !(d_is_zero(Zfe[L.rm].re.m) && d_is_zero(Zfe[L.rm].im.m)));
        if (deriv) { // J' = 2 z J + 1 with the pre-step z (mp.cpp:3436-3441, 3478-3497)
            if (!tiny) {
                lane_j_advance(L);
            } else { // z outside the lane type's range: in floatexp
                const FE zero = fe_make(0.0, 0);
                const FE S0 = fe_from_te(L.S);
                lane_j_step_fe(L, fe_add(L.m ? Zfe[L.rm].re : zero, fe_mul_d(S0, (double)L.wr)), fe_add(L.m ? Zfe[L.rm].im : zero, fe_mul_d(S0, (double)L.wi)));
            }
        }
        if (!tiny) {
            T nwr, nwi;
            typename R::E nerr2;
            lane_step<T>(L.Xc, L.s, L.wr, L.wi, L.dr, L.di, L.err2, L.g2, nwr, nwi, nerr2);
            L.wr = nwr;
            L.wi = nwi;
            L.err2 = nerr2;
        } else if constexpr (std::is_same<T, float>::value) {
            ++n_exact;
            const F32E S0 = L.S;
            const F32E zero{0.0f, 0};
            const F32E Xr = L.m ? te_from_fe_f(Zfe[L.rm].re) : zero, Xi = L.m ? te_from_fe_f(Zfe[L.rm].im) : zero;
            F32E S = S0;
            float wr = L.wr, wi = L.wi;
            exact_step_f(Xr, Xi, te_norm(L.dcm.x, L.dce), te_norm(L.dcm.y, L.dce), S, wr, wi);
            if (R::kTrackError) {
                // error carried into the new units: |2 z|^2 (S0 / S)^2 err2, z = X + S0 w
                const F32E zr = te_add_f(Xr, te_norm(S0.m * L.wr, S0.e)), zi = te_add_f(Xi, te_norm(S0.m * L.wi, S0.e));
                const int ez = zr.m == 0.0f ? zi.e : (zi.m == 0.0f ? zr.e : imax(zr.e, zi.e));
                const float mr = te_align_f(zr.m, zr.e, ez), mi = te_align_f(zi.m, zi.e, ez);
                const float q = S.m == 0.0f ? 0.0f : S0.m / S.m;
                const float amp = ldexp_ftz(4.0f * (mr * mr + mi * mi) * q * q, imax(-300, imin(300, 2 * ez + 2 * (S0.e - S.e))));
                L.err2 = fminf(amp * L.err2, 3e38f) + R::kEps2;
            }
            L.S = S;
            L.wr = wr;
            L.wi = wi;
            lane_refresh(L);
        } else if constexpr (std::is_same<T, df32>::value) {
            ++n_exact;
            const TE<df32> S0 = L.S;
            const TE<df32> zero{df32(0.0f), 0};
            const TE<df32> Xr = L.m ? te_from_fe_df(Zfe[L.rm].re) : zero, Xi = L.m ? te_from_fe_df(Zfe[L.rm].im) : zero;
            TE<df32> S = S0;
            df32 wr = L.wr, wi = L.wi;
            exact_step_df(Xr, Xi, te_norm(L.dcm.x, L.dce), te_norm(L.dcm.y, L.dce), S, wr, wi);
            if (R::kTrackError) {
                // error carried into the new units: |2 z|^2 (S0 / S)^2 err2, z = X + S0 w
                const TE<df32> zr = te_add_df(Xr, te_norm(S0.m * L.wr, S0.e)), zi = te_add_df(Xi, te_norm(S0.m * L.wi, S0.e));
                const int ez = zr.m.hi == 0.0f ? zi.e : (zi.m.hi == 0.0f ? zr.e : imax(zr.e, zi.e));
                const float mr = te_align_df(zr.m, zr.e, ez).hi, mi = te_align_df(zi.m, zi.e, ez).hi;
                const float q = S.m.hi == 0.0f ? 0.0f : S0.m.hi / S.m.hi;
                const float amp = ldexp_ftz(4.0f * (mr * mr + mi * mi) * q * q, imax(-300, imin(300, 2 * ez + 2 * (S0.e - S.e))));
                L.err2 = fminf(amp * L.err2, 3e38f) + R::kEps2;
            }
            L.S = S;
            L.wr = wr;
            L.wi = wi;
            lane_refresh(L);
        } else {
            ++n_exact;
            double wr = (double)L.wr, wi = (double)L.wi;
            const FE S0 = fe_from_te(L.S);
            FE S = S0;
            const FE zero = fe_make(0.0, 0);
            const FE Xr = L.m ? Zfe[L.rm].re : zero, Xi = L.m ? Zfe[L.rm].im : zero;
            exact_step(Xr, Xi, lane_dc_re(p, L), lane_dc_im(p, L), S, wr, wi);
            if (R::kTrackError) {
                // error carried into the new units: |2 z|^2 (S0 / S)^2 err2,
                // z = X + S0 w in floatexp (z may lie below FP32's range)
                const FE zr = fe_add(Xr, fe_mul_d(S0, (double)L.wr)), zi = fe_add(Xi, fe_mul_d(S0, (double)L.wi));
                const FE z2 = fe_add(fe_mul(zr, zr), fe_mul(zi, zi));
                const FE q = fe_div(S0, S);
                const double amp = S.m == 0.0 ? 0.0 : 4.0 * fe_to_double(fe_mul(z2, fe_mul(q, q)));
                L.err2 = (typename R::E)fmin(amp * (double)L.err2, (double)R::kErrMax) + R::kEps2;
            }
            L.S = te_from_fe<T>(S);
            L.wr = (T)wr;
            L.wi = (T)wi;
            lane_refresh(L);
        }
        ++L.m;
        ++L.iter;
        ++L.rm;
        if (per && L.rm == per) L.rm = 0;
        L.Xc = orb[L.rm];
        const T zr = lane_zc<T>(L.Xc.x, L.s, L.wr), zi = lane_zc<T>(L.Xc.y, L.s, L.wi);
        const Z zrad = R::zabs2(zr, zi);
        if (zrad > ESC2lo) {
            Z zesc = zrad;
            bool esc = zrad > ESC2hi;
            if (!esc) {
                double zdr, zdi;
                lane_z_double(L, Zd, zdr, zdi);
                const double zr2 = zdr * zdr + zdi * zdi;
                esc = zr2 > g.ESC2;
                zesc = (Z)zr2;
            }
            if (esc) {
                zrad_out = T(zesc);
                if (R::kTrackError) {
                    // Keep N only if the estimated error of |z|^2 (2 rho |dz| / |z|,
                    // doubled) cannot carry |z_N|^2 or |z_(N-1)|^2 across the bailout.
                    const float sf = R::tof(L.s), wrf = R::tof(L.wr), wif = R::tof(L.wi), zf = (float)zesc, Ef = (float)ESC2z;
                    const float dzm2 = sf * sf * (wrf * wrf + wif * wif);
                    const float amb = 4.0f * sqrtf((float)lane_rel_err2(L.err2, L.wr, L.wi) * dzm2 / zf);
                    if (!(zf >= Ef * (1.0f + amb)) || !(0.25f * L.g2 <= Ef * (1.0f - amb))) return 5; // (a NaN estimate fails too)
                    if (deriv && !((float)lane_rel_err2(L.err2, L.wr, L.wi) <= kLaneDeTol2)) return 5;
                }
                L.ezr = zr;
                L.ezi = zi;
                return 1;
            }
        }
        if (INTR && p.use_interior) {
            if (L.conf_P > 0) {
                L.conf_D2 *= 4.0f * (float)zrad;
                if (L.conf_D2 > 1e18f) L.conf_D2 = 1e18f;
                if (L.iter >= L.conf_next) {
                    double zdr, zdi;
                    lane_z_double(L, Zd, zdr, zdi);
                    const double qr = zdr - L.conf_zr, qi = zdi - L.conf_zi;
                    if (qr * qr + qi * qi < p.interior_eps2 * (zdr * zdr + zdi * zdi) && L.conf_D2 < 1.0f) {
                        if (++L.conf_count >= p.interior_confirm) return lane_interior(L);
                        L.conf_zr = zdr;
                        L.conf_zi = zdi;
                        L.conf_D2 = 1.0f;
                        L.conf_next = L.iter + L.conf_P;
                    } else {
                        L.conf_P = 0;
                        ++L.conf_giveup;
                    }
                }
            } else if ((L.iter & 15) == 0 && L.conf_giveup < 3) {
                const float zrf = R::tof(zr), zif = R::tof(zi);
                const float qr = zrf - L.zsr_f, qi = zif - L.zsi_f;
                const bool maybe = qr * qr + qi * qi < 1e-11f * (float)zrad;
                const bool save = L.iter - L.save_iter >= L.period_win;
                if (maybe || save) {
                    double zdr, zdi;
                    lane_z_double(L, Zd, zdr, zdi);
                    if (maybe) {
                        const double dqr = zdr - L.zsr, dqi = zdi - L.zsi;
                        if (dqr * dqr + dqi * dqi < p.interior_eps2 * (zdr * zdr + zdi * zdi)) {
                            L.conf_P = imax(L.iter - L.save_iter, 1);
                            L.conf_zr = zdr;
                            L.conf_zi = zdi;
                            L.conf_D2 = 1.0f;
                            L.conf_next = L.iter + L.conf_P;
                            L.conf_count = 0;
                        }
                    }
                    if (save) {
                        L.zsr = zdr;
                        L.zsi = zdi;
                        L.zsr_f = zrf;
                        L.zsi_f = zif;
                        L.save_iter = L.iter;
                        L.period_win += L.period_win;
                    }
                }
            }
        }
        if (R::kTrackError) L.g2 = 4.0f * (typename R::E)zrad;
        // keep |w| ~ 1 (rescale window [1/wmax2, wmax2], autotuned); the scale
        // factor only needs to be near |w|, as long as S and w change by it
        // and its exact reciprocal
        const Z wm2 = R::zabs2(L.wr, L.wi);
        if (R::kTrackError && wm2 > Z(0) && !(L.err2 <= kLaneCap2 * (typename R::E)wm2)) return 3; // precision spent (or a NaN estimate)
        if (wm2 > Z(p.wmax2) || (wm2 < Z(p.wmin2) && wm2 > Z(0))) {
            // |w| fell below the type's floor in one step (a near-zero |2 z|):
            // the absolute estimate err2 ~ |w|^2 may have left the normal range
            if (R::kTrackError && wm2 < Z(R::kWFloor)) return 3;
            if constexpr (std::is_same<T, float>::value) {
                lane_rescale_pow2(L, wm2); // exact, as the common-step loop does it
            } else {
                const T wmag = T(tsqrt(wm2)), inv = T(1) / wmag;
                L.S = te_mulr(L.S, wmag);
                L.wr *= inv;
                L.wi *= inv;
                // err2 in the new units: err2 inv^2 = err2 / |w|^2 (no overflow of inv^2)
                if (R::kTrackError) L.err2 = L.err2 / (typename R::E)wm2;
                lane_refresh(L);
            }
        }
        // Rebase (mp.cpp:3584-3615): |z|^2 < |dz|^2 decided on floatexp with a
        // 1e-4 margin; FP64 floatexp inside the margin, for strong
        // cancellation in X + dz, and at the end of the reference.
        const int decide = lane_rebase_decision<T>(L.S, L.s, L.wr, L.wi, L.Xc, L.m, zrad, per, reflen);
        const TE<T> S0 = L.S;
        if (decide == 1) {
            lane_rebase_to(L, zr, zi);
            ++n_rebase;
        } else if (decide == 2 && std::is_same<T, float>::value) {
            // the decision and the new delta in FP32 floatexp: z = X + S w
            // per component, |z| against |dz| on mantissa/exponent pairs
            ++n_ferebase;
            const F32E zero{0.0f, 0};
            const F32E Xr = L.m ? te_from_fe_f(Zfe[L.rm].re) : zero, Xi = L.m ? te_from_fe_f(Zfe[L.rm].im) : zero;
            const float Sm = R::tof(L.S.m), wrf = R::tof(L.wr), wif = R::tof(L.wi);
            const F32E zr = te_add_f(Xr, te_norm(Sm * wrf, L.S.e)), zi = te_add_f(Xi, te_norm(Sm * wif, L.S.e));
            const int ez = zr.m == 0.0f ? zi.e : (zi.m == 0.0f ? zr.e : imax(zr.e, zi.e));
            const float mr = te_align_f(zr.m, zr.e, ez), mi = te_align_f(zi.m, zi.e, ez);
            const float mz = sqrtf(mr * mr + mi * mi);
            const F32E zn = te_norm(mz, ez), dn = te_norm(fabsf(Sm) * sqrtf(wrf * wrf + wif * wif), L.S.e);
            const bool smaller = zn.m == 0.0f ? dn.m != 0.0f : (dn.m != 0.0f && (zn.e < dn.e || (zn.e == dn.e && zn.m < dn.m)));
            if ((!per && L.m >= reflen) || smaller) {
                if (mz == 0.0f) {
                    L.wr = L.wi = T(0);
                } else {
                    L.S = TE<T>{T(zn.m), zn.e};
                    L.wr = T(mr / mz);
                    L.wi = T(mi / mz);
                    lane_refresh(L);
                    if (R::kTrackError) {
                        // plus the roundings of X + dz in float, relative to |z|:
                        // (|X|^2 + |dz|^2) / |z|^2 times the per-step variance
                        const int ex = Xr.m == 0.0f ? Xi.e : (Xi.m == 0.0f ? Xr.e : imax(Xr.e, Xi.e));
                        const float ar = te_align_f(Xr.m, Xr.e, ex), ai = te_align_f(Xi.m, Xi.e, ex);
                        const float cx = (Xr.m == 0.0f && Xi.m == 0.0f) ? 0.0f : ldexp_ftz((ar * ar + ai * ai) / (mz * mz), imax(-300, imin(300, 2 * (ex - ez))));
                        const float cd = ldexp_ftz(Sm * Sm * (wrf * wrf + wif * wif) / (mz * mz), imax(-300, imin(300, 2 * (S0.e - ez))));
                        L.err2 = L.err2 * lane_scale_ratio2(S0, L.S) + R::kEps2 * (1.0f + fminf(cx + cd, 1e30f));
                    }
                }
                L.m = 0;
                L.rm = -1;
                L.Xc = R::make2(T(0), T(0));
                ++n_rebase;
            }
        } else if (decide == 2) {
            ++n_ferebase;
            const FE S = fe_from_te(L.S);
            FE Xmr = L.m ? Zfe[L.rm].re : fe_make(0.0, 0);
            FE Xmi = L.m ? Zfe[L.rm].im : fe_make(0.0, 0);
            FE Swr = fe_mul_d(S, (double)L.wr), Swi = fe_mul_d(S, (double)L.wi);
            FE zrfe = fe_add(Xmr, Swr), zife = fe_add(Xmi, Swi);
            FE zradfe = fe_add(fe_mul(zrfe, zrfe), fe_mul(zife, zife));
            FE dzfe = fe_add(fe_mul(Swr, Swr), fe_mul(Swi, Swi));
            if ((!per && L.m >= reflen) || fe_abs_less(zradfe, dzfe)) {
                FE Snew = fe_sqrt(zradfe);
                if (Snew.m == 0.0) {
                    L.wr = L.wi = T(0);
                } else {
                    L.S = te_from_fe<T>(Snew);
                    L.wr = (T)fe_to_double(fe_div(zrfe, Snew));
                    L.wi = (T)fe_to_double(fe_div(zife, Snew));
                    lane_refresh(L);
                    if (R::kTrackError) L.err2 = L.err2 * lane_scale_ratio2(S0, L.S) + R::kEps2;
                }
                L.m = 0;
                L.rm = -1;
                L.Xc = R::make2(T(0), T(0));
                ++n_rebase;
            }
        }
    }
    return 0;
}

} // namespace mbx

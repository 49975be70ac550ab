// ORACLE — test infrastructure only. CPU restatement of the reference
// engine's quadratic-Mandelbrot perturbation path (cbotx/Mandelbrot-Explorer,
// src/engine/mandel_perturbation.cpp, "mp.cpp" below) used to check the CUDA
// renderer. Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
// reference legs may load it; the product never does.
//
// Scope: Mandel::Compute for coloring flags {0, SUPER_SAMPLING, EXTERIOR_DIST_EST, STRIPE_AVERAGE, ORBIT_TRAP,
// DE_OVERLAY} with the reference's default engine switches (BLA on, interior
// detection on, floatexp gate at scale > 1e280, periodic reference auto,
// BigFixed auto, fused rescaled step). The per-pixel loops follow the scalar
// reference semantics (mp.cpp's AVX2 kernels are documented there as bit-identical
// to the scalar loops) except where the reference itself routes to a kernel with
// different semantics (solveRescaledSimd8NoBla), which is restated separately.
//
// Pinning: tests/golden/make_golden.py renders fixtures with the reference engine
// itself compiled here (oracle/ref_build), and tests compare this file against them
// bit for bit. All arithmetic is compiled with -ffp-contract=off so that the
// operation order below is the operation order executed.
#include "oracle_gmp.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr float EMPTY = -10.0f; // mp.h:23 EMPTYPIXEL
constexpr int CM_SS = 1, CM_EDE = 2, CM_SAC = 8, CM_NORMAL = 16, CM_TRAP = 32, CM_DEOVL = 64; // mp.h:30-49

// Orbit colourings (src/engine/orbit_coloring.h:21-132): the stripe average
// over a triangular window of the last 256 terms 1/2 + sin(7 arg z)/2, and the
// orbit traps (min distance to 0, the cross weighted 1.5, the circle |z| = 1/2).
struct OrbitAcc {
    static constexpr int W = 256;
    bool sac = false, trap = false;
    double ring[W];
    double RS = 0, TS = 0, last = 0;
    int pos = 0, fill = 0;
    double minP = 1e300, minX = 1e300, minC = 1e300;
    void init(int cm) {
        sac = (cm & CM_SAC) != 0;
        trap = (cm & CM_TRAP) != 0;
        RS = TS = last = 0;
        pos = fill = 0;
        minP = minX = minC = 1e300;
    }
    void push(double zr, double zi) {
        if (sac) {
            double t = 0.5 + 0.5 * std::sin(7.0 * std::atan2(zi, zr));
            last = t;
            double ev = fill == W ? ring[pos] : (++fill, 0.0);
            TS += (double)W * t - RS;
            RS += t - ev;
            ring[pos] = t;
            pos = (pos + 1) % W;
        }
        if (trap) {
            double m2 = zr * zr + zi * zi;
            if (m2 < minP) minP = m2;
            double x = std::min(std::fabs(zr), std::fabs(zi));
            if (x < minX) minX = x;
            double c = std::fabs(std::sqrt(m2) - 0.5);
            if (c < minC) minC = c;
        }
    }
    void skipped() { // a BLA jump breaks the stripe window
        if (sac) {
            RS = TS = 0;
            pos = fill = 0;
        }
    }
    float sacValue(double zrad, double radius) const {
        double f = 1.0 - std::log(std::log(zrad) * 0.5 / std::log(radius)) / std::log(2.0);
        double w = (double)fill * W - (double)fill * (fill - 1) / 2.0;
        double inc = w > 0.0 ? TS / w : 0.0;
        double exc = w > (double)W ? (TS - (double)W * last) / (w - (double)W) : inc;
        f -= std::floor(f);
        return (float)(exc + (inc - exc) * f);
    }
    float trapValue(double mu) const {
        double d = std::min(std::min(std::sqrt(minP), minX * 1.5), minC);
        if (d > 1.0) d = 1.0;
        double tr = -std::log10(std::max(d, 1e-14));
        if (mu < 0.0) mu = 0.0;
        return (float)(0.17 * tr + 0.025 * mu);
    }
    // the loops' escape value when no DE/normal/overlay colouring applies: trap first
    float escaped(double mu, double zrad, double radius) const { return trap ? trapValue(mu) : sacValue(zrad, radius); }
    float interior() const { return trap ? trapValue(0.0) : -2.0f; }
};
constexpr int SA_N = 30;                            // mp.h:288

// ---------------------------------------------------------------------------
// FloatExp (src/engine/floatexp.h:17-107): m * 2^e, 0.5 <= |m| < 1.
struct FE {
    double m;
    int64_t e;
};
static inline FE fe_from(double x) {
    if (x == 0.0) return FE{0.0, 0};
    int ex;
    double mm = std::frexp(x, &ex);
    return FE{mm, (int64_t)ex};
}
static inline double fe_to_double(FE a) {
    if (a.m == 0.0) return 0.0;
    if (a.e > 1100) return a.m > 0 ? INFINITY : -INFINITY;
    if (a.e < -1100) return 0.0;
    return std::ldexp(a.m, (int)a.e);
}
static inline FE fe_renorm(double m, int64_t e) {
    if (m == 0.0) return FE{0.0, 0};
    int ex;
    double mm = std::frexp(m, &ex);
    return FE{mm, e + ex};
}
static inline FE fe_mul(FE a, FE b) {
    if (a.m == 0.0 || b.m == 0.0) return FE{0.0, 0};
    return fe_renorm(a.m * b.m, a.e + b.e);
}
static inline FE fe_mul_d(FE a, double b) {
    if (a.m == 0.0 || b == 0.0) return FE{0.0, 0};
    return fe_renorm(a.m * b, a.e);
}
static inline FE fe_scale2(FE a, int64_t k) { return a.m == 0.0 ? a : FE{a.m, a.e + k}; }
static inline FE fe_add(FE a, FE b) {
    if (a.m == 0.0) return b;
    if (b.m == 0.0) return a;
    int64_t d = a.e - b.e;
    if (d > 54) return a;
    if (d < -54) return b;
    if (d >= 0) return fe_renorm(a.m + std::ldexp(b.m, -(int)d), a.e);
    return fe_renorm(b.m + std::ldexp(a.m, (int)d), b.e);
}
static inline FE fe_neg(FE a) { return FE{-a.m, a.e}; }
static inline FE fe_sub(FE a, FE b) { return fe_add(a, fe_neg(b)); }
static inline FE fe_div(FE a, FE b) {
    if (a.m == 0.0) return FE{0.0, 0};
    return fe_renorm(a.m / b.m, a.e - b.e);
}
static inline bool fe_abs_less(FE a, FE b) {
    if (a.m == 0.0) return b.m != 0.0;
    if (b.m == 0.0) return false;
    if (a.e != b.e) return a.e < b.e;
    return std::fabs(a.m) < std::fabs(b.m);
}
static inline FE fe_sqrt(FE a) {
    if (a.m <= 0.0) return FE{0.0, 0};
    int64_t e = a.e;
    double m = a.m;
    if (e & 1) {
        m *= 2.0;
        --e;
    }
    return fe_renorm(std::sqrt(m), e / 2);
}

// ---------------------------------------------------------------------------
// std::complex<double> arithmetic as GCC evaluates it for finite operands:
// multiply inline (a*c-b*d, a*d+b*c); divide through libgcc's __divdc3, whose
// scaled Smith algorithm is restated here (checked bit-identical against
// std::complex division on finite inputs).
struct C2 {
    double re, im;
};
static inline C2 c_add(C2 a, C2 b) { return C2{a.re + b.re, a.im + b.im}; }
static inline C2 c_mul(C2 x, C2 y) { return C2{x.re * y.re - x.im * y.im, x.re * y.im + x.im * y.re}; }
static inline C2 c_div(C2 num, C2 den) {
    double a = num.re, b = num.im, c = den.re, d = den.im;
    const double RBIG = DBL_MAX / 2, RMIN = DBL_MIN, RMIN2 = DBL_EPSILON, RMINSCAL = 1.0 / DBL_EPSILON, RMAX2 = RBIG * RMIN2;
    double ratio, denom, x, y;
    if (std::fabs(c) < std::fabs(d)) {
        if (std::fabs(d) >= RBIG) { a /= 2; b /= 2; c /= 2; d /= 2; }
        if (std::fabs(d) < RMIN2) {
            a *= RMINSCAL; b *= RMINSCAL; c *= RMINSCAL; d *= RMINSCAL;
        } else if ((std::fabs(a) < RMIN && std::fabs(b) < RMAX2 && std::fabs(d) < RMAX2) || (std::fabs(b) < RMIN && std::fabs(a) < RMAX2 && std::fabs(d) < RMAX2)) {
            a *= RMINSCAL; b *= RMINSCAL; c *= RMINSCAL; d *= RMINSCAL;
        }
        ratio = c / d;
        denom = (c * ratio) + d;
        if (std::fabs(ratio) > RMIN) {
            x = ((a * ratio) + b) / denom;
            y = ((b * ratio) - a) / denom;
        } else {
            x = ((c * (a / d)) + b) / denom;
            y = ((c * (b / d)) - a) / denom;
        }
    } else {
        if (std::fabs(c) >= RBIG) { a /= 2; b /= 2; c /= 2; d /= 2; }
        if (std::fabs(c) < RMIN2) {
            a *= RMINSCAL; b *= RMINSCAL; c *= RMINSCAL; d *= RMINSCAL;
        } else if ((std::fabs(a) < RMIN && std::fabs(b) < RMAX2 && std::fabs(c) < RMAX2) || (std::fabs(b) < RMIN && std::fabs(a) < RMAX2 && std::fabs(c) < RMAX2)) {
            a *= RMINSCAL; b *= RMINSCAL; c *= RMINSCAL; d *= RMINSCAL;
        }
        ratio = d / c;
        denom = (d * ratio) + c;
        if (std::fabs(ratio) > RMIN) {
            x = ((b * ratio) + a) / denom;
            y = (b - (a * ratio)) / denom;
        } else {
            x = (a + (d * (b / c))) / denom;
            y = (b - (d * (a / c))) / denom;
        }
    }
    return C2{x, y};
}

// mpf -> double, truncating (src/engine/float_math.cpp:13-17).
static inline double mpf_ld(mpf_srcptr a) {
    long e;
    double d = mpf_get_d_2exp(&e, a);
    return std::ldexp(d, (int)e);
}
// mpf -> FloatExp (mp.cpp:69-74).
static inline FE mpf_fe(mpf_srcptr x) {
    if (mpf_sgn(x) == 0) return FE{0.0, 0};
    long ex;
    double d = mpf_get_d_2exp(&ex, x);
    return FE{d, (int64_t)ex};
}
// floor(log2|x|) (float_math.cpp:22-27) for SA magnitude checks.
static inline int exp_of(double x) {
    if (x == 0.0) return -0x40000000;
    int e;
    (void)std::frexp(x, &e);
    return e - 1;
}

// ---------------------------------------------------------------------------
// Fixed-point big real (src/engine/bigfixed.h): L little-endian 64-bit limbs,
// binary point below the top limb, sign-magnitude, round-to-nearest multiply.
struct BF {
    int L = 0;
    int sign = 0;
    std::vector<uint64_t> m;
    void setL(int l) {
        L = l;
        sign = 0;
        m.assign((size_t)l, 0ull);
    }
};
typedef unsigned __int128 u128;
static int bf_cmp(const uint64_t* a, const uint64_t* b, int L) {
    for (int i = L - 1; i >= 0; --i)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}
static void bf_addm(uint64_t* r, const uint64_t* a, const uint64_t* b, int L) {
    uint64_t c = 0;
    for (int i = 0; i < L; ++i) {
        u128 s = (u128)a[i] + b[i] + c;
        r[i] = (uint64_t)s;
        c = (uint64_t)(s >> 64);
    }
}
static void bf_subm(uint64_t* r, const uint64_t* a, const uint64_t* b, int L) {
    uint64_t br = 0;
    for (int i = 0; i < L; ++i) {
        uint64_t ai = a[i], bi = b[i];
        uint64_t d = ai - bi - br;
        br = (ai < bi) || (ai - bi < br) ? 1 : 0;
        r[i] = d;
    }
}
static void bf_addsub(BF& r, const BF& a, int sa, const BF& b, int sb) {
    const int L = a.L;
    r.L = L;
    if ((int)r.m.size() != L) r.m.resize(L);
    if (sa == 0) {
        std::memcpy(r.m.data(), b.m.data(), 8 * (size_t)L);
        r.sign = sb;
        return;
    }
    if (sb == 0) {
        std::memcpy(r.m.data(), a.m.data(), 8 * (size_t)L);
        r.sign = sa;
        return;
    }
    if (sa == sb) {
        bf_addm(r.m.data(), a.m.data(), b.m.data(), L);
        r.sign = sa;
        return;
    }
    int c = bf_cmp(a.m.data(), b.m.data(), L);
    if (c == 0) {
        std::fill(r.m.begin(), r.m.end(), 0ull);
        r.sign = 0;
    } else if (c > 0) {
        bf_subm(r.m.data(), a.m.data(), b.m.data(), L);
        r.sign = sa;
    } else {
        bf_subm(r.m.data(), b.m.data(), a.m.data(), L);
        r.sign = sb;
    }
}
// Add row a_i * b[jstart..L) into acc at offset t, carrying to index <= top.
static void bf_row(uint64_t* acc, int t, const uint64_t* b, int n, uint64_t ai, int top) {
    uint64_t carry = 0;
    for (int j = 0; j < n; ++j) {
        u128 p = (u128)ai * b[j] + acc[t + j] + carry;
        acc[t + j] = (uint64_t)p;
        carry = (uint64_t)(p >> 64);
    }
    for (int u = t + n; carry && u <= top; ++u) {
        u128 s = (u128)acc[u] + carry;
        acc[u] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
    }
}
// bigfixed.h:106-125: high-half (16 <= L < 72, 3 guard limbs) or full product,
// keep limbs [L-1, 2L-1), round on the top dropped bit.
static void bf_mulshift(uint64_t* r, const uint64_t* a, const uint64_t* b, int L, uint64_t* tmp) {
    if (L >= 16 && L < 72) {
        const int G = 3, lo = L - 1 - G, nout = 2 * L - lo;
        std::memset(tmp, 0, 8 * (size_t)(nout + 1));
        for (int i = 0; i < L; ++i) {
            int js = lo - i;
            if (js < 0) js = 0;
            bf_row(tmp, i + js - lo, b + js, L - js, a[i], nout);
        }
        for (int i = 0; i < L; ++i) r[i] = tmp[i + G];
        if (tmp[G - 1] >> 63)
            for (int i = 0; i < L; ++i)
                if (++r[i] != 0) break;
        return;
    }
    std::memset(tmp, 0, 8 * (size_t)(2 * L));
    for (int i = 0; i < L; ++i) bf_row(tmp, i, b, L, a[i], 2 * L - 1);
    const int drop = L - 1;
    for (int i = 0; i < L; ++i) r[i] = tmp[drop + i];
    if (drop > 0 && (tmp[drop - 1] >> 63))
        for (int i = 0; i < L; ++i)
            if (++r[i] != 0) break;
}
static void bf_mul(BF& r, const BF& a, const BF& b, uint64_t* tmp) {
    const int L = a.L;
    r.L = L;
    if ((int)r.m.size() != L) r.m.resize(L);
    if (a.sign == 0 || b.sign == 0) {
        std::fill(r.m.begin(), r.m.end(), 0ull);
        r.sign = 0;
        return;
    }
    bf_mulshift(r.m.data(), a.m.data(), b.m.data(), L, tmp);
    r.sign = (a.sign == b.sign) ? 1 : -1;
}
// bigfixed.h:283-299: truncate |x| * 2^(64(L-1)) to an integer.
static void bf_from_mpf(BF& a, mpf_srcptr x, int L) {
    a.setL(L);
    if (mpf_sgn(x) == 0) return;
    a.sign = mpf_sgn(x);
    const int n = x->_mp_size < 0 ? -x->_mp_size : x->_mp_size;
    for (int i = 0; i < n; ++i) {
        long k = (long)i - n + x->_mp_exp + L - 1;
        if (k >= 0 && k < L) a.m[k] = x->_mp_d[i];
    }
}
// bigfixed.h:272-280.
static void bf_to_mpf(mpf_ptr out, const BF& a) {
    mpz_t z;
    mpz_init(z);
    mpz_import(z, (size_t)a.L, -1, sizeof(uint64_t), 0, 0, a.m.data());
    mpf_set_z(out, z);
    mpf_div_2exp(out, out, (mp_bitcnt_t)64 * (a.L - 1));
    if (a.sign < 0) mpf_neg(out, out);
    mpz_clear(z);
}
// bigfixed.h:305-320.
static FE bf_to_fe(const BF& a) {
    if (a.sign == 0) return FE{0.0, 0};
    int top = a.L - 1;
    while (top >= 0 && a.m[top] == 0) --top;
    if (top < 0) return FE{0.0, 0};
    double mant = (double)a.m[top] * 18446744073709551616.0 + (double)(top >= 1 ? a.m[top - 1] : 0ull);
    FE r = fe_from(mant);
    r.e += (int64_t)64 * (top - a.L);
    return a.sign < 0 ? fe_neg(r) : r;
}

// ---------------------------------------------------------------------------
struct Opts {
    int bla = 1;          // MANDEL_BLA
    int bla_minskip = 8;  // MANDEL_BLA_MINSKIP
    double bla_eps = 0.0; // MANDEL_BLA_EPS (0 -> 2^-53)
    int interior = 1;     // MANDEL_INTERIOR
    double int_eps = 3e-9;
    int int_confirm = 4;
    int int_rep = 1;
    int fe = -1;       // MANDEL_FE: -1 auto (scale > 1e280)
    int periodic = -1; // MANDEL_PERIODIC
    int bigfixed = -1; // MANDEL_BIGFIXED
    int fused = 1;     // MANDEL_FUSED_PERTURB
    double ss_k = 8.0; // MANDEL_SS_K
    double sac_ss_steps = 0.0;  // MANDEL_SAC_SS_STEPS (0: the set boundary only)
    double trap_ss_steps = 3.0; // MANDEL_TRAP_SS_STEPS
    float ss_density = 60.0f;   // Mandel::_ss_density (setDensity; the compute backend leaves the default)
};

struct Pix {
    int a[4]; // {row, col, subrow, subcol} exactly like the reference's std::array<int,4>
};

class Engine {
  public:
    Engine(int w, int h, int mxit, int sub, float* iter, float* normal, int32_t* escn, double bailout, const Opts& o)
        : W(w), H(h), MXIT(mxit), SUB(sub), iter_(iter), normal_(normal), escn_(escn), opt(o) {
        escf = (float)bailout;
        ESC2 = (double)(escf * escf); // mp.h:115-118: float*float, widened
        zfr.resize(MXIT + 1);
        zfi.resize(MXIT + 1);
        zfr_fe.resize(MXIT + 1);
        zfi_fe.resize(MXIT + 1);
        dfr.resize(MXIT + 1);
        dfi.resize(MXIT + 1);
        z_m3.resize(MXIT + 1);
        mpf_init(c0_re); mpf_init(c0_im); mpf_init(dx); mpf_init(dy); mpf_init(scale_);
        mpf_init(ref_re); mpf_init(ref_im); mpf_init(t1); mpf_init(t2);
        for (int i = 0; i < 2; ++i) { mpf_init(zre[i]); mpf_init(zim[i]); }
    }
    ~Engine() {
        mpf_clear(c0_re); mpf_clear(c0_im); mpf_clear(dx); mpf_clear(dy); mpf_clear(scale_);
        mpf_clear(ref_re); mpf_clear(ref_im); mpf_clear(t1); mpf_clear(t2);
        for (int i = 0; i < 2; ++i) { mpf_clear(zre[i]); mpf_clear(zim[i]); }
    }
    void setPrecision(int p) { // mp.cpp:2030-2045
        mpf_set_prec(c0_re, p); mpf_set_prec(c0_im, p); mpf_set_prec(dx, p); mpf_set_prec(dy, p);
        mpf_set_prec(scale_, p); mpf_set_prec(ref_re, p); mpf_set_prec(ref_im, p);
        mpf_set_prec(t1, p); mpf_set_prec(t2, p);
        for (int i = 0; i < 2; ++i) { mpf_set_prec(zre[i], p); mpf_set_prec(zim[i], p); }
    }
    void compute(mpf_srcptr cre, mpf_srcptr cim, mpf_srcptr scale, int mxit, int cm, int full_h, int row_base);
    // Brute-force arbitrary-precision value of listed samples on the frame
    // grid (ComputeDirect semantics, mp.cpp:959-990, at `wp` bits).
    void truth(mpf_srcptr c_re, mpf_srcptr c_im, mpf_srcptr scale, int full_h, int row_base, int mxit, int cm, const int* keys, int n, int wp, float* out, int* nout);

    long long stat_steps = 0, stat_bla = 0, stat_skipped = 0, stat_passes = 0, stat_refs = 0, stat_gmp = 0;
    int method = 0;

  private:
    const int W, H, MXIT, SUB;
    float* iter_;
    float* normal_;
    int32_t* escn_; // escape iteration N per sample (instrumentation; -1 interior)
    Opts opt;
    float escf;
    double ESC2;
    mpf_t c0_re, c0_im, dx, dy, scale_, ref_re, ref_im, t1, t2;
    mpf_t zre[2], zim[2];
    std::vector<double> zfr, zfi, dfr, dfi, z_m3;
    std::vector<FE> zfr_fe, zfi_fe;
    FE dfe_r{1.0, 0}, dfe_i{0.0, 0};
    C2 Adf_old[SA_N], Adf_new[SA_N], Bdf_old[SA_N], Bdf_new[SA_N], SA_delta{0, 0};
    bool SA_flag = false;
    int SA_order = 0, SA_it = 0;
    // BLA (mp.h:193-206)
    std::vector<std::vector<double>> bla_r2;
    std::vector<std::vector<std::array<double, 4>>> bla_ab, bla_ce;
    double bla_rmax2 = 0.0, bla_dcmax2 = 0.0, bla_eps = 0.0;
    bool use_bla = false;
    int bla_minlevel = 0;
    bool ref_bounded = false, ref_escaped = false;
    int ref_escape_iteration = 0;
    bool use_interior = false;
    double interior_eps2 = 0.0;
    int interior_confirm = 4;
    bool use_floatexp = false, fe_cutoff_sensitive = false;
    FE dxfe{0, 0}, dyfe{0, 0};
    Pix ref_{{0, 0, 0, 0}}, new_ref{{-1, -1, -1, -1}};
    double ref_x = 0.0, ref_y = 0.0;
    bool ref_virtual = false;
    int ref_period = 0;
    bool ref_subpixel = false, ref_deep_zero = false;
    double ref_frac_re = 0.0, ref_frac_im = 0.0;
    C2 ref_z_f{0, 0};
    bool use_bigfixed = false;
    BF bz_re[2], bz_im[2], bc_re, bc_im, bt1, bt2, bab, bre, bim;
    std::vector<uint64_t> bftmp;
    int bfL = 0;

    int idx(const Pix& p) const { // mp.cpp:4334-4340
        return (p.a[0] * SUB + SUB / 2 + p.a[2]) * W * SUB + (p.a[1] * SUB + SUB / 2 + p.a[3]);
    }
    void setPixel(const Pix& p, float v, int n) {
        iter_[idx(p)] = v;
        if (escn_) escn_[idx(p)] = n;
    }
    static bool deriv_of(int cm) { return (cm & (CM_EDE | CM_NORMAL | CM_DEOVL)) != 0; }

    double floatPoint(double c_re, double c_im, int mxit, int cm, double* nrm, int* nout = nullptr) const;
    float shallowSimd(double cr, double ci, int mxit, int cm, int* nout = nullptr) const;
    float accuratePoint(mpf_srcptr c_re, mpf_srcptr c_im, int mxit, int cm, int* nout = nullptr) const;
    float accuratePixel(const Pix& p, int mxit, int cm, int* nout = nullptr) const;
    bool refTailEscapes(int last, int extra) const;
    int findNucleus(mpf_ptr nre, mpf_ptr nim, int maxp);
    int createPeriodicRef(int period, int cm);
    FE nucleusSize() const;
    int buildReferenceOrbit(std::set<std::array<int, 4>>& s, mpf_srcptr scale, int mxit, int cm);
    int createRef(std::set<std::array<int, 4>>& s, int pr_it, int mxit, bool random, int cm, bool view_center = false);
    bool calCoefficient(int i, int pr_it, int cm, bool past = false);
    int saCheck() const;
    void buildBLA(int reflen, bool ede);
    int tryBLA(int s, double& dzr, double& dzi, double& ddr, double& ddi, double dcr, double dci, bool ede, int mx_ref_it) const;
    int tryBLAfe(int s, FE& S, FE S2, double& wr, double& wi, double dr, double di, int mx_ref_it, double* ab) const;
    float pixelRescaled(FE dcr, FE dci, int mx_ref_it, int mxit, int cm, float* nrm, int* nout) const;
    float rescaledNoBla(FE dcr, FE dci, int mx_ref_it, int mxit, int* nout) const;
    void stepParallel(std::set<std::array<int, 4>>& s, int mx_ref_it, int mxit, int cm, const std::vector<std::array<int, 4>>* contiguous = nullptr);
};

static inline Pix P(const std::array<int, 4>& a) { return Pix{{a[0], a[1], a[2], a[3]}}; }

// mp.cpp:330-399 (smooth / EDE / DE-overlay branches).
double Engine::floatPoint(double c_re, double c_im, int mxit, int cm, double* nrm, int* nout) const {
    if (nout) *nout = -1;
    double z_re = c_re, z_im = c_im, d_re = 2, d_im = 0, dc_re = 1, dc_im = 0, tmp;
    const bool de_ovl = (cm & CM_DEOVL) != 0;
    const bool normal = (cm & CM_NORMAL) != 0;
    const bool deriv = (cm & CM_EDE) || normal || de_ovl;
    OrbitAcc oc; // mp.cpp:347-351
    oc.init(cm);
    const bool ocol = oc.sac || oc.trap;
    int i = 1;
    while (i < mxit) {
        tmp = 2.0 * (d_re * z_re - d_im * z_im);
        d_im = 2.0 * (d_re * z_im + d_im * z_re);
        d_re = tmp;
        if (deriv) {
            tmp = 2.0 * (dc_re * z_re - dc_im * z_im) + 1;
            dc_im = 2.0 * (dc_re * z_im + dc_im * z_re);
            dc_re = tmp;
        }
        tmp = z_re * z_re - z_im * z_im + c_re;
        z_im = 2.0 * z_re * z_im + c_im;
        z_re = tmp;
        if (ocol) oc.push((double)z_re, (double)z_im);
        tmp = z_re * z_re + z_im * z_im;
        if (tmp > ESC2) {
            if (nout) *nout = i + 1;
            if (cm & CM_EDE) return std::sqrt(tmp) * std::log(tmp) / std::sqrt(dc_re * dc_re + dc_im * dc_im);
            if (normal) { // mp.cpp:375-378
                if (nrm) *nrm = std::atan2((double)z_im, (double)z_re) - std::atan2((double)dc_im, (double)dc_re);
                return (i + 1 - std::log(std::log(tmp) / 2 / std::log(2)) / std::log(2));
            }
            if (de_ovl) {
                if (nrm) *nrm = std::sqrt(tmp) * std::log(tmp) / std::sqrt(dc_re * dc_re + dc_im * dc_im);
                return (i + 1 - std::log(std::log(tmp) / 2 / std::log(2)) / std::log(2));
            }
            if (ocol) return oc.escaped(i + 1 - std::log(std::log(tmp) / 2 / std::log(2)) / std::log(2), (double)tmp, (double)escf); // mp.cpp:383-389
            return (i + 1 - std::log(std::log(tmp) / 2 / std::log(2)) / std::log(2));
        }
        tmp = d_re * d_re + d_im * d_im;
        if (tmp < 0.000000001) return oc.interior();
        ++i;
    }
    return oc.interior();
}

// mp.cpp:416-532 for one pixel (lane refill does not change per-pixel values).
float Engine::shallowSimd(double cr, double ci, int mxit, int cm, int* nout) const {
    if (nout) *nout = -1;
    const bool ede = (cm & CM_EDE) != 0;
    const double LG2 = std::log(2.0);
    double zr = cr, zi = ci, dr = 2, di = 0, dcr = 1, dci = 0, jv = 1;
    for (;;) {
        double ndr = 2.0 * ((dr * zr) - (di * zi));
        double ndi = 2.0 * ((dr * zi) + (di * zr));
        double ndcr = (2.0 * ((dcr * zr) - (dci * zi))) + 1.0;
        double ndci = 2.0 * ((dcr * zi) + (dci * zr));
        double nzr = ((zr * zr) - (zi * zi)) + cr;
        double nzi = (2.0 * (zr * zi)) + ci;
        zr = nzr; zi = nzi; dr = ndr; di = ndi; dcr = ndcr; dci = ndci;
        double zrad = (zr * zr) + (zi * zi);
        double dmag = (dr * dr) + (di * di);
        double jnext = jv + 1.0;
        if (zrad > ESC2) {
            if (nout) *nout = (int)jv + 1;
            if (ede) return (float)(std::sqrt(zrad) * std::log(zrad) / std::sqrt(dcr * dcr + dci * dci));
            return (float)(jv + 1 - std::log(std::log(zrad) / 2 / LG2) / LG2);
        }
        if (dmag < 1e-9) return -2.0f;
        if (jnext >= (double)mxit) return -2.0f;
        jv = jnext;
    }
}

// Truth of the normal-map angle (private flag of Engine::truth only): the same
// GMP orbit and derivative dz/dc as the EDE branch, returning arg z_N - arg dz/dc
// at the escape. The reference's point routine has no normal-map branch; its
// render path (accuratePixel) never sets this flag.
constexpr int kTruthAngle = 1 << 20;

// mp.cpp:719-894 (smooth / EDE branches; derivative tracked, no env overrides).
float Engine::accuratePoint(mpf_srcptr c_re, mpf_srcptr c_im, int mxit, int cm, int* nout) const {
    if (nout) *nout = -1;
    const mp_bitcnt_t wp = mpf_get_prec(c_re);
    mpf_t tt1, tt2, z_re, z_im, d_re, d_im, dc_re, dc_im, e1, e2;
    mpf_init2(tt1, wp); mpf_init2(tt2, wp);
    mpf_init2(z_re, wp); mpf_set(z_re, c_re);
    mpf_init2(z_im, wp); mpf_set(z_im, c_im);
    mpf_init2(d_re, wp); mpf_init2(d_im, wp);
    mpf_set_str(d_re, "2", 10);
    const bool ede = (cm & CM_EDE) != 0;
    const bool angle = !ede && (cm & kTruthAngle) != 0;
    mpf_init2(dc_re, wp); mpf_set_ui(dc_re, 1);
    mpf_init2(dc_im, wp); mpf_init2(e1, wp); mpf_init2(e2, wp);
    OrbitAcc oc; // mp.cpp:763-770 (the stripe average takes precedence at escape here, :851-863)
    oc.init(cm);
    int i = 1;
    float res = -2;
    while (i < mxit) {
        mpf_mul(tt1, d_re, z_im);
        mpf_mul(d_re, d_re, z_re);
        mpf_mul(tt2, d_im, z_im);
        mpf_mul(d_im, d_im, z_re);
        mpf_sub(d_re, d_re, tt2);
        mpf_mul_ui(d_re, d_re, 2);
        mpf_add(d_im, d_im, tt1);
        mpf_mul_ui(d_im, d_im, 2);
        if (ede || angle) {
            mpf_mul(e1, dc_re, z_im);
            mpf_mul(e2, dc_im, z_re);
            mpf_add(e2, e1, e2);
            mpf_mul(e1, dc_re, z_re);
            mpf_mul(tt2, dc_im, z_im);
            mpf_sub(e1, e1, tt2);
            mpf_mul_ui(dc_re, e1, 2);
            mpf_add_ui(dc_re, dc_re, 1);
            mpf_mul_ui(dc_im, e2, 2);
        }
        mpf_mul(tt1, z_re, z_im);
        mpf_mul(z_re, z_re, z_re);
        mpf_mul(z_im, z_im, z_im);
        mpf_sub(z_re, z_re, z_im);
        mpf_add(z_re, z_re, c_re);
        mpf_mul_ui(z_im, tt1, 2);
        mpf_add(z_im, z_im, c_im);
        oc.push(mpf_get_d(z_re), mpf_get_d(z_im)); // mp.cpp:819-820
        mpf_mul(tt1, z_re, z_re);
        mpf_mul(tt2, z_im, z_im);
        mpf_add(tt1, tt1, tt2);
        double rad = mpf_get_d(tt1);
        if (rad > ESC2) {
            if (nout) *nout = i + 1;
            if (angle) {
                // arg z - arg J, J = dz/dc scaled by its larger component (mpf_get_d
                // of the ratios stays in range whatever the size of J)
                mpf_abs(e1, dc_re);
                mpf_abs(e2, dc_im);
                if (mpf_cmp(e1, e2) < 0) mpf_set(e1, e2);
                double jr = 0.0, ji = 0.0;
                if (mpf_sgn(e1) != 0) {
                    mpf_div(e2, dc_re, e1);
                    jr = mpf_get_d(e2);
                    mpf_div(e2, dc_im, e1);
                    ji = mpf_get_d(e2);
                }
                res = (float)(std::atan2(mpf_get_d(z_im), mpf_get_d(z_re)) - std::atan2(ji, jr));
                break;
            }
            if (ede) {
                mpf_mul(e1, dc_re, dc_re);
                mpf_mul(e2, dc_im, dc_im);
                mpf_add(e1, e1, e2);
                mpf_sqrt(e1, e1);
                mpf_abs(tt1, dx);
                mpf_mul(e1, e1, tt1);
                double num = std::isfinite(rad) && rad > 0.0 ? std::sqrt(rad) * std::log(rad) : 0.0;
                mpf_set_d(e2, num);
                if (mpf_sgn(e1) != 0) {
                    mpf_div(e1, e2, e1);
                    res = (float)mpf_get_d(e1);
                } else
                    res = 0.f;
            } else if (oc.sac) {
                res = oc.sacValue(rad, (double)escf);
            } else if (oc.trap) {
                res = oc.trapValue((double)i + 1 - std::log(std::log(rad) / 2 / std::log(2)) / std::log(2));
            } else {
                res = (i + 1 - std::log(std::log(rad) / 2 / std::log(2)) / std::log(2));
            }
            break;
        }
        mpf_mul(tt1, d_re, d_re);
        mpf_mul(tt2, d_im, d_im);
        mpf_add(tt1, tt1, tt2);
        rad = mpf_get_d(tt1);
        if (rad < 0.000000001) break;
        ++i;
    }
    if (oc.trap && res == -2.0f) res = oc.trapValue(0.0); // mp.cpp:882
    mpf_clears(tt1, tt2, z_re, z_im, d_re, d_im, dc_re, dc_im, e1, e2, (mpf_ptr)0);
    return res;
}

// mp.cpp:896-919.
float Engine::accuratePixel(const Pix& p, int mxit, int cm, int* nout) const {
    mpf_t cre, cim, off, soff;
    mpf_init(cre); mpf_set(cre, c0_re);
    mpf_init(cim); mpf_set(cim, c0_im);
    mpf_init(off); mpf_init(soff);
    mpf_mul_ui(off, dx, p.a[1]);
    mpf_add(cre, cre, off);
    mpf_mul_ui(off, dx, std::abs(p.a[3]));
    mpf_set(soff, off);
    if (p.a[3] < 0) mpf_neg(soff, soff);
    mpf_div_ui(soff, soff, SUB);
    mpf_add(cre, cre, soff);
    mpf_mul_ui(off, dy, p.a[0]);
    mpf_add(cim, cim, off);
    mpf_mul_ui(off, dy, std::abs(p.a[2]));
    mpf_set(soff, off);
    if (p.a[2] < 0) mpf_neg(soff, soff);
    mpf_div_ui(soff, soff, SUB);
    mpf_add(cim, cim, soff);
    float r = accuratePoint(cre, cim, mxit, cm, nout);
    mpf_clears(cre, cim, off, soff, (mpf_ptr)0);
    return r;
}

// mp.cpp:927-957.
bool Engine::refTailEscapes(int last, int extra) const {
    mpf_t zr, zi, a1, a2;
    mpf_init(zr); mpf_init(zi); mpf_init(a1); mpf_init(a2);
    if (use_bigfixed) {
        bf_to_mpf(zr, bz_re[last & 1]);
        bf_to_mpf(zi, bz_im[last & 1]);
    } else {
        mpf_set(zr, zre[last & 1]);
        mpf_set(zi, zim[last & 1]);
    }
    bool esc = false;
    for (int k = 0; k < extra && !esc; ++k) {
        mpf_mul(a1, zr, zi);
        mpf_mul(zr, zr, zr);
        mpf_mul(a2, zi, zi);
        mpf_sub(zr, zr, a2);
        mpf_add(zr, zr, ref_re);
        mpf_mul_ui(zi, a1, 2);
        mpf_add(zi, zi, ref_im);
        mpf_mul(a1, zr, zr);
        mpf_mul(a2, zi, zi);
        mpf_add(a1, a1, a2);
        if (mpf_get_d(a1) > ESC2) esc = true;
    }
    mpf_clears(zr, zi, a1, a2, (mpf_ptr)0);
    return esc;
}

// Ball period and Newton nucleus (mp.cpp:96-223).
static void g_sqadd(mpf_ptr zr, mpf_ptr zi, mpf_srcptr cr, mpf_srcptr ci, mpf_ptr s1, mpf_ptr s2, mpf_ptr s3) {
    mpf_add(s1, zr, zi);
    mpf_sub(s2, zr, zi);
    mpf_mul(s3, zr, zi);
    mpf_mul(zr, s1, s2);
    mpf_add(zr, zr, cr);
    mpf_mul_ui(zi, s3, 2);
    mpf_add(zi, zi, ci);
}
static int g_ballPeriod(mpf_srcptr cr, mpf_srcptr ci, mpf_srcptr r, int maxp, mp_bitcnt_t prec) {
    mpf_t s1, s2, s3, zr, zi, R, R2m, zabs2, nb, ru, t;
    mpf_init2(s1, prec); mpf_init2(s2, prec); mpf_init2(s3, prec);
    mpf_init2(zr, prec); mpf_init2(zi, prec); mpf_init2(R, prec); mpf_init2(R2m, prec);
    mpf_init2(zabs2, prec); mpf_init2(nb, prec); mpf_init2(ru, prec); mpf_init2(t, prec);
    mpf_set_ui(zr, 0); mpf_set_ui(zi, 0); mpf_set_ui(R, 0);
    const double cab = std::hypot(mpf_get_d(cr), mpf_get_d(ci));
    mpf_set_ui(ru, 1);
    mpf_div_2exp(ru, ru, prec > 64 ? prec - 32 : prec / 2);
    int period = 0;
    for (int p = 1; p <= maxp; ++p) {
        double za = std::hypot(mpf_get_d(zr), mpf_get_d(zi));
        mpf_set_d(t, 2.0 * za);
        mpf_add(nb, t, R);
        mpf_mul(nb, nb, R);
        mpf_add(nb, nb, r);
        mpf_set_d(t, za * za + cab + 1.0);
        mpf_mul(t, t, ru);
        mpf_add(nb, nb, t);
        mpf_set(R, nb);
        g_sqadd(zr, zi, cr, ci, s1, s2, s3);
        mpf_mul(s1, zr, zr);
        mpf_mul(s2, zi, zi);
        mpf_add(zabs2, s1, s2);
        mpf_mul(R2m, R, R);
        if (mpf_cmp(zabs2, R2m) <= 0) {
            period = p;
            break;
        }
        double zb = std::hypot(mpf_get_d(zr), mpf_get_d(zi));
        if (zb > cab + 2.0 + mpf_get_d(R)) break;
    }
    mpf_clears(s1, s2, s3, zr, zi, R, R2m, zabs2, nb, ru, t, (mpf_ptr)0);
    return period;
}
static bool g_newton(mpf_ptr cr, mpf_ptr ci, int period, mp_bitcnt_t prec, int maxit) {
    mpf_t s1, s2, s3, zr, zi, dr, di, den, nr, ni, tol, step2;
    mpf_init2(s1, prec); mpf_init2(s2, prec); mpf_init2(s3, prec);
    mpf_init2(zr, prec); mpf_init2(zi, prec); mpf_init2(dr, prec); mpf_init2(di, prec);
    mpf_init2(den, prec); mpf_init2(nr, prec); mpf_init2(ni, prec); mpf_init2(tol, prec); mpf_init2(step2, prec);
    mpf_set_ui(tol, 1);
    mpf_div_2exp(tol, tol, prec > 96 ? prec - 48 : prec / 2);
    mpf_mul(tol, tol, tol);
    bool conv = false;
    for (int it = 0; it < maxit; ++it) {
        mpf_set_ui(zr, 0); mpf_set_ui(zi, 0); mpf_set_ui(dr, 0); mpf_set_ui(di, 0);
        for (int i = 0; i < period; ++i) {
            mpf_mul(s1, zr, dr);
            mpf_mul(s2, zi, di);
            mpf_sub(s3, s1, s2);
            mpf_mul_ui(s3, s3, 2);
            mpf_add_ui(s3, s3, 1);
            mpf_mul(s1, zr, di);
            mpf_mul(s2, zi, dr);
            mpf_add(di, s1, s2);
            mpf_mul_ui(di, di, 2);
            mpf_set(dr, s3);
            g_sqadd(zr, zi, cr, ci, s1, s2, s3);
        }
        mpf_mul(s1, dr, dr);
        mpf_mul(s2, di, di);
        mpf_add(den, s1, s2);
        if (mpf_sgn(den) == 0) break;
        mpf_mul(s1, zr, dr);
        mpf_mul(s2, zi, di);
        mpf_add(s3, s1, s2);
        mpf_div(nr, s3, den);
        mpf_mul(s1, zi, dr);
        mpf_mul(s2, zr, di);
        mpf_sub(s3, s1, s2);
        mpf_div(ni, s3, den);
        mpf_sub(cr, cr, nr);
        mpf_sub(ci, ci, ni);
        mpf_mul(s1, nr, nr);
        mpf_mul(s2, ni, ni);
        mpf_add(step2, s1, s2);
        if (mpf_cmp(step2, tol) <= 0) {
            conv = true;
            break;
        }
    }
    mpf_clears(s1, s2, s3, zr, zi, dr, di, den, nr, ni, tol, step2, (mpf_ptr)0);
    return conv;
}

// mp.cpp:1072-1107.
int Engine::findNucleus(mpf_ptr nre, mpf_ptr nim, int maxp) {
    const mp_bitcnt_t prec = mpf_get_prec(c0_re);
    mpf_t cre, cim, r, dh, dist, dr, di;
    mpf_init2(cre, prec); mpf_init2(cim, prec); mpf_init2(r, prec); mpf_init2(dh, prec);
    mpf_init2(dist, prec); mpf_init2(dr, prec); mpf_init2(di, prec);
    mpf_set_ui(r, 2);
    mpf_div(r, r, scale_);
    mpf_add(cre, c0_re, r);
    mpf_mul_ui(dh, r, H);
    mpf_div_ui(dh, dh, W);
    mpf_add(cim, c0_im, dh);
    int period = g_ballPeriod(cre, cim, r, maxp, prec);
    int result = 0;
    if (period > 0) {
        mpf_set(nre, cre);
        mpf_set(nim, cim);
        if (g_newton(nre, nim, period, prec, 200)) {
            mpf_sub(dr, nre, cre);
            mpf_sub(di, nim, cim);
            mpf_mul(dr, dr, dr);
            mpf_mul(di, di, di);
            mpf_add(dist, dr, di);
            mpf_sqrt(dist, dist);
            if (mpf_cmp(dist, r) <= 0) result = period;
        }
    }
    mpf_clears(cre, cim, r, dh, dist, dr, di, (mpf_ptr)0);
    return result;
}

// mp.cpp:1109-1172.
int Engine::createPeriodicRef(int period, int cm) {
    ref_escaped = false;
    ref_escape_iteration = 0;
    ref_z_f = C2{mpf_ld(ref_re), mpf_ld(ref_im)};
    ref_virtual = true;
    mpf_sub(t1, ref_re, c0_re);
    mpf_div(t1, t1, dx);
    ref_x = mpf_get_d(t1);
    mpf_sub(t1, ref_im, c0_im);
    mpf_div(t1, t1, dy);
    ref_y = mpf_get_d(t1);
    int px = (int)std::lround(ref_x), py = (int)std::lround(ref_y);
    ref_ = Pix{{py, px, 0, 0}};
    ref_frac_re = (ref_x - px) * mpf_ld(dx);
    ref_frac_im = (ref_y - py) * mpf_ld(dy);
    mpf_set(zre[0], ref_re);
    mpf_set(zim[0], ref_im);
    use_bigfixed = false;
    zfr[0] = ref_z_f.re;
    zfi[0] = ref_z_f.im;
    zfr_fe[0] = mpf_fe(ref_re);
    zfi_fe[0] = mpf_fe(ref_im);
    z_m3[0] = (zfr[0] * zfr[0] + zfi[0] * zfi[0]) / 1000000;
    dfr[0] = 1.0;
    dfi[0] = 0.0;
    dfe_r = FE{1.0, 0};
    dfe_i = FE{0.0, 0};
    mpf_mul_ui(t1, dx, W);
    mpf_div_ui(t1, t1, 2);
    mpf_mul_ui(t2, dy, H);
    mpf_div_ui(t2, t2, 2);
    SA_delta = C2{mpf_ld(t1), mpf_ld(t2)};
    SA_flag = false;
    SA_it = 0;
    SA_order = 0;
    for (int i = 0; i < SA_N; ++i) Adf_old[i] = Bdf_old[i] = C2{0, 0};
    Adf_old[0] = SA_delta;
    bool save_fe = use_floatexp;
    use_floatexp = true;
    for (int i = 1; i < period; ++i) calCoefficient(i, 0, cm);
    use_floatexp = save_fe;
    ref_period = period;
    return period;
}

// mp.cpp:1195-1219.
FE Engine::nucleusSize() const {
    const int p = ref_period;
    if (p < 2) return FE{1.0, 1000000};
    FE lr{1.0, 0}, li{0.0, 0}, br{1.0, 0}, bi{0.0, 0};
    for (int k = 1; k < p; ++k) {
        FE zr = zfr_fe[k - 1], zi = zfi_fe[k - 1];
        FE nr = fe_scale2(fe_sub(fe_mul(zr, lr), fe_mul(zi, li)), 1);
        FE ni = fe_scale2(fe_add(fe_mul(zr, li), fe_mul(zi, lr)), 1);
        lr = nr;
        li = ni;
        FE l2 = fe_add(fe_mul(lr, lr), fe_mul(li, li));
        if (l2.m == 0.0) continue;
        br = fe_add(br, fe_div(lr, l2));
        bi = fe_sub(bi, fe_div(li, l2));
    }
    FE lmag = fe_sqrt(fe_add(fe_mul(lr, lr), fe_mul(li, li)));
    FE bmag = fe_sqrt(fe_add(fe_mul(br, br), fe_mul(bi, bi)));
    FE denom = fe_mul(bmag, fe_mul(lmag, lmag));
    if (denom.m == 0.0) return FE{1.0, 1000000};
    return fe_div(FE{1.0, 0}, denom);
}

// mp.cpp:1227-1386.
int Engine::buildReferenceOrbit(std::set<std::array<int, 4>>& s, mpf_srcptr scale, int mxit, int cm) {
    int ref_it = 0;
    ref_period = 0;
    ref_subpixel = false;
    ref_deep_zero = false;
    bool periodic_done = false;
    bool periodic_want = (opt.periodic == 1) || (opt.periodic != 0 && mpf_cmp_d(scale, 1e280) > 0);
    if (periodic_want && use_bla) {
        mpf_t save_re, save_im;
        mpf_init2(save_re, mpf_get_prec(ref_re));
        mpf_set(save_re, ref_re);
        mpf_init2(save_im, mpf_get_prec(ref_im));
        mpf_set(save_im, ref_im);
        int p = findNucleus(ref_re, ref_im, mxit);
        if (p > 2 && p <= mxit) {
            ref_it = createPeriodicRef(p, cm);
            FE sizeMag = nucleusSize();
            ref_subpixel = fe_abs_less(sizeMag, fe_mul_d(dxfe, 4.0));
            if (!ref_subpixel) {
                ref_bounded = true;
                periodic_done = true;
                if (!use_floatexp) {
                    double refmin2 = 1e300;
                    bool uf = false;
                    for (int q = 1; q < p; ++q) {
                        double m2 = z_m3[q] * 1e6;
                        if (m2 <= 0.0) {
                            uf = true;
                            break;
                        }
                        if (m2 < refmin2) refmin2 = m2;
                    }
                    double dcmax = 2.0 / mpf_get_d(scale);
                    if (uf || std::sqrt(refmin2) * dcmax < 1e-300) use_floatexp = true;
                }
            } else {
                mpf_set(ref_re, save_re);
                mpf_set(ref_im, save_im);
                ref_period = 0;
                ref_virtual = false;
                ref_bounded = false;
            }
        }
        mpf_clear(save_re);
        mpf_clear(save_im);
    }
    if (!periodic_done) {
        s.insert({H / 2, W / 2, 0, 0});
        ref_it = createRef(s, mxit, mxit, true, cm);
        if (!use_floatexp && mpf_cmp_d(scale, 1e150) > 0) {
            double refmin2 = 1e300;
            bool underflowed = false;
            for (int q = 1; q <= ref_it; ++q) {
                double m2 = z_m3[q] * 1e6;
                if (m2 <= 0.0) {
                    underflowed = true;
                    break;
                }
                if (m2 < refmin2) refmin2 = m2;
            }
            double dcmax = 2.0 / mpf_get_d(scale);
            if (underflowed || std::sqrt(refmin2) * dcmax < 1e-300) {
                use_floatexp = true;
                s.insert({H / 2, W / 2, 0, 0});
                ref_it = createRef(s, mxit, mxit, true, cm, true);
            }
        }
        if (use_floatexp && (!ref_escaped || ref_escape_iteration >= mxit - 16)) {
            bool sensitive = ref_escaped || refTailEscapes(ref_it, 80);
            if (sensitive) {
                s.insert({H / 2, W / 2, 0, 0});
                ref_it = createRef(s, mxit, mxit, true, cm, true);
            }
        }
        ref_bounded = !ref_escaped;
        if (use_floatexp && !ref_bounded) {
            for (int q = 0; q <= ref_it; ++q) {
                if (zfr[q] == 0.0 && zfi[q] == 0.0 && (zfr_fe[q].m != 0.0 || zfi_fe[q].m != 0.0)) {
                    ref_deep_zero = true;
                    break;
                }
            }
        }
    }
    return ref_it;
}

// mp.cpp:4014-4187. `random` picks with libc rand() exactly like the reference.
int Engine::createRef(std::set<std::array<int, 4>>& s, int pr_it, int mxit, bool random, int cm, bool view_center) {
    if (s.empty()) return 0;
    ref_period = 0;
    ref_escaped = false;
    ref_escape_iteration = 0;
    ++stat_refs;
    std::array<int, 4> p{H / 2, W / 2, 0, 0};
    if (view_center) {
        ref_virtual = true;
        fe_cutoff_sensitive = false;
        ref_x = (W - 1) * 0.5;
        ref_y = (H - 1) * 0.5;
        mpf_set(ref_re, c0_re);
        mpf_mul_ui(t1, dx, W - 1);
        mpf_div_ui(t1, t1, 2);
        mpf_add(ref_re, ref_re, t1);
        mpf_set(ref_im, c0_im);
        mpf_mul_ui(t1, dy, H - 1);
        mpf_div_ui(t1, t1, 2);
        mpf_add(ref_im, ref_im, t1);
    } else {
        ref_virtual = false;
        if (random) {
            auto r = rand() % s.size();
            auto it = s.begin();
            std::advance(it, r);
            p = *it;
            s.erase(it);
        } else {
            std::array<int, 4> nr{new_ref.a[0], new_ref.a[1], new_ref.a[2], new_ref.a[3]};
            auto it = s.find(nr);
            if (it == s.end()) {
                auto r = rand() % s.size();
                it = s.begin();
                std::advance(it, r);
            }
            p = *it;
            s.erase(it);
        }
        ref_x = p[1] + (double)p[3] / SUB;
        ref_y = p[0] + (double)p[2] / SUB;
        mpf_set(ref_re, c0_re);
        mpf_set(ref_im, c0_im);
        mpf_mul_ui(t1, dx, p[1]);
        mpf_add(ref_re, ref_re, t1);
        mpf_mul_ui(t1, dx, std::abs(p[3]));
        if (p[3] < 0) mpf_neg(t1, t1);
        mpf_div_ui(t1, t1, SUB);
        mpf_add(ref_re, ref_re, t1);
        mpf_mul_ui(t1, dy, p[0]);
        mpf_add(ref_im, ref_im, t1);
        mpf_mul_ui(t1, dy, std::abs(p[2]));
        if (p[2] < 0) mpf_neg(t1, t1);
        mpf_div_ui(t1, t1, SUB);
        mpf_add(ref_im, ref_im, t1);
    }
    ref_z_f = C2{mpf_ld(ref_re), mpf_ld(ref_im)};
    ref_ = P(p);
    mpf_set(zre[0], ref_re);
    mpf_set(zim[0], ref_im);
    const bool bfReq = (opt.bigfixed == -1) ? use_floatexp : (opt.bigfixed > 0);
    use_bigfixed = bfReq;
    if (use_bigfixed) {
        int prec = (int)mpf_get_prec(ref_re);
        bfL = (prec + 63) / 64 + 2;
        bftmp.assign((size_t)2 * bfL + 8, 0ull);
        bf_from_mpf(bc_re, ref_re, bfL);
        bf_from_mpf(bc_im, ref_im, bfL);
        bz_re[0] = bc_re;
        bz_im[0] = bc_im;
        bt1.setL(bfL); bt2.setL(bfL); bab.setL(bfL); bre.setL(bfL); bim.setL(bfL);
        bz_re[1].setL(bfL); bz_im[1].setL(bfL);
    }
    zfr[0] = ref_z_f.re;
    zfi[0] = ref_z_f.im;
    if (use_floatexp) {
        zfr_fe[0] = mpf_fe(ref_re);
        zfi_fe[0] = mpf_fe(ref_im);
    }
    dfr[0] = 1.0;
    dfi[0] = 0.0;
    dfe_r = FE{1.0, 0};
    dfe_i = FE{0.0, 0};
    mpf_mul_ui(t1, dx, W);
    mpf_div_ui(t1, t1, 2);
    mpf_mul_ui(t2, dy, H);
    mpf_div_ui(t2, t2, 2);
    SA_delta = C2{mpf_ld(t1), mpf_ld(t2)};
    for (int i = 0; i < SA_N; ++i) Adf_old[i] = Bdf_old[i] = C2{0, 0};
    Adf_old[0] = SA_delta;
    SA_flag = true;
    SA_it = 0;
    for (int i = 1; i <= mxit; ++i) {
        if (!calCoefficient(i, pr_it, cm)) {
            ref_escaped = true;
            ref_escape_iteration = i;
            if (ref_virtual && use_floatexp && i >= mxit - 16) fe_cutoff_sensitive = true;
            if (!ref_virtual) {
                if (cm) {
                    int nn;
                    float rv = accuratePoint(ref_re, ref_im, mxit, cm, &nn);
                    setPixel(ref_, rv, nn);
                } else {
                    if (use_bigfixed) {
                        bf_to_mpf(zre[i & 1], bz_re[i & 1]);
                        bf_to_mpf(zim[i & 1], bz_im[i & 1]);
                    }
                    mpf_mul(t1, zre[i & 1], zre[i & 1]);
                    mpf_mul(t2, zim[i & 1], zim[i & 1]);
                    mpf_add(t1, t1, t2);
                    double rad = mpf_get_d(t1);
                    setPixel(ref_, (float)(i + 1 - std::log(std::log(rad) / 2 / std::log(2)) / std::log(2)), i + 1);
                }
            }
            return i;
        }
    }
    if (ref_virtual && use_floatexp) fe_cutoff_sensitive = accuratePoint(ref_re, ref_im, mxit + 64, cm) >= 0;
    if (!ref_virtual) setPixel(ref_, (cm & CM_TRAP) ? accuratePoint(ref_re, ref_im, mxit, cm) : -2.f, -1); // mp.cpp:4179-4184
    return mxit;
}

// mp.cpp:4189-4305.
bool Engine::calCoefficient(int i, int pr_it, int cm, bool past) {
    const bool deriv = deriv_of(cm);
    const int c = i & 1, p = (i - 1) & 1;
    if (use_bigfixed) {
        const BF& a = bz_re[p];
        const BF& b = bz_im[p];
        bf_addsub(bt1, a, a.sign, b, b.sign);
        bf_addsub(bt2, a, a.sign, b, -b.sign);
        bf_mul(bab, a, b, bftmp.data());
        bf_mul(bre, bt1, bt2, bftmp.data());
        bf_addsub(bim, bab, bab.sign, bab, bab.sign);
        bf_addsub(bz_re[c], bre, bre.sign, bc_re, bc_re.sign);
        bf_addsub(bz_im[c], bim, bim.sign, bc_im, bc_im.sign);
        if (use_floatexp) {
            FE fr = bf_to_fe(bz_re[c]), fi = bf_to_fe(bz_im[c]);
            zfr_fe[i] = fr;
            zfi_fe[i] = fi;
            zfr[i] = fe_to_double(fr);
            zfi[i] = fe_to_double(fi);
        } else {
            // bigfixed.h:179-189 toDouble.
            auto todbl = [](const BF& v) -> double {
                if (v.sign == 0) return 0.0;
                int top = v.L - 1;
                while (top >= 0 && v.m[top] == 0) --top;
                if (top < 0) return 0.0;
                double hi = (double)v.m[top];
                double lo = (top >= 1) ? (double)v.m[top - 1] : 0.0;
                double val = hi * 18446744073709551616.0 + lo;
                val = std::ldexp(val, 64 * (top - (v.L - 1) - 1));
                return v.sign < 0 ? -val : val;
            };
            zfr[i] = todbl(bz_re[c]);
            zfi[i] = todbl(bz_im[c]);
        }
    } else {
        mpf_add(t1, zre[p], zim[p]);
        mpf_sub(t2, zre[p], zim[p]);
        mpf_mul(zim[c], zre[p], zim[p]);
        mpf_mul(zre[c], t1, t2);
        mpf_mul_ui(zim[c], zim[c], 2);
        mpf_add(zre[c], zre[c], ref_re);
        mpf_add(zim[c], zim[c], ref_im);
        zfr[i] = mpf_ld(zre[c]);
        zfi[i] = mpf_ld(zim[c]);
        if (use_floatexp) {
            zfr_fe[i] = mpf_fe(zre[c]);
            zfi_fe[i] = mpf_fe(zim[c]);
        }
    }
    z_m3[i] = (zfr[i] * zfr[i] + zfi[i] * zfi[i]) / 1000000;
    if (deriv) {
        if (use_floatexp) {
            FE a = dfe_r, b = dfe_i, zr = zfr_fe[i - 1], zi = zfi_fe[i - 1];
            FE re = fe_add(fe_scale2(fe_sub(fe_mul(a, zr), fe_mul(b, zi)), 1), FE{1.0, 0});
            FE im = fe_scale2(fe_add(fe_mul(a, zi), fe_mul(b, zr)), 1);
            dfe_r = re;
            dfe_i = im;
            dfr[i] = fe_to_double(re);
            dfi[i] = fe_to_double(im);
        } else {
            double a = dfr[i - 1], b = dfi[i - 1], zr = zfr[i - 1], zi = zfi[i - 1];
            dfr[i] = 2.0 * (a * zr - b * zi) + 1.0;
            dfi[i] = 2.0 * (a * zi + b * zr);
        }
    }
    // escape(_zf[i]): std::abs(complex) > escapeRadius() (mp.cpp:2047-2049).
    if (std::hypot(zfr[i], zfi[i]) > (double)escf && !past) return false;
    if (i <= pr_it) {
        if (SA_flag) {
            C2 zprev{zfr[i - 1], zfi[i - 1]};
            C2 dprev{dfr[i - 1], dfi[i - 1]};
            for (int j = 0; j < SA_N; ++j) {
                Adf_new[j] = c_mul(c_mul(C2{2, 0}, zprev), Adf_old[j]);
                for (int k = 0; k < j / 2; ++k) Adf_new[j] = c_add(Adf_new[j], c_mul(c_mul(C2{2, 0}, Adf_old[k]), Adf_old[j - k - 1]));
                if (j % 2) Adf_new[j] = c_add(Adf_new[j], c_mul(Adf_old[j / 2], Adf_old[j / 2]));
            }
            if (deriv) {
                for (int j = 0; j < SA_N; ++j) {
                    Bdf_new[j] = c_add(c_mul(Bdf_old[j], zprev), c_mul(Adf_old[j], dprev));
                    for (int k = 0; k < j; ++k) Bdf_new[j] = c_add(Bdf_new[j], c_mul(Adf_old[k], Bdf_old[j - k - 1]));
                    Bdf_new[j] = c_mul(Bdf_new[j], C2{2, 0});
                }
            }
            Adf_new[0] = c_add(Adf_new[0], SA_delta);
            int order = saCheck();
            if (order < 0) {
                SA_flag = false;
            } else {
                SA_it = i;
                SA_order = order;
                for (int j = 0; j < SA_N; ++j) Adf_old[j] = Adf_new[j];
                if (cm & CM_EDE)
                    for (int j = 0; j < SA_N; ++j) Bdf_old[j] = Bdf_new[j];
            }
        }
    }
    return true;
}

// mp.cpp:4307-4332.
int Engine::saCheck() const {
    int pre_mn[SA_N], suf_mx[SA_N];
    pre_mn[0] = std::min(exp_of(Adf_new[0].re), exp_of(Adf_new[0].im));
    suf_mx[SA_N - 1] = std::max(exp_of(Adf_new[SA_N - 1].re), exp_of(Adf_new[SA_N - 1].im));
    for (int i = 1; i < SA_N; ++i) pre_mn[i] = std::max(pre_mn[i - 1], std::min(exp_of(Adf_new[i].re), exp_of(Adf_new[i].im)));
    for (int i = SA_N - 2; i >= 0; --i) suf_mx[i] = std::max(suf_mx[i + 1], std::max(exp_of(Adf_new[i].re), exp_of(Adf_new[i].im)));
    for (int i = 0; i < SA_N - 10; ++i)
        if (pre_mn[i] - suf_mx[i + 1] >= 80) return std::max(i, 5);
    return -1;
}

// mp.cpp:2613-2709.
void Engine::buildBLA(int reflen, bool ede) {
    bla_r2.clear();
    bla_ab.clear();
    bla_ce.clear();
    bla_rmax2 = 0.0;
    if (reflen < 3) return;
    double eps = bla_eps > 0 ? bla_eps : std::ldexp(1.0, -53);
    double dxf = std::fabs(mpf_ld(dx)), dyf = std::fabs(mpf_ld(dy));
    double mxx = std::max(ref_x, (double)(W - 1) - ref_x) + 0.5;
    double mxy = std::max(ref_y, (double)(H - 1) - ref_y) + 0.5;
    double dcmax = std::sqrt(dxf * dxf * mxx * mxx + dyf * dyf * mxy * mxy);
    bla_dcmax2 = dcmax * dcmax;
    std::vector<double> r0;
    std::vector<std::array<double, 4>> ab0, ce0;
    for (int s = 1; s < reflen; ++s) {
        double zr = zfr[s], zi = zfi[s];
        double Zmag = std::sqrt(zr * zr + zi * zi);
        double ar = 2.0 * zr, ai = 2.0 * zi;
        double Amag = 2.0 * Zmag;
        double R = eps * (Zmag - dcmax) / (Amag + 1.0);
        double r2 = R > 0 ? R * R : 0.0;
        if (r2 > bla_rmax2) bla_rmax2 = r2;
        r0.push_back(r2);
        ab0.push_back({ar, ai, 1.0, 0.0});
        if (ede) ce0.push_back({2.0 * dfr[s], 2.0 * dfi[s], 0.0, 0.0});
    }
    bla_r2.push_back(std::move(r0));
    bla_ab.push_back(std::move(ab0));
    if (ede) bla_ce.push_back(std::move(ce0));
    while (bla_r2.back().size() > 1) {
        const std::vector<double>& pr = bla_r2.back();
        const std::vector<std::array<double, 4>>& pc = bla_ab.back();
        const std::vector<std::array<double, 4>>* pd = ede ? &bla_ce.back() : nullptr;
        std::vector<double> nr;
        std::vector<std::array<double, 4>> nc, nd;
        for (size_t i = 0; i + 1 < pr.size(); i += 2) {
            const auto& xc = pc[i];
            const auto& yc = pc[i + 1];
            std::array<double, 4> zc;
            zc[0] = yc[0] * xc[0] - yc[1] * xc[1];
            zc[1] = yc[0] * xc[1] + yc[1] * xc[0];
            zc[2] = yc[0] * xc[2] - yc[1] * xc[3] + yc[2];
            zc[3] = yc[0] * xc[3] + yc[1] * xc[2] + yc[3];
            if (ede) {
                const auto& xd = (*pd)[i];
                const auto& yd = (*pd)[i + 1];
                std::array<double, 4> zd;
                zd[0] = (yd[0] * xc[0] - yd[1] * xc[1]) + (yc[0] * xd[0] - yc[1] * xd[1]);
                zd[1] = (yd[0] * xc[1] + yd[1] * xc[0]) + (yc[0] * xd[1] + yc[1] * xd[0]);
                zd[2] = (yd[0] * xc[2] - yd[1] * xc[3]) + (yc[0] * xd[2] - yc[1] * xd[3]) + yd[2];
                zd[3] = (yd[0] * xc[3] + yd[1] * xc[2]) + (yc[0] * xd[3] + yc[1] * xd[2]) + yd[3];
                nd.push_back(zd);
            }
            double Rx = std::sqrt(pr[i]), Ry = std::sqrt(pr[i + 1]);
            double Axmag = std::sqrt(xc[0] * xc[0] + xc[1] * xc[1]);
            double Bxmag = std::sqrt(xc[2] * xc[2] + xc[3] * xc[3]);
            double cand = Axmag > 0 ? (Ry - Bxmag * dcmax) / Axmag : 0.0;
            double R = std::min(Rx, cand);
            nr.push_back(R > 0 ? R * R : 0.0);
            nc.push_back(zc);
        }
        bla_r2.push_back(std::move(nr));
        bla_ab.push_back(std::move(nc));
        if (ede) bla_ce.push_back(std::move(nd));
    }
}

static inline int tz32(unsigned x) { return x ? __builtin_ctz(x) : 32; }

// mp.cpp:2714-2755.
int Engine::tryBLA(int s, double& dzr, double& dzi, double& ddr, double& ddi, double dcr, double dci, bool ede, int mx_ref_it) const {
    if (s < 1 || bla_r2.empty()) return 0;
    double zmag2 = dzr * dzr + dzi * dzi;
    int maxp = (int)bla_r2.size() - 1;
    int startp = (s == 1) ? maxp : tz32((unsigned)(s - 1));
    if (startp > maxp) startp = maxp;
    if (startp < bla_minlevel) return 0;
    for (int p = startp; p >= bla_minlevel; --p) {
        int i = (s - 1) >> p;
        if (i >= (int)bla_r2[p].size()) continue;
        double r2 = bla_r2[p][i];
        if (r2 <= 0 || zmag2 >= r2) continue;
        int l = 1 << p;
        int land = s + l;
        if (land >= mx_ref_it - 1) continue;
        const auto& bc = bla_ab[p][i];
        double nzr = bc[0] * dzr - bc[1] * dzi + bc[2] * dcr - bc[3] * dci;
        double nzi = bc[0] * dzi + bc[1] * dzr + bc[2] * dci + bc[3] * dcr;
        double fr = zfr[land] + nzr, fi = zfi[land] + nzi;
        if (fr * fr + fi * fi > ESC2) return 0;
        if (ede) {
            const auto& bd = bla_ce[p][i];
            double nddr = (bd[0] * dzr - bd[1] * dzi) + (bc[0] * ddr - bc[1] * ddi) + (bd[2] * dcr - bd[3] * dci);
            double nddi = (bd[0] * dzi + bd[1] * dzr) + (bc[0] * ddi + bc[1] * ddr) + (bd[2] * dci + bd[3] * dcr);
            ddr = nddr;
            ddi = nddi;
        }
        dzr = nzr;
        dzi = nzi;
        return l;
    }
    return 0;
}

// mp.cpp:2770-2781.
static void blaReRescaleUnderflow(FE& S, double& wr, double& wi, double nwr, double nwi) {
    if (nwr == 0.0 && nwi == 0.0) {
        S = FE{1.0, 0};
        wr = wi = 0.0;
        return;
    }
    FE wmag = fe_sqrt(fe_add(fe_mul(fe_from(nwr), fe_from(nwr)), fe_mul(fe_from(nwi), fe_from(nwi))));
    S = fe_mul(S, wmag);
    double inv = 1.0 / fe_to_double(wmag);
    wr = nwr * inv;
    wi = nwi * inv;
}
static inline double pow2d(int64_t d) { // exact normalized 2^d for -1022 <= d <= 1023
    uint64_t bits = (uint64_t)(d + 1023) << 52;
    double r;
    std::memcpy(&r, &bits, 8);
    return r;
}
// mp.cpp:2794-2835.
static void feStepUnderflow(FE Xr, FE Xi, FE dcr, FE dci, FE& S, double& wr, double& wi) {
    const double sm = S.m, sm2 = sm * sm;
    const int64_t se = S.e;
    int64_t e = INT64_MIN;
    const bool has_w = wr != 0.0 || wi != 0.0;
    if (has_w && Xr.m != 0.0) e = std::max(e, Xr.e + se);
    if (has_w && Xi.m != 0.0) e = std::max(e, Xi.e + se);
    if (has_w) e = std::max(e, se + se);
    if (dcr.m != 0.0) e = std::max(e, dcr.e);
    if (dci.m != 0.0) e = std::max(e, dci.e);
    if (e == INT64_MIN) {
        S = FE{1.0, 0};
        wr = wi = 0.0;
        return;
    }
    auto align = [e](double m, int64_t te) {
        int64_t d = te - e;
        if (m == 0.0 || d < -54) return 0.0;
        return m * pow2d(d);
    };
    const double xs_r = align(Xr.m * sm, Xr.e + se);
    const double xs_i = align(Xi.m * sm, Xi.e + se);
    const double s2 = align(sm2, se + se);
    const double cr = align(dcr.m, dcr.e);
    const double ci = align(dci.m, dci.e);
    const double nr = 2.0 * (xs_r * wr - xs_i * wi) + s2 * (wr * wr - wi * wi) + cr;
    const double ni = 2.0 * (xs_r * wi + xs_i * wr) + 2.0 * s2 * wr * wi + ci;
    const double mag2 = nr * nr + ni * ni;
    const double mag = mag2 > 0.0 ? std::sqrt(mag2) : std::hypot(nr, ni);
    if (mag == 0.0) {
        S = FE{1.0, 0};
        wr = wi = 0.0;
        return;
    }
    S = fe_renorm(mag, e);
    wr = nr / mag;
    wi = ni / mag;
}
// mp.cpp:2842-2876.
static void feDerivUnderflow(FE zr, FE zi, FE& SJ, double& jr, double& ji, double& invSJd) {
    double im = 0.5 / SJ.m;
    int64_t ie = 1 - SJ.e;
    if (im >= 1.0) {
        im *= 0.5;
        ++ie;
    }
    FE invSJ{im, ie};
    int64_t e = invSJ.e;
    if (zr.m != 0.0) e = std::max(e, zr.e);
    if (zi.m != 0.0) e = std::max(e, zi.e);
    auto align = [e](FE x) {
        if (x.m == 0.0) return 0.0;
        int64_t d = x.e - e;
        if (d < -54) return 0.0;
        return x.m * pow2d(d);
    };
    double azr = align(zr), azi = align(zi);
    double ar = 2.0 * (azr * jr - azi * ji) + align(invSJ);
    double ai = 2.0 * (azr * ji + azi * jr);
    double mag = std::sqrt(ar * ar + ai * ai);
    if (mag == 0.0) {
        SJ = FE{1.0, 0};
        jr = ji = 0.0;
        invSJd = 1.0;
        return;
    }
    SJ = fe_mul(SJ, fe_renorm(mag, e));
    jr = ar / mag;
    ji = ai / mag;
    invSJd = 1.0 / fe_to_double(SJ);
}

// mp.cpp:2883-2970.
int Engine::tryBLAfe(int s, FE& S, FE S2, double& wr, double& wi, double dr, double di, int mx_ref_it, double* ab) const {
    if (s < 1 || bla_r2.empty()) return 0;
    int maxp = (int)bla_r2.size() - 1;
    int startp = (s == 1) ? maxp : tz32((unsigned)(s - 1));
    if (startp > maxp) startp = maxp;
    if (startp < bla_minlevel) return 0;
    FE dz2 = fe_mul(S2, fe_from(wr * wr + wi * wi));
    if (bla_rmax2 <= 0.0 || !fe_abs_less(dz2, fe_from(bla_rmax2))) return 0;
    for (int p = startp; p >= bla_minlevel; --p) {
        int i = (s - 1) >> p;
        if (i >= (int)bla_r2[p].size()) continue;
        double r2 = bla_r2[p][i];
        if (r2 <= 0 || !fe_abs_less(dz2, fe_from(r2))) continue;
        int l = 1 << p;
        int land = s + l;
        if (land >= mx_ref_it - 1) continue;
        const auto& bc = bla_ab[p][i];
        double nwr = (bc[0] * wr - bc[1] * wi) + (bc[2] * dr - bc[3] * di);
        double nwi = (bc[0] * wi + bc[1] * wr) + (bc[2] * di + bc[3] * dr);
        const double BIG = 1e150;
        if (std::isfinite(nwr) && std::isfinite(nwi) && std::fabs(nwr) < BIG && std::fabs(nwi) < BIG) {
            double fr = zfr[land] + fe_to_double(fe_mul_d(S, nwr));
            double fi = zfi[land] + fe_to_double(fe_mul_d(S, nwi));
            if (fr * fr + fi * fi > ESC2) return 0;
            double wm2 = nwr * nwr + nwi * nwi;
            if (wm2 == 0.0) {
                if (ref_period > 0)
                    blaReRescaleUnderflow(S, wr, wi, nwr, nwi);
                else
                    return 0;
            } else {
                double wmag = std::sqrt(wm2);
                S = fe_mul(S, fe_from(wmag));
                double inv = 1.0 / wmag;
                wr = nwr * inv;
                wi = nwi * inv;
            }
        } else {
            FE dzr = fe_mul_d(S, wr), dzi = fe_mul_d(S, wi);
            FE dcrfe = fe_mul_d(S, dr), dcife = fe_mul_d(S, di);
            FE nzr = fe_add(fe_sub(fe_mul_d(dzr, bc[0]), fe_mul_d(dzi, bc[1])), fe_sub(fe_mul_d(dcrfe, bc[2]), fe_mul_d(dcife, bc[3])));
            FE nzi = fe_add(fe_add(fe_mul_d(dzr, bc[1]), fe_mul_d(dzi, bc[0])), fe_add(fe_mul_d(dcrfe, bc[3]), fe_mul_d(dcife, bc[2])));
            double fr = zfr[land] + fe_to_double(nzr), fi = zfi[land] + fe_to_double(nzi);
            if (fr * fr + fi * fi > ESC2) return 0;
            FE Snew = fe_sqrt(fe_add(fe_mul(nzr, nzr), fe_mul(nzi, nzi)));
            if (Snew.m == 0.0) {
                S = FE{1.0, 0};
                wr = wi = 0.0;
            } else {
                S = Snew;
                wr = fe_to_double(fe_div(nzr, S));
                wi = fe_to_double(fe_div(nzi, S));
            }
        }
        if (ab) {
            ab[0] = bc[0];
            ab[1] = bc[1];
            ab[2] = bc[2];
            ab[3] = bc[3];
        }
        return l;
    }
    return 0;
}

// mp.cpp:3287-3618 (smooth / EDE / DE-overlay; no stripe or trap accumulators).
float Engine::pixelRescaled(FE dcr, FE dci, int mx_ref_it, int mxit, int cm, float* nrm, int* nout) const {
    *nout = -1;
    const double LG2 = std::log(2.0);
    const int reflen = mx_ref_it + 1;
    const int per = ref_period;
    int rm = 0;
    FE S = fe_sqrt(fe_add(fe_mul(dcr, dcr), fe_mul(dci, dci)));
    double wr, wi, dr, di;
    if (S.m == 0.0) {
        S = FE{1.0, 0};
        wr = wi = dr = di = 0.0;
    } else {
        wr = fe_to_double(fe_div(dcr, S));
        wi = fe_to_double(fe_div(dci, S));
        dr = wr;
        di = wi;
    }
    double s = fe_to_double(S);
    FE S2 = fe_mul(S, S);
    int m = 1, iter = 1;
    double zsr = 1e30, zsi = 1e30;
    int save_iter = 1, period_win = 1;
    int conf_P = 0, conf_next = 0, conf_count = 0, conf_giveup = 0;
    double conf_D2 = 0, conf_zr = 0, conf_zi = 0;
    const bool ede = (cm & CM_EDE) != 0;
    const bool de_ovl = (cm & CM_DEOVL) != 0;
    const bool normal = (cm & CM_NORMAL) != 0;
    const bool deriv = ede || normal || de_ovl;
    FE SJ{1.0, 0};
    double jr = 1.0, ji = 0.0, invSJd = 1.0;
    const bool detect_interior = use_interior;
    OrbitAcc oc; // mp.cpp:3338-3346, 3365-3366
    oc.init(cm);
    const bool int_rep = opt.int_rep > 0 && detect_interior && !oc.trap;
    double swr = 1e300, swi = 1e300;
    FE sS{1e300, 0};
    int sm = -1, save_iter2 = 1, twin2r = 1;
    while (iter < mxit) {
        if (int_rep) {
            if (m == sm && wr == swr && wi == swi && S.m == sS.m && S.e == sS.e) return -2.f;
            if (iter - save_iter2 >= twin2r) {
                swr = wr;
                swi = wi;
                sS = S;
                sm = m;
                save_iter2 = iter;
                twin2r += twin2r;
            }
        }
        if (use_bla && !oc.trap && m >= 2) { // mp.cpp:3389
            double ab[4];
            int skip = tryBLAfe(rm, S, S2, wr, wi, dr, di, per ? per : reflen, deriv ? ab : nullptr);
            if (skip > 0) {
                oc.skipped(); // mp.cpp:3393-3397
                if (deriv) {
                    FE Jr = fe_mul_d(SJ, jr), Ji = fe_mul_d(SJ, ji);
                    FE nJr = fe_add(fe_sub(fe_mul_d(Jr, ab[0]), fe_mul_d(Ji, ab[1])), fe_from(ab[2]));
                    FE nJi = fe_add(fe_add(fe_mul_d(Jr, ab[1]), fe_mul_d(Ji, ab[0])), fe_from(ab[3]));
                    SJ = fe_sqrt(fe_add(fe_mul(nJr, nJr), fe_mul(nJi, nJi)));
                    if (SJ.m == 0.0) {
                        SJ = FE{1.0, 0};
                        jr = ji = 0.0;
                        invSJd = 1.0;
                    } else {
                        jr = fe_to_double(fe_div(nJr, SJ));
                        ji = fe_to_double(fe_div(nJi, SJ));
                        invSJd = 1.0 / fe_to_double(SJ);
                    }
                }
                m += skip;
                iter += skip;
                rm += skip;
                if (per && rm >= per) rm -= per;
                s = fe_to_double(S);
                S2 = fe_mul(S, S);
                dr = fe_to_double(fe_div(dcr, S));
                di = fe_to_double(fe_div(dci, S));
                zsr = 1e30;
                zsi = 1e30;
                save_iter = iter;
                period_win = 1;
                conf_P = 0;
                conf_giveup = 0;
                continue;
            }
        }
        double Xr = m ? zfr[rm] : 0.0, Xi = m ? zfi[rm] : 0.0;
        double zmr = Xr + s * wr, zmi = Xi + s * wi;
        const bool deriv_underflow = deriv && zmr == 0.0 && zmi == 0.0 && invSJd == 0.0;
        FE zmrfe{0, 0}, zmife{0, 0};
        if (deriv_underflow) {
            FE Xrfe = m ? zfr_fe[rm] : FE{0.0, 0};
            FE Xife = m ? zfi_fe[rm] : FE{0.0, 0};
            zmrfe = fe_add(Xrfe, fe_mul_d(S, wr));
            zmife = fe_add(Xife, fe_mul_d(S, wi));
        }
        double nwr, nwi;
        if (opt.fused > 0) {
            const double fR = Xr + Xr + s * wr;
            const double fI = Xi + Xi + s * wi;
            nwr = fR * wr - fI * wi + dr;
            nwi = fR * wi + fI * wr + di;
        } else {
            double w2r = wr * wr - wi * wi, w2i = 2.0 * wr * wi;
            nwr = 2.0 * (Xr * wr - Xi * wi) + s * w2r + dr;
            nwi = 2.0 * (Xr * wi + Xi * wr) + s * w2i + di;
        }
        const bool step_underflow = std::fabs(nwr) < 0x1p-1056 && std::fabs(nwi) < 0x1p-1056;
        if (step_underflow && (nwr != 0.0 || nwi != 0.0 || wr != 0.0 || wi != 0.0 || dcr.m != 0.0 || dci.m != 0.0)) {
            FE Xrfe = m ? zfr_fe[rm] : FE{0.0, 0};
            FE Xife = m ? zfi_fe[rm] : FE{0.0, 0};
            feStepUnderflow(Xrfe, Xife, dcr, dci, S, wr, wi);
            s = fe_to_double(S);
            S2 = fe_mul(S, S);
            dr = fe_to_double(fe_div(dcr, S));
            di = fe_to_double(fe_div(dci, S));
        } else {
            wr = nwr;
            wi = nwi;
        }
        ++m;
        ++iter;
        rm++;
        if (per && rm == per) rm = 0;
        if (deriv) {
            if (deriv_underflow) {
                feDerivUnderflow(zmrfe, zmife, SJ, jr, ji, invSJd);
            } else {
                double a = 2.0 * (zmr * jr - zmi * ji) + invSJd;
                double b = 2.0 * (zmr * ji + zmi * jr);
                jr = a;
                ji = b;
                double jm2 = jr * jr + ji * ji;
                if (jm2 > 1e16 || (jm2 > 0.0 && jm2 < 1e-16)) {
                    FE jmag = fe_sqrt(fe_from(jm2));
                    SJ = fe_mul(SJ, jmag);
                    double inv = 1.0 / fe_to_double(jmag);
                    jr *= inv;
                    ji *= inv;
                    invSJd = 1.0 / fe_to_double(SJ);
                }
            }
        }
        Xr = m ? zfr[rm] : 0.0;
        Xi = m ? zfi[rm] : 0.0;
        double zr = Xr + s * wr, zi = Xi + s * wi;
        double zrad = zr * zr + zi * zi;
        oc.push(zr, zi); // mp.cpp:3503-3504
        if (zrad > ESC2) {
            *nout = iter;
            if (ede) {
                double num = std::sqrt(zrad) * std::log(zrad);
                FE Jmag = fe_mul_d(SJ, std::sqrt(jr * jr + ji * ji));
                return (float)fe_to_double(fe_div(fe_from(num), fe_mul(dxfe, Jmag)));
            }
            if (normal) { // mp.cpp:3512-3515
                if (nrm) *nrm = (float)(std::atan2(zi, zr) - std::atan2(ji, jr));
                return (float)((double)iter - std::log(std::log(zrad) / 2.0 / LG2) / LG2);
            }
            if (de_ovl) {
                double num = std::sqrt(zrad) * std::log(zrad);
                FE Jmag = fe_mul_d(SJ, std::sqrt(jr * jr + ji * ji));
                if (nrm) *nrm = (float)fe_to_double(fe_div(fe_from(num), fe_mul(dxfe, Jmag)));
                return (float)((double)iter - std::log(std::log(zrad) / 2.0 / LG2) / LG2);
            }
            if (oc.sac || oc.trap) return oc.escaped((double)iter - std::log(std::log(zrad) / 2.0 / LG2) / LG2, zrad, (double)escf); // mp.cpp:3524-3529
            return (float)((double)iter - std::log(std::log(zrad) / 2.0 / LG2) / LG2);
        }
        if (detect_interior) {
            if (conf_P > 0) {
                conf_D2 *= 4.0 * zrad;
                if (conf_D2 > 1e18) conf_D2 = 1e18;
                if (iter >= conf_next) {
                    double pr = zr - conf_zr, pi = zi - conf_zi;
                    if (pr * pr + pi * pi < interior_eps2 * zrad && conf_D2 < 1.0) {
                        if (++conf_count >= interior_confirm) return oc.interior();
                        conf_zr = zr;
                        conf_zi = zi;
                        conf_D2 = 1;
                        conf_next = iter + conf_P;
                    } else {
                        conf_P = 0;
                        ++conf_giveup;
                    }
                }
            } else if ((iter & 15) == 0 && conf_giveup < 3) {
                double pr = zr - zsr, pi = zi - zsi;
                if (pr * pr + pi * pi < interior_eps2 * zrad) {
                    conf_P = iter - save_iter;
                    if (conf_P < 1) conf_P = 1;
                    conf_zr = zr;
                    conf_zi = zi;
                    conf_D2 = 1;
                    conf_next = iter + conf_P;
                    conf_count = 0;
                }
                if (iter - save_iter >= period_win) {
                    zsr = zr;
                    zsi = zi;
                    save_iter = iter;
                    period_win += period_win;
                }
            }
        }
        double wmag2 = wr * wr + wi * wi;
        if (wmag2 > 1e16 || (wmag2 < 1e-16 && wmag2 > 0.0)) {
            FE wmag = fe_sqrt(fe_from(wmag2));
            S = fe_mul(S, wmag);
            s = fe_to_double(S);
            S2 = fe_mul(S, S);
            double inv = 1.0 / fe_to_double(wmag);
            wr *= inv;
            wi *= inv;
            dr = fe_to_double(fe_div(dcr, S));
            di = fe_to_double(fe_div(dci, S));
        }
        double dzmag2 = s * s * (wr * wr + wi * wi);
        if (zrad < 1e-8 || zrad < dzmag2 || (!per && m >= reflen)) {
            FE Xmr = m ? zfr_fe[rm] : FE{0.0, 0};
            FE Xmi = m ? zfi_fe[rm] : FE{0.0, 0};
            FE Swr = fe_mul_d(S, wr), Swi = fe_mul_d(S, wi);
            FE zrfe = fe_add(Xmr, Swr), zife = fe_add(Xmi, Swi);
            FE zradfe = fe_add(fe_mul(zrfe, zrfe), fe_mul(zife, zife));
            FE dzfe = fe_add(fe_mul(Swr, Swr), fe_mul(Swi, Swi));
            if ((!per && m >= reflen) || fe_abs_less(zradfe, dzfe)) {
                FE Snew = fe_sqrt(zradfe);
                if (Snew.m == 0.0) {
                    wr = wi = 0.0;
                } else {
                    S = Snew;
                    s = fe_to_double(S);
                    S2 = fe_mul(S, S);
                    wr = fe_to_double(fe_div(zrfe, S));
                    wi = fe_to_double(fe_div(zife, S));
                    dr = fe_to_double(fe_div(dcr, S));
                    di = fe_to_double(fe_div(dci, S));
                }
                m = 0;
                rm = -1;
            }
        }
    }
    return oc.interior();
}

// mp.cpp:3620-3816 for one lane (lanes are independent).
float Engine::rescaledNoBla(FE dcr, FE dci, int mx_ref_it, int mxit, int* nout) const {
    *nout = -1;
    const double logTwo = std::log(2.0);
    const int referenceLength = mx_ref_it + 1;
    double wr = 0, wi = 0, sd, dr = 0, di = 0;
    FE scale;
    const FE s0 = fe_sqrt(fe_add(fe_mul(dcr, dcr), fe_mul(dci, dci)));
    if (s0.m == 0.0) {
        scale = FE{1.0, 0};
    } else {
        scale = s0;
        wr = fe_to_double(fe_div(dcr, s0));
        wi = fe_to_double(fe_div(dci, s0));
        dr = wr;
        di = wi;
    }
    sd = fe_to_double(scale);
    int index = 1, iteration = 1;
    for (;;) {
        if (iteration >= mxit) return -2.0f;
        double pr = 0, pi = 0;
        if (index > 0) {
            pr = zfr[index - 1];
            pi = zfi[index - 1];
        }
        const int current = index > mx_ref_it ? mx_ref_it : index;
        double cr = zfr[current], ci = zfi[current];
        double nwr, nwi;
        if (opt.fused > 0) {
            const double fR = (pr + pr) + (sd * wr);
            const double fI = (pi + pi) + (sd * wi);
            nwr = ((fR * wr) - (fI * wi)) + dr;
            nwi = ((fR * wi) + (fI * wr)) + di;
        } else {
            const double sqR = (wr * wr) - (wi * wi), sqI = 2.0 * (wr * wi);
            const double lR = (pr * wr) - (pi * wi), lI = (pr * wi) + (pi * wr);
            nwr = ((2.0 * lR) + (sd * sqR)) + dr;
            nwi = ((2.0 * lI) + (sd * sqI)) + di;
        }
        const double aR = cr + (sd * nwr), aI = ci + (sd * nwi);
        double actual = (aR * aR) + (aI * aI);
        double delta = (nwr * nwr) + (nwi * nwi);
        if (delta == 0.0 && (nwr != 0.0 || nwi != 0.0 || wr != 0.0 || wi != 0.0 || dcr.m != 0.0 || dci.m != 0.0)) {
            const FE rR = index ? zfr_fe[index - 1] : FE{0.0, 0};
            const FE rI = index ? zfi_fe[index - 1] : FE{0.0, 0};
            feStepUnderflow(rR, rI, dcr, dci, scale, wr, wi);
            sd = fe_to_double(scale);
            dr = fe_to_double(fe_div(dcr, scale));
            di = fe_to_double(fe_div(dci, scale));
            const FE ar = fe_add(zfr_fe[current], fe_mul_d(scale, wr));
            const FE ai = fe_add(zfi_fe[current], fe_mul_d(scale, wi));
            actual = fe_to_double(fe_add(fe_mul(ar, ar), fe_mul(ai, ai)));
            delta = wr * wr + wi * wi;
        } else {
            wr = nwr;
            wi = nwi;
        }
        ++index;
        ++iteration;
        if (actual > ESC2) {
            *nout = iteration;
            return static_cast<float>(static_cast<double>(iteration) - std::log(std::log(actual) / 2.0 / logTwo) / logTwo);
        }
        if (delta > 1e16 || (delta < 1e-16 && delta > 0.0)) {
            const FE nm = fe_sqrt(fe_from(delta));
            scale = fe_mul(scale, nm);
            sd = fe_to_double(scale);
            const double inverse = 1.0 / fe_to_double(nm);
            wr *= inverse;
            wi *= inverse;
            dr = fe_to_double(fe_div(dcr, scale));
            di = fe_to_double(fe_div(dci, scale));
        }
        const double absd = sd * sd * (wr * wr + wi * wi);
        if (actual < 1e-8 || actual < absd || index >= referenceLength) {
            const FE rR = index ? zfr_fe[index - 1] : FE{0.0, 0};
            const FE rI = index ? zfi_fe[index - 1] : FE{0.0, 0};
            const FE sR = fe_mul_d(scale, wr), sI = fe_mul_d(scale, wi);
            const FE aRf = fe_add(rR, sR), aIf = fe_add(rI, sI);
            const FE a2 = fe_add(fe_mul(aRf, aRf), fe_mul(aIf, aIf));
            const FE d2 = fe_add(fe_mul(sR, sR), fe_mul(sI, sI));
            if (index >= referenceLength || fe_abs_less(a2, d2)) {
                const FE ns = fe_sqrt(a2);
                if (ns.m == 0.0) {
                    wr = wi = 0.0;
                } else {
                    scale = ns;
                    sd = fe_to_double(ns);
                    wr = fe_to_double(fe_div(aRf, ns));
                    wi = fe_to_double(fe_div(aIf, ns));
                    dr = fe_to_double(fe_div(dcr, ns));
                    di = fe_to_double(fe_div(dci, ns));
                }
                index = 0;
            }
        }
    }
}

// mp.cpp:2092-2607 (scalar delta loop; SAC/trap/custom branches omitted).
void Engine::stepParallel(std::set<std::array<int, 4>>& s, int mx_ref_it, int mxit, int cm, const std::vector<std::array<int, 4>>* contiguous) {
    ++stat_passes;
    std::vector<std::array<int, 4>> owned;
    if (!contiguous) owned.assign(s.begin(), s.end());
    const std::vector<std::array<int, 4>>& v = contiguous ? *contiguous : owned;
    const int n = (int)v.size();
    std::vector<char> done(n, 0);
    std::vector<double> glitch_p(n, -1.0);
    const bool ede = (cm & CM_EDE) != 0;
    const bool de_ovl = (cm & CM_DEOVL) != 0;
    const bool normal = (cm & CM_NORMAL) != 0;
    const bool deriv = ede || normal || de_ovl;
    long long steps = 0, blas = 0, skipped = 0, gmp = 0;
    if (use_floatexp) {
        const bool noBla = !use_bla && !deriv && !(cm & (CM_SAC | CM_TRAP)); // mp.cpp:2148
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : gmp)
        for (int i = 0; i < n; ++i) {
            const Pix arr = P(v[i]);
            double px = arr.a[1] + (double)arr.a[3] / SUB;
            double py = arr.a[0] + (double)arr.a[2] / SUB;
            FE Dcr = fe_mul_d(dxfe, px - ref_x);
            FE Dci = fe_mul_d(dyfe, py - ref_y);
            float nrm = 0.0f;
            int nn = -1;
            float value = noBla ? rescaledNoBla(Dcr, Dci, mx_ref_it, mxit, &nn) : pixelRescaled(Dcr, Dci, mx_ref_it, mxit, cm, (normal || de_ovl) ? &nrm : nullptr, &nn);
            if (value == EMPTY || (fe_cutoff_sensitive && (value < 0 || value > mxit - 16))) {
                value = accuratePixel(arr, mxit, cm, &nn);
                ++gmp;
            }
            setPixel(arr, value, nn);
            if ((normal || de_ovl) && normal_) normal_[idx(arr)] = nrm;
            done[i] = 1;
        }
        stat_gmp += gmp;
        if (contiguous) return;
        int i = 0;
        for (auto it = s.begin(); it != s.end(); ++i)
            if (done[i]) it = s.erase(it);
            else ++it;
        return;
    }
    const double dxf = mpf_ld(dx);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : steps, blas, skipped)
    for (int i = 0; i < n; ++i) {
        const Pix arr = P(v[i]);
        mpf_t a1, a2;
        mpf_init(a1);
        mpf_init(a2);
        int xpix = SUB * (arr.a[1] - ref_.a[1]) + (arr.a[3] - ref_.a[3]);
        int ypix = SUB * (arr.a[0] - ref_.a[0]) + (arr.a[2] - ref_.a[2]);
        mpf_mul_ui(a1, dx, std::abs(xpix));
        mpf_mul_ui(a2, dy, std::abs(ypix));
        if (xpix < 0) mpf_neg(a1, a1);
        if (ypix < 0) mpf_neg(a2, a2);
        if (SUB > 1) {
            mpf_div_ui(a1, a1, SUB);
            mpf_div_ui(a2, a2, SUB);
        }
        C2 dc{mpf_ld(a1), mpf_ld(a2)};
        mpf_clear(a1);
        mpf_clear(a2);
        if (ref_period) dc = C2{dc.re - ref_frac_re, dc.im - ref_frac_im};
        C2 dz{0, 0}, dd{0, 0};
        for (int x = SA_order; x >= 0; --x) {
            dz = c_add(dz, Adf_old[x]);
            dz = c_mul(dz, dc);
            dz = c_div(dz, SA_delta);
        }
        if (deriv) {
            for (int x = SA_order; x >= 0; --x) {
                dd = c_add(dd, Bdf_old[x]);
                dd = c_mul(dd, dc);
                dd = c_div(dd, SA_delta);
            }
        }
        int j = SA_it + 1;
        double dzr = dz.re, dzi = dz.im, dcr = dc.re, dci = dc.im, ddr = dd.re, ddi = dd.im;
        double tmp, zr, zi, dr = 0, di = 0, dzr2, dzi2, zrad;
        int k = j;
        const int per = ref_period;
        int rk = k, rkm1 = k - 1;
        double zsr = 1e30, zsi = 1e30;
        int save_j = j, period_win = 1;
        int conf_P = 0, conf_next = 0, conf_count = 0, conf_giveup = 0;
        double conf_D2 = 0, conf_zr = 0, conf_zi = 0;
        const bool detect_interior = use_interior;
        OrbitAcc oc; // mp.cpp:2362-2364, 2387-2388
        oc.init(cm);
        const bool int_rep = opt.int_rep > 0 && detect_interior && !oc.trap;
        double sdzr = 1e300, sdzi = 1e300;
        int sk = -1, save_j2 = j, twin2 = 1;
        bool fin = false;
        while (j < mxit) {
            if (int_rep) {
                if (k == sk && dzr == sdzr && dzi == sdzi) {
                    setPixel(arr, -2, -1);
                    done[i] = 1;
                    fin = true;
                    break;
                }
                if (j - save_j2 >= twin2) {
                    sdzr = dzr;
                    sdzi = dzi;
                    sk = k;
                    save_j2 = j;
                    twin2 += twin2;
                }
            }
            if (use_bla && !oc.trap && dzr * dzr + dzi * dzi < bla_rmax2) { // mp.cpp:2121
                int skip = tryBLA(rkm1, dzr, dzi, ddr, ddi, dcr, dci, deriv, mx_ref_it);
                if (skip > 0) {
                    ++blas;
                    skipped += skip;
                    k += skip;
                    j += skip;
                    rk += skip;
                    if (per && rk >= per) rk -= per;
                    rkm1 = (per && rk == 0) ? per - 1 : rk - 1;
                    oc.skipped(); // mp.cpp:2422-2427
                    zsr = 1e30;
                    zsi = 1e30;
                    save_j = j;
                    period_win = 1;
                    conf_P = 0;
                    conf_giveup = 0;
                    continue;
                }
            }
            ++steps;
            if (deriv) {
                if (k == 0) {
                    tmp = (dzr * (1 + ddr) - dzi * (1 + ddi)) * 2;
                    ddi = (dzr * (1 + ddi) + dzi * (1 + ddr)) * 2;
                } else {
                    tmp = (ddr * zfr[k - 1] - ddi * zfi[k - 1] + dzr * (dfr[k - 1] + ddr) - dzi * (dfi[k - 1] + ddi)) * 2;
                    ddi = (ddr * zfi[k - 1] + ddi * zfr[k - 1] + dzr * (dfi[k - 1] + ddi) + dzi * (dfr[k - 1] + ddr)) * 2;
                }
                ddr = tmp;
                dr = ddr + dfr[k];
                di = ddi + dfi[k];
            }
            dzr2 = dzr * dzr;
            dzi2 = dzi * dzi;
            if (k == 0) {
                tmp = dzr2 - dzi2 + dcr;
                dzi = dzr * dzi * 2 + dci;
            } else {
                tmp = (dzr * zfr[rkm1] - dzi * zfi[rkm1]) * 2 + dzr2 - dzi2 + dcr;
                dzi = (dzr * zfi[rkm1] + dzi * zfr[rkm1]) * 2 + dzr * dzi * 2 + dci;
            }
            dzr = tmp;
            zr = dzr + zfr[rk];
            zi = dzi + zfi[rk];
            zrad = zr * zr + zi * zi;
            oc.push(zr, zi); // mp.cpp:2471-2472
            ++k;
            rkm1 = rk;
            if (per) {
                if (++rk == per) rk = 0;
            } else
                rk = k;
            if (zrad > ESC2) {
                if (ede) {
                    setPixel(arr, std::sqrt(zrad) / dxf * std::log(zrad) / std::sqrt(dr * dr + di * di), j + 1);
                } else if (normal) { // mp.cpp:2489-2492
                    setPixel(arr, j + 1 - std::log(std::log((double)zrad) / 2 / std::log(2)) / std::log(2), j + 1);
                    if (normal_) normal_[idx(arr)] = (float)(std::atan2((double)zi, (double)zr) - std::atan2((double)di, (double)dr));
                } else if (de_ovl) {
                    setPixel(arr, j + 1 - std::log(std::log((double)zrad) / 2 / std::log(2)) / std::log(2), j + 1);
                    if (normal_) normal_[idx(arr)] = (float)(std::sqrt(zrad) / dxf * std::log(zrad) / std::sqrt(dr * dr + di * di));
                } else if (oc.sac || oc.trap) { // mp.cpp:2497-2500
                    setPixel(arr, oc.escaped(j + 1 - std::log(std::log((double)zrad) / 2 / std::log(2)) / std::log(2), (double)zrad, (double)escf), j + 1);
                } else {
                    setPixel(arr, j + 1 - std::log(std::log((double)zrad) / 2 / std::log(2)) / std::log(2), j + 1);
                }
                done[i] = 1;
                fin = true;
                break;
            }
            if (detect_interior) {
                if (conf_P > 0) {
                    conf_D2 *= 4 * zrad;
                    if (conf_D2 > 1e18) conf_D2 = 1e18;
                    if (j >= conf_next) {
                        double pr = zr - conf_zr, pi = zi - conf_zi;
                        bool ret = (pr * pr + pi * pi < interior_eps2 * zrad);
                        if (ret && conf_D2 < 1.0) {
                            if (++conf_count >= interior_confirm) {
                                setPixel(arr, oc.interior(), -1);
                                done[i] = 1;
                                fin = true;
                                break;
                            }
                            conf_zr = zr;
                            conf_zi = zi;
                            conf_D2 = 1;
                            conf_next = j + conf_P;
                        } else {
                            conf_P = 0;
                            ++conf_giveup;
                        }
                    }
                } else if ((j & 15) == 0 && conf_giveup < 3) {
                    double pr = zr - zsr, pi = zi - zsi;
                    if (pr * pr + pi * pi < interior_eps2 * zrad) {
                        conf_P = j - save_j;
                        if (conf_P < 1) conf_P = 1;
                        conf_zr = zr;
                        conf_zi = zi;
                        conf_D2 = 1;
                        conf_next = j + conf_P;
                        conf_count = 0;
                    }
                    if (j - save_j >= period_win) {
                        zsr = zr;
                        zsi = zi;
                        save_j = j;
                        period_win += period_win;
                    }
                }
            }
            if (zrad < dzr * dzr + dzi * dzi || (!per && k == mx_ref_it)) {
                if ((dzr * dzr + dzi * dzi) / zrad > 10000000) {
                    glitch_p[i] = zrad / z_m3[per ? j % per : j];
                    fin = true;
                    break;
                }
                dzr = zr;
                dzi = zi;
                if (deriv) {
                    ddr = dr - 1;
                    ddi = di;
                }
                k = 0;
                rk = 0;
                rkm1 = per ? per - 1 : -1;
            }
            if (!per && k == mx_ref_it) {
                glitch_p[i] = (double)zrad / z_m3[j];
                fin = true;
                break;
            }
            ++j;
        }
        (void)fin;
        if (j >= mxit) {
            setPixel(arr, oc.interior(), -1);
            done[i] = 1;
        }
    }
    stat_steps += steps;
    stat_bla += blas;
    stat_skipped += skipped;
    double min_orbit = 1e100;
    for (int i = 0; i < n; ++i) {
        if (glitch_p[i] >= 0 && glitch_p[i] < min_orbit) {
            min_orbit = glitch_p[i];
            new_ref = P(v[i]);
        }
    }
    int i = 0;
    for (auto it = s.begin(); it != s.end(); ++i) {
        if (done[i]) it = s.erase(it);
        else ++it;
    }
}

void Engine::truth(mpf_srcptr c_re, mpf_srcptr c_im, mpf_srcptr scale, int full_h, int row_base, int mxit, int cm, const int* keys, int n, int wp, float* out, int* nout) {
    // Same grid as compute() (mp.cpp:1403-1424).
    int rows = (full_h > 0) ? full_h : H;
    mpf_t dw, dh;
    mpf_init_set_ui(dw, 2);
    mpf_div(dw, dw, scale);
    mpf_init_set(dh, dw);
    mpf_div_ui(dh, dh, W);
    mpf_mul_ui(dh, dh, rows);
    mpf_sub(c0_re, c_re, dw);
    mpf_sub(c0_im, c_im, dh);
    mpf_div_ui(dx, dw, W - 1);
    mpf_mul_ui(dx, dx, 2);
    mpf_div_ui(dy, dh, rows - 1);
    mpf_mul_ui(dy, dy, 2);
    if (row_base > 0) {
        mpf_t off;
        mpf_init(off);
        mpf_mul_ui(off, dy, row_base);
        mpf_add(c0_im, c0_im, off);
        mpf_clear(off);
    }
    mpf_clear(dw);
    mpf_clear(dh);
#pragma omp parallel for schedule(dynamic, 1)
    for (int q = 0; q < n; ++q) {
        mpf_t cre, cim, off, soff;
        mpf_init2(cre, wp); mpf_init2(cim, wp); mpf_init2(off, wp); mpf_init2(soff, wp);
        const int* a = keys + 4 * q;
        mpf_set(cre, c0_re);
        mpf_set(cim, c0_im);
        mpf_mul_ui(off, dx, a[1]);
        mpf_add(cre, cre, off);
        mpf_mul_ui(off, dx, std::abs(a[3]));
        mpf_set(soff, off);
        if (a[3] < 0) mpf_neg(soff, soff);
        mpf_div_ui(soff, soff, SUB);
        mpf_add(cre, cre, soff);
        mpf_mul_ui(off, dy, a[0]);
        mpf_add(cim, cim, off);
        mpf_mul_ui(off, dy, std::abs(a[2]));
        mpf_set(soff, off);
        if (a[2] < 0) mpf_neg(soff, soff);
        mpf_div_ui(soff, soff, SUB);
        mpf_add(cim, cim, soff);
        int nn = -1;
        // the normal map's truth is the angle (the reference's point routine
        // returns the smooth value there)
        out[q] = accuratePoint(cre, cim, mxit, (cm & CM_NORMAL) && !(cm & CM_EDE) ? (cm | kTruthAngle) : cm, &nn);
        if (nout) nout[q] = nn;
        mpf_clears(cre, cim, off, soff, (mpf_ptr)0);
    }
}

// mp.cpp:1388-2028 (Mandelbrot mode).
void Engine::compute(mpf_srcptr c_re, mpf_srcptr c_im, mpf_srcptr scale, int mxit, int cm, int full_h, int row_base) {
    mpf_set(scale_, scale);
    int rows = (full_h > 0) ? full_h : H;
    mpf_t dw, dh;
    mpf_init_set_ui(dw, 2);
    mpf_div(dw, dw, scale);
    mpf_init_set(dh, dw);
    mpf_div_ui(dh, dh, W);
    mpf_mul_ui(dh, dh, rows);
    mpf_sub(c0_re, c_re, dw);
    mpf_sub(c0_im, c_im, dh);
    mpf_div_ui(dx, dw, W - 1);
    mpf_mul_ui(dx, dx, 2);
    mpf_div_ui(dy, dh, rows - 1);
    mpf_mul_ui(dy, dy, 2);
    if (row_base > 0) {
        mpf_t off;
        mpf_init(off);
        mpf_mul_ui(off, dy, row_base);
        mpf_add(c0_im, c0_im, off);
        mpf_clear(off);
    }
    mpf_clear(dw);
    mpf_clear(dh);
    std::set<std::array<int, 4>> s;
    method = mpf_cmp_d(scale, 1e6) > 0 ? 1 : 0;
    int ref_it = 0;
    if (method == 0) {
        double c0r = mpf_ld(c0_re), c0i = mpf_ld(c0_im), dxf = mpf_ld(dx), dyf = mpf_ld(dy);
        const bool ede = (cm & CM_EDE) != 0;
        const bool deovl = (cm & CM_DEOVL) != 0;
        const bool nmap = (cm & CM_NORMAL) != 0;
#pragma omp parallel for schedule(dynamic, 1)
        for (int i = 0; i < H; ++i) {
            double cim = c0i + dyf * i;
            for (int j = 0; j < W; ++j) {
                Pix p{{i, j, 0, 0}};
                int nn = -1;
                if (nmap) { // mp.cpp:1504-1507
                    double nv = 0.0;
                    iter_[idx(p)] = (float)floatPoint(c0r + dxf * j, cim, mxit, cm, &nv, &nn);
                    if (escn_) escn_[idx(p)] = nn;
                    if (normal_) normal_[idx(p)] = (float)nv;
                } else if (cm & (CM_SAC | CM_TRAP)) { // scalar path (mp.cpp:1459, 1512-1515)
                    iter_[idx(p)] = (float)floatPoint(c0r + dxf * j, cim, mxit, cm, nullptr, &nn);
                    if (ede && iter_[idx(p)] >= 0) iter_[idx(p)] /= dxf;
                    if (escn_) escn_[idx(p)] = nn;
                } else if (!deovl) {
                    double val = shallowSimd(c0r + dxf * j, cim, mxit, cm, &nn);
                    if (ede && val >= 0) val /= dxf;
                    iter_[idx(p)] = (float)val;
                    if (escn_) escn_[idx(p)] = nn;
                } else {
                    double de = 0.0;
                    iter_[idx(p)] = (float)floatPoint(c0r + dxf * j, cim, mxit, cm, &de, &nn);
                    if (escn_) escn_[idx(p)] = nn;
                    if (normal_) normal_[idx(p)] = (iter_[idx(p)] < 0) ? 0.0f : (float)(de / dxf);
                }
            }
        }
    } else {
        use_bla = opt.bla != 0;
        bla_eps = opt.bla_eps;
        bla_minlevel = 0;
        while ((1 << (bla_minlevel + 1)) <= opt.bla_minskip) ++bla_minlevel;
        use_interior = opt.interior != 0;
        interior_eps2 = opt.int_eps * opt.int_eps;
        interior_confirm = opt.int_confirm;
        use_floatexp = opt.fe >= 0 ? opt.fe != 0 : (mpf_cmp_d(scale, 1e280) > 0);
        fe_cutoff_sensitive = false;
        dxfe = mpf_fe(dx);
        dyfe = mpf_fe(dy);
        ref_it = buildReferenceOrbit(s, scale, mxit, cm);
        if (ref_subpixel) use_bla = false;
        if (use_bla) buildBLA(ref_it, deriv_of(cm));
        if (use_interior) { // probe on the 1/8 grid (mp.cpp:1668-1720); coarse preview has no lasting effect
            const int C = 8;
            std::set<std::array<int, 4>> probe;
            for (int i = 0; i < H; i += C)
                for (int j = 0; j < W; j += C) probe.insert({i, j, 0, 0});
            if (!probe.empty()) stepParallel(probe, ref_it, mxit, cm);
            int nint = 0;
            for (int i = 0; i < H; i += C)
                for (int j = 0; j < W; j += C)
                    if (iter_[idx(Pix{{i, j, 0, 0}})] == -2) ++nint;
            if (nint == 0) use_interior = false;
        }
        for (int i = 0; i < H; ++i)
            for (int j = 0; j < W; ++j) s.insert({i, j, 0, 0});
        if (!ref_virtual) s.erase({H / 2, W / 2, 0, 0});
        while (!s.empty()) {
            stepParallel(s, ref_it, mxit, cm);
            if (s.empty()) break;
            ref_it = createRef(s, mxit, mxit, false, cm);
            ref_bounded = !ref_escaped;
            const bool ss_follows = (SUB > 1) && (cm & CM_SS);
            if ((!s.empty() || ss_follows) && use_bla) buildBLA(ref_it, deriv_of(cm));
        }
    }
    const bool is_ss = (SUB > 1) && (cm & CM_SS);
    if (!is_ss) return;
    // Adaptive supersampling (mp.cpp:1796-2006).
    std::vector<std::array<int, 2>> v;
    const double ss_thresh = std::log((double)mxit) / opt.ss_k;
    // the stripe average and the orbit traps store a value, not an iteration
    // count: the set boundary (a sign change) and, for traps, a colour change of
    // more than trap_ss_steps palette entries per pixel (mp.cpp:1810-1838, 1864-1870)
    const bool sac = (cm & CM_SAC) != 0, trap = (cm & CM_TRAP) != 0;
    const double sac_gain = (double)opt.ss_density * (2048.0 / 20.0);
    const double trap_gain = (double)opt.ss_density / 60.0 * 2048.0;
    for (int i = 0; i < H; ++i) {
        for (int j = 0; j < W; ++j) {
            bool need = false;
            if (cm & CM_EDE) {
                for (int xi = -1; xi <= 1 && !need; ++xi)
                    for (int yi = -1; yi <= 1; ++yi) {
                        if (xi == 0 && yi == 0) continue;
                        int ny = i + yi, nx = j + xi;
                        if (nx >= 0 && nx < W && ny >= 0 && ny < H && iter_[idx(Pix{{i, j, 0, 0}})] * iter_[idx(Pix{{ny, nx, 0, 0}})] < 0) {
                            need = true;
                            break;
                        }
                    }
            } else {
                float cv = iter_[idx(Pix{{i, j, 0, 0}})];
                float diff = 0;
                bool boundary = false;
                for (int xi = -1; xi <= 1; ++xi)
                    for (int yi = -1; yi <= 1; ++yi) {
                        if (xi == 0 && yi == 0) continue;
                        int ny = i + yi, nx = j + xi;
                        if (nx >= 0 && nx < W && ny >= 0 && ny < H) {
                            const float nv = iter_[idx(Pix{{ny, nx, 0, 0}})];
                            diff = std::max(diff, std::abs(cv - nv));
                            if ((sac || trap) && cv * nv < 0) boundary = true;
                        }
                    }
                if (sac)
                    need = boundary || (opt.sac_ss_steps > 0 && diff * sac_gain > opt.sac_ss_steps);
                else if (trap)
                    need = boundary || (diff * trap_gain > opt.trap_ss_steps);
                else
                    need = (std::log((double)diff) > ss_thresh); // log(float) resolves to ::log(double) in the reference build
            }
            if (need) v.push_back({i, j});
        }
    }
    if (method == 0) {
        double c0r = mpf_ld(c0_re), c0i = mpf_ld(c0_im), dxf = mpf_ld(dx), dyf = mpf_ld(dy);
        const bool ede = (cm & CM_EDE) != 0;
#pragma omp parallel for schedule(dynamic, 1)
        for (int q = 0; q < (int)v.size(); ++q) {
            for (int xi = -SUB / 2; xi <= SUB / 2; ++xi)
                for (int yi = -SUB / 2; yi <= SUB / 2; ++yi) {
                    if (xi == 0 && yi == 0) continue;
                    double cr = c0r + dxf * v[q][1] + dxf * xi / SUB;
                    double ci = c0i + dyf * v[q][0] + dyf * yi / SUB;
                    // sub^2 <= 128 takes the lane-refill kernel (float result; it has
                    // no stripe average, so SAC frames take the scalar path, and no
                    // orbit traps, so a trap frame's subsamples get the smooth count),
                    // larger sub the scalar floatPointCompute (double result)
                    // (mp.cpp:1931-1967).
                    int nn = -1;
                    const bool simd = (SUB * SUB <= 128) && !sac;
                    double it = simd ? (double)shallowSimd(cr, ci, mxit, cm, &nn) : floatPoint(cr, ci, mxit, cm & (CM_EDE | CM_SAC | CM_TRAP), nullptr, &nn);
                    if (ede && it >= 0) it /= dxf;
                    setPixel(Pix{{v[q][0], v[q][1], yi, xi}}, (float)it, nn);
                }
        }
        return;
    }
    const bool contiguous_fe = use_floatexp;
    std::vector<std::array<int, 4>> ssc;
    for (const auto& p : v)
        for (int yi = -SUB / 2; yi <= SUB / 2; ++yi)
            for (int xi = -SUB / 2; xi <= SUB / 2; ++xi) {
                if (xi == 0 && yi == 0) continue;
                if (contiguous_fe)
                    ssc.push_back({p[0], p[1], yi, xi});
                else
                    s.insert({p[0], p[1], yi, xi});
            }
    bool saved_bla = use_bla;
    if (contiguous_fe && !ssc.empty()) stepParallel(s, ref_it, mxit, cm, &ssc);
    while (!contiguous_fe && !s.empty()) {
        stepParallel(s, ref_it, mxit, cm);
        if (s.empty()) break;
        ref_it = createRef(s, mxit, mxit, false, cm);
        use_bla = false;
    }
    use_bla = saved_bla;
}

} // namespace

extern "C" {

// Oracle entry point. Renders one frame exactly like the reference's
// Mandel(W,H,mxit,sub,iter) + setPrecision(prec) + Compute(...) sequence after
// mpf_set_default_prec(prec). iter/normal hold (W*sub)*(H*sub) floats and are
// filled with EMPTYPIXEL / 0 first. stats (optional, 8 slots): executed delta
// steps, BLA applies, BLA-skipped iterations, passes, references built, GMP
// per-pixel recomputations, method (0 shallow / 1 perturbation). escn
// (optional) receives each sample's escape iteration N (-1 interior), an
// instrumentation output with no counterpart in the reference.
int mbx_oracle_render(const char* cx, const char* cy, const char* scale_digits, int prec_bits, int W, int H, int mxit, int sub, int cmethod, double bailout, int full_h, int row_base, int threads, float* iter, float* normal, int32_t* escn, long long* stats) {
    if (W < 2 || H < 1 || mxit < 1 || sub < 1 || (sub % 2) == 0 || !iter) return -1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    const size_t n = (size_t)W * H * sub * sub;
    for (size_t i = 0; i < n; ++i) iter[i] = EMPTY;
    if (normal)
        for (size_t i = 0; i < n; ++i) normal[i] = 0.0f;
    if (escn)
        for (size_t i = 0; i < n; ++i) escn[i] = -10;
    mpf_set_default_prec((mp_bitcnt_t)prec_bits);
    mpf_t mcx, mcy, msc;
    mpf_init_set_str(mcx, cx, 10);
    mpf_init_set_str(mcy, cy, 10);
    mpf_init_set_str(msc, scale_digits, 10);
    Opts o;
    {
        Engine e(W, H, mxit, sub, iter, normal, escn, bailout, o);
        e.setPrecision(prec_bits);
        e.compute(mcx, mcy, msc, mxit, cmethod, full_h, row_base);
        if (stats) {
            stats[0] = e.stat_steps;
            stats[1] = e.stat_bla;
            stats[2] = e.stat_skipped;
            stats[3] = e.stat_passes;
            stats[4] = e.stat_refs;
            stats[5] = e.stat_gmp;
            stats[6] = e.method;
            stats[7] = 0;
        }
    }
    mpf_clear(mcx);
    mpf_clear(mcy);
    mpf_clear(msc);
    return 0;
}

// Arbitrary-precision ground truth for listed samples (keys: n x {row, col,
// subrow, subcol}) of a frame, iterated at work_bits of precision with the
// reference's per-pixel GMP iteration (accuratePointCompute, mp.cpp:719-894).
int mbx_oracle_truth(const char* cx, const char* cy, const char* scale_digits, int prec_bits, int work_bits, int W, int H, int mxit, int sub, int cmethod, double bailout, int full_h, int row_base, int threads, const int* keys, int n, float* out, int32_t* nout) {
    if (W < 2 || H < 1 || mxit < 1 || sub < 1 || !keys || !out) return -1;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    mpf_set_default_prec((mp_bitcnt_t)prec_bits);
    mpf_t mcx, mcy, msc;
    mpf_init_set_str(mcx, cx, 10);
    mpf_init_set_str(mcy, cy, 10);
    mpf_init_set_str(msc, scale_digits, 10);
    Opts o;
    std::vector<float> dummy(1);
    {
        Engine e(W, H, mxit, sub, dummy.data(), nullptr, nullptr, bailout, o);
        e.setPrecision(prec_bits);
        e.truth(mcx, mcy, msc, full_h, row_base, mxit, cmethod, keys, n, work_bits > 0 ? work_bits : prec_bits, out, nout);
    }
    mpf_clear(mcx);
    mpf_clear(mcy);
    mpf_clear(msc);
    return 0;
}

// Resets libc rand() to its initial state so that repeated renders in one
// process replay the reference's rand() draws (createRef picks with rand()).
void mbx_oracle_reset_rand(void) { srand(1); }

// Mandel::ComputeJulia (mp.cpp:992-1044): geometry in mpf as written there,
// then per sample the scalar semantics of solveJuliaShallowSimdList
// (mp.cpp:534-636): z0 the sample, c fixed, D_0 = 1 and D' = 2 z D under EDE.
// escn receives the escape index (jv + 1; 0 when z0 is already outside; -1
// interior), which the reference does not output.
int mbx_oracle_julia(const char* cx, const char* cy, const char* scale_digits, int prec_bits, const char* fcr, const char* fci, int W, int H,
                     int mxit, int cmethod, double bailout, int full_h, int row_base, float* iter, int32_t* escn) {
    if (W < 2 || H < 1 || mxit < 1 || (cmethod & ~CM_EDE) != 0) return -1;
    if (full_h <= 0) full_h = H;
    if (full_h < H || row_base < 0 || row_base > full_h - H) return -1;
    mpf_set_default_prec((mp_bitcnt_t)prec_bits);
    mpf_t z0r, z0i, sc, cr, ci, dw, dh, c0r, c0i, dx, dy;
    mpf_init2(z0r, prec_bits); mpf_init2(z0i, prec_bits); mpf_init2(sc, prec_bits); mpf_init2(cr, prec_bits); mpf_init2(ci, prec_bits);
    mpf_init2(c0r, prec_bits); mpf_init2(c0i, prec_bits); mpf_init2(dx, prec_bits); mpf_init2(dy, prec_bits);
    int rc = 0;
    if (mpf_set_str(z0r, cx, 10) || mpf_set_str(z0i, cy, 10) || mpf_set_str(sc, scale_digits, 10) || mpf_set_str(cr, fcr, 10) || mpf_set_str(ci, fci, 10)) rc = -1;
    if (rc == 0) {
        mpf_init_set_ui(dw, 2);
        mpf_div(dw, dw, sc);
        mpf_init_set(dh, dw);
        mpf_mul_ui(dh, dh, full_h);
        mpf_div_ui(dh, dh, W);
        mpf_sub(c0r, z0r, dw);
        mpf_sub(c0i, z0i, dh);
        mpf_mul_ui(dx, dw, 2);
        mpf_div_ui(dx, dx, W - 1);
        mpf_mul_ui(dy, dh, 2);
        mpf_div_ui(dy, dy, full_h - 1);
        if (row_base != 0) {
            mpf_mul_ui(dw, dy, (unsigned long)row_base);
            mpf_add(c0i, c0i, dw);
        }
        mpf_clear(dw);
        mpf_clear(dh);
        const float escf = (float)(bailout > 0 ? bailout : 1e8);
        const double ESC2 = (double)(escf * escf); // escapeRadiusSquared (mp.h:115-118)
        const double LG2 = std::log(2.0);
        const double cRe = mpf_ld(cr), cIm = mpf_ld(ci);
        const double z0Re = mpf_ld(c0r), z0Im = mpf_ld(c0i);
        const double ddx = mpf_ld(dx), ddy = mpf_ld(dy);
        const bool ede = (cmethod & CM_EDE) != 0;
#pragma omp parallel for schedule(dynamic, 1)
        for (int i = 0; i < H; ++i) {
            const double imag = z0Im + ddy * i;
            for (int j = 0; j < W; ++j) {
                double zr = z0Re + ddx * j, zi = imag;
                double zrad = zr * zr + zi * zi;
                float result = -2.0f;
                int n = -1;
                if (zrad > ESC2) {
                    result = ede ? (float)(std::sqrt(zrad) * std::log(zrad)) : (float)(-std::log(std::log(zrad) / 2 / LG2) / LG2);
                    n = 0;
                } else {
                    double dr = 1.0, di = 0.0, jv = 0.0;
                    for (;;) {
                        double ndr = dr, ndi = di;
                        if (ede) {
                            ndr = 2.0 * (dr * zr - di * zi);
                            ndi = 2.0 * (dr * zi + di * zr);
                        }
                        const double nzr = zr * zr - zi * zi + cRe;
                        const double nzi = 2.0 * (zr * zi) + cIm;
                        zr = nzr;
                        zi = nzi;
                        dr = ndr;
                        di = ndi;
                        zrad = zr * zr + zi * zi;
                        const double jnext = jv + 1.0;
                        if (zrad > ESC2) {
                            if (ede) {
                                const double denom = std::sqrt(dr * dr + di * di);
                                result = denom > 0.0 ? (float)(std::sqrt(zrad) * std::log(zrad) / denom) : 0.0f;
                            } else {
                                result = (float)(jv + 1 - std::log(std::log(zrad) / 2 / LG2) / LG2);
                            }
                            n = (int)jv + 1;
                            break;
                        }
                        if (jnext >= (double)mxit) break;
                        jv = jnext;
                    }
                }
                if (ede && result >= 0.0f) result /= (float)ddx;
                iter[(size_t)i * W + j] = result;
                if (escn) escn[(size_t)i * W + j] = n;
            }
        }
    }
    mpf_clears(z0r, z0i, sc, cr, ci, c0r, c0i, dx, dy, (mpf_ptr)0);
    return rc;
}

// findNucleus on a disk (mp.cpp:1089-1102 after the disk set-up): ball period,
// Newton (200 iterations), inside-the-disk check. Writes the nucleus as GMP's
// shortest round-trip digits "d1d2...@exp" and returns the period (0: none).
int mbx_oracle_nucleus(const char* cx, const char* cy, const char* radius, int maxp, int prec, char* re, char* im, int len) {
    mpf_t cr, ci, r, nr, ni, dr, di, dist;
    mpf_init2(cr, prec); mpf_init2(ci, prec); mpf_init2(r, prec); mpf_init2(nr, prec);
    mpf_init2(ni, prec); mpf_init2(dr, prec); mpf_init2(di, prec); mpf_init2(dist, prec);
    int result = -1;
    if (mpf_set_str(cr, cx, 10) == 0 && mpf_set_str(ci, cy, 10) == 0 && mpf_set_str(r, radius, 10) == 0) {
        result = 0;
        const int p = g_ballPeriod(cr, ci, r, maxp, prec);
        mpf_set(nr, cr);
        mpf_set(ni, ci);
        if (p > 0 && g_newton(nr, ni, p, prec, 200)) {
            mpf_sub(dr, nr, cr);
            mpf_sub(di, ni, ci);
            mpf_mul(dr, dr, dr);
            mpf_mul(di, di, di);
            mpf_add(dist, dr, di);
            mpf_sqrt(dist, dist);
            if (mpf_cmp(dist, r) <= 0) result = p;
        }
        if (result > 0) {
            mpf_ptr v[2] = {nr, ni};
            char* out[2] = {re, im};
            for (int k = 0; k < 2; ++k) {
                mp_exp_t e;
                char* d = mpf_get_str(nullptr, &e, 10, 0, v[k]);
                snprintf(out[k], (size_t)len, "%s@%ld", d, (long)e);
                free(d);
            }
        }
    }
    mpf_clears(cr, ci, r, nr, ni, dr, di, dist, (mpf_ptr)0);
    return result;
}

} // extern "C"

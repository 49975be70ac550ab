// Host side of the GB300 renderer: view geometry and the serial arbitrary-
// precision reference orbit (GMP, on the host, uploaded once per reference),
// series-approximation coefficients, the periodic-nucleus reference, and the
// frame orchestration that drives the CUDA passes (probe gate, glitch
// re-reference passes, adaptive supersampling).
//
// The mpf operation sequences reproduce the reference's exactly, because the
// double/floatexp orbit shadows must be bit-identical for the per-pixel results
// to be. Citations: cbotx/Mandelbrot-Explorer src/engine/mandel_perturbation.cpp
// ("mp.cpp"), src/engine/bigfixed.h, src/engine/float_math.cpp.
#include "engine.h"
#include "orbit_color.h"
#include "parmul.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

namespace mbx {

namespace {

double now_ms() { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

// float_math.cpp:13-17 (truncating mpf -> double).
inline double mpf_ld(mpf_srcptr a) {
    long e;
    double d = mpf_get_d_2exp(&e, a);
    return xldexp(d, (int)e);
}
// mp.cpp:69-74.
inline FE mpf_fe(mpf_srcptr x) {
    if (mpf_sgn(x) == 0) return fe_make(0.0, 0);
    long ex;
    double d = mpf_get_d_2exp(&ex, x);
    return fe_make(d, (int64_t)ex);
}
// float_math.cpp:22-27.
inline int exp_floor_log2(double x) {
    if (x == 0.0) return -0x40000000;
    int e;
    (void)xfrexp(x, &e);
    return e - 1;
}

struct MpfTemp {
    mpf_t v;
    explicit MpfTemp(mp_bitcnt_t p) { mpf_init2(v, p); }
    ~MpfTemp() { mpf_clear(v); }
    operator mpf_ptr() { return v; }
    mpf_ptr operator->() { return v; }
};

// Parallel product rounds (parmul.h): destination k = a[k] * b[k].
struct MpfMulJob {
    mpf_ptr r[8];
    mpf_ptr a[8];
    mpf_ptr b[8];
};
void mpf_mul_job(void* ctx, int k) {
    MpfMulJob* j = static_cast<MpfMulJob*>(ctx);
    mpf_mul(j->r[k], j->a[k], j->b[k]);
}
// Precision from which the helpers pay for their synchronisation (a round of
// six products, of three or four, of two). Measured on the Neoverse V2 host: a
// parallel round costs ~0.5 us more than its products alone, which 18-limb
// (1100-bit) products do not repay and 54-limb (3400-bit) ones repay ~3x.
constexpr mp_bitcnt_t kParBits6 = 1600, kParBits4 = 2000, kParBits2 = 2800;

} // namespace

// ---------------------------------------------------------------------------
// Fixed-point reference arithmetic (the reference's BigFixed, bigfixed.h:143-320):
// L little-endian limbs, binary point below the top limb, sign-magnitude,
// round-to-nearest product.
void FixedReal::set_len(int l) {
    L = l;
    sign = 0;
    limb.assign((size_t)l, 0ull);
}

namespace {
typedef unsigned __int128 u128;
int mag_cmp(const uint64_t* a, const uint64_t* b, int L) {
    for (int i = L - 1; i >= 0; --i)
        if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
    return 0;
}
void mag_add(uint64_t* r, const uint64_t* a, const uint64_t* b, int L) {
    uint64_t c = 0;
    for (int i = 0; i < L; ++i) {
        u128 s = (u128)a[i] + b[i] + c;
        r[i] = (uint64_t)s;
        c = (uint64_t)(s >> 64);
    }
}
void mag_sub(uint64_t* r, const uint64_t* a, const uint64_t* b, int L) {
    uint64_t borrow = 0;
    for (int i = 0; i < L; ++i) {
        u128 d = (u128)a[i] - b[i] - borrow;
        r[i] = (uint64_t)d;
        borrow = (uint64_t)(d >> 127);
    }
}
// acc[t..] += a * b[0..n), propagating the carry no higher than index `top`.
void mul_row(uint64_t* acc, int t, const uint64_t* b, int n, uint64_t a, int top) {
    uint64_t carry = 0;
    for (int j = 0; j < n; ++j) {
        u128 p = (u128)a * b[j] + acc[t + j] + carry;
        acc[t + j] = (uint64_t)p;
        carry = (uint64_t)(p >> 64);
    }
    for (int u = t + n; carry && u <= top; ++u) {
        u128 s = (u128)acc[u] + carry;
        acc[u] = (uint64_t)s;
        carry = (uint64_t)(s >> 64);
    }
}
void round_up(uint64_t* r, int L) {
    for (int i = 0; i < L; ++i)
        if (++r[i] != 0) break;
}
} // namespace

void FixedReal::addsub(FixedReal& r, const FixedReal& a, int sa, const FixedReal& b, int sb) { // bigfixed.h:195-230
    const int L = a.L;
    r.L = L;
    if ((int)r.limb.size() != L) r.limb.resize(L);
    if (sa == 0) {
        memcpy(r.limb.data(), b.limb.data(), 8 * (size_t)L);
        r.sign = sb;
        return;
    }
    if (sb == 0) {
        memcpy(r.limb.data(), a.limb.data(), 8 * (size_t)L);
        r.sign = sa;
        return;
    }
    if (sa == sb) {
        mag_add(r.limb.data(), a.limb.data(), b.limb.data(), L);
        r.sign = sa;
        return;
    }
    int c = mag_cmp(a.limb.data(), b.limb.data(), L);
    if (c == 0) {
        std::fill(r.limb.begin(), r.limb.end(), 0ull);
        r.sign = 0;
    } else if (c > 0) {
        mag_sub(r.limb.data(), a.limb.data(), b.limb.data(), L);
        r.sign = sa;
    } else {
        mag_sub(r.limb.data(), b.limb.data(), a.limb.data(), L);
        r.sign = sb;
    }
}

void FixedReal::mul(FixedReal& r, const FixedReal& a, const FixedReal& b, uint64_t* tmp) { // bigfixed.h:106-125, 242-254
    const int L = a.L;
    r.L = L;
    if ((int)r.limb.size() != L) r.limb.resize(L);
    if (a.sign == 0 || b.sign == 0) {
        std::fill(r.limb.begin(), r.limb.end(), 0ull);
        r.sign = 0;
        return;
    }
    const uint64_t* x = a.limb.data();
    const uint64_t* y = b.limb.data();
    uint64_t* out = r.limb.data();
    if (L >= 16 && L < 72) { // high-half product with 3 guard limbs
        const int G = 3, lo = L - 1 - G, nout = 2 * L - lo;
        memset(tmp, 0, 8 * (size_t)(nout + 1));
        for (int i = 0; i < L; ++i) {
            int js = std::max(0, lo - i);
            mul_row(tmp, i + js - lo, y + js, L - js, x[i], nout);
        }
        for (int i = 0; i < L; ++i) out[i] = tmp[i + G];
        if (tmp[G - 1] >> 63) round_up(out, L);
    } else {
        memset(tmp, 0, 8 * (size_t)(2 * L));
        for (int i = 0; i < L; ++i) mul_row(tmp, i, y, L, x[i], 2 * L - 1);
        for (int i = 0; i < L; ++i) out[i] = tmp[L - 1 + i];
        if (L > 1 && (tmp[L - 2] >> 63)) round_up(out, L);
    }
    r.sign = (a.sign == b.sign) ? 1 : -1;
}

void FixedReal::from_mpf(mpf_srcptr x, int l) { // bigfixed.h:283-299
    set_len(l);
    if (mpf_sgn(x) == 0) return;
    sign = mpf_sgn(x);
    const int n = x->_mp_size < 0 ? -x->_mp_size : x->_mp_size;
    for (int i = 0; i < n; ++i) {
        long k = (long)i - n + x->_mp_exp + L - 1;
        if (k >= 0 && k < L) limb[k] = x->_mp_d[i];
    }
}

void FixedReal::to_mpf(mpf_ptr out) const { // bigfixed.h:272-280
    mpz_t z;
    mpz_init(z);
    mpz_import(z, (size_t)L, -1, sizeof(uint64_t), 0, 0, limb.data());
    mpf_set_z(out, z);
    mpf_div_2exp(out, out, (mp_bitcnt_t)64 * (L - 1));
    if (sign < 0) mpf_neg(out, out);
    mpz_clear(z);
}

FE FixedReal::to_fe() const { // bigfixed.h:305-320
    if (sign == 0) return fe_make(0.0, 0);
    int top = L - 1;
    while (top >= 0 && limb[top] == 0) --top;
    if (top < 0) return fe_make(0.0, 0);
    double mant = (double)limb[top] * 18446744073709551616.0 + (double)(top >= 1 ? limb[top - 1] : 0ull);
    FE r = fe_from(mant);
    r.e += (int64_t)64 * (top - L);
    return sign < 0 ? fe_neg(r) : r;
}

double FixedReal::to_double() const { // bigfixed.h:179-189
    if (sign == 0) return 0.0;
    int top = L - 1;
    while (top >= 0 && limb[top] == 0) --top;
    if (top < 0) return 0.0;
    double hi = (double)limb[top];
    double lo = (top >= 1) ? (double)limb[top - 1] : 0.0;
    double val = hi * 18446744073709551616.0 + lo;
    val = xldexp(val, 64 * (top - (L - 1) - 1));
    return sign < 0 ? -val : val;
}

// ---------------------------------------------------------------------------
Engine::Engine(int device) : device_(device) {}

Engine::~Engine() {
    release_device();
    if (mpf_ready_) {
        mpf_clear(c0_re_); mpf_clear(c0_im_); mpf_clear(dx_); mpf_clear(dy_); mpf_clear(scale_);
        mpf_clear(ref_re_); mpf_clear(ref_im_); mpf_clear(t1_); mpf_clear(t2_);
        for (int i = 0; i < 2; ++i) { mpf_clear(zre_[i]); mpf_clear(zim_[i]); }
    }
}

int Engine::init(std::string& err) {
    cudaError_t e = cudaSetDevice(device_);
    if (e != cudaSuccess) {
        err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return -1;
    }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device_);
    if (e != cudaSuccess) {
        err = std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e);
        return -1;
    }
    nsm_ = prop.multiProcessorCount;
    snprintf(devname_, sizeof(devname_), "%s (sm_%d%d, %d SMs)", prop.name, prop.major, prop.minor, nsm_);
    if (cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking) != cudaSuccess) return -1;
    // Counters of a pass, and of the double-float rerun pass that follows a mixed pass.
    if (cudaMalloc(&dctr_, 2 * sizeof(Counters)) != cudaSuccess) return -1;
    if (cudaEventCreate(&ev0_) != cudaSuccess || cudaEventCreate(&ev1_) != cudaSuccess || cudaEventCreate(&evm_) != cudaSuccess) return -1;
    if (cudaHostAlloc(&hctr_, 2 * sizeof(Counters), cudaHostAllocDefault) != cudaSuccess) return -1;
    if (cudaHostAlloc((void**)&hcancel_, sizeof(int), cudaHostAllocMapped) != cudaSuccess) return -1;
    *hcancel_ = 0;
    if (cudaHostGetDevicePointer((void**)&dcancel_, (void*)hcancel_, 0) != cudaSuccess) return -1;
    return 0;
}

void Engine::release_device() {
    if (st_) cudaStreamSynchronize(st_);
    for (void* p : {(void*)dZ_.p, (void*)dZfe_.p, (void*)dD_.p, (void*)dzm3_.p, (void*)dr2_.p, (void*)dab_.p, (void*)dce_.p,
                    (void*)ddcx_.p, (void*)ddcy_.p, (void*)diter_own_.p, (void*)dnormal_own_.p, (void*)descN_own_.p, (void*)dkeys_.p,
                    (void*)dglitch_.p, (void*)ddone_.p, (void*)dgmp_.p, (void*)dflags_.p, (void*)dZf_.p, (void*)dZq_.p, (void*)dZsmall_.p, (void*)dbla32_.p, (void*)dblamax_.p,
                    (void*)drerun_keys_.p, (void*)drerun_flag_.p, (void*)dflag_sums_.p, (void*)drerun_done_.p, (void*)drerun_gmp_.p, (void*)drerun2_keys_.p, (void*)dbladf_.p, (void*)dZdf_.p,
                    (void*)dcost_.p, (void*)dblac_.p, (void*)dpgrid_.p, (void*)ddpxy_.p, (void*)ddpxyf_.p})
        if (p) cudaFree(p);
    if (dctr_) cudaFree(dctr_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (evm_) cudaEventDestroy(evm_);
    if (hctr_) cudaFreeHost(hctr_);
    if (hcancel_) cudaFreeHost((void*)hcancel_);
    if (st_) cudaStreamDestroy(st_);
    st_ = nullptr;
    dctr_ = nullptr;
    hctr_ = nullptr;
    hcancel_ = nullptr;
}

void Engine::cancel() {
    cancel_.store(true);
    if (hcancel_) *hcancel_ = 1;
}
void Engine::reset_cancel() {
    if (!active_.load()) {
        cancel_.store(false);
        if (hcancel_) *hcancel_ = 0;
    }
}


void Engine::set_precision(int p) { // mp.cpp:2030-2045
    if (!mpf_ready_) {
        mpf_init2(c0_re_, p); mpf_init2(c0_im_, p); mpf_init2(dx_, p); mpf_init2(dy_, p); mpf_init2(scale_, p);
        mpf_init2(ref_re_, p); mpf_init2(ref_im_, p); mpf_init2(t1_, p); mpf_init2(t2_, p);
        for (int i = 0; i < 2; ++i) { mpf_init2(zre_[i], p); mpf_init2(zim_[i], p); }
        mpf_ready_ = true;
    }
    mpf_set_prec(c0_re_, p); mpf_set_prec(c0_im_, p); mpf_set_prec(dx_, p); mpf_set_prec(dy_, p);
    mpf_set_prec(scale_, p); mpf_set_prec(ref_re_, p); mpf_set_prec(ref_im_, p);
    mpf_set_prec(t1_, p); mpf_set_prec(t2_, p);
    for (int i = 0; i < 2; ++i) { mpf_set_prec(zre_[i], p); mpf_set_prec(zim_[i], p); }
}

// ---------------------------------------------------------------------------
// Reference orbit (mp.cpp:4014-4305 createRef/calCoefficient).
bool Engine::orbit_step(int i, int pr_it, bool past) {
    const int c = i & 1, p = (i - 1) & 1;
    if (use_fixed_) {
        const FixedReal& a = fz_re_[p];
        const FixedReal& b = fz_im_[p];
        FixedReal::addsub(ft1_, a, a.sign, b, b.sign);
        FixedReal::addsub(ft2_, a, a.sign, b, -b.sign);
        struct Job {
            Engine* e;
            const FixedReal* a;
            const FixedReal* b;
        } job{this, &a, &b};
        ParMul::instance().run(
            [](void* ctx, int k) {
                Job* j = static_cast<Job*>(ctx);
                if (k == 0) FixedReal::mul(j->e->fab_, *j->a, *j->b, j->e->ftmp_.data());
                else FixedReal::mul(j->e->fre_, j->e->ft1_, j->e->ft2_, j->e->ftmp2_.data());
            },
            &job, 2);
        FixedReal::addsub(fim_, fab_, fab_.sign, fab_, fab_.sign);
        FixedReal::addsub(fz_re_[c], fre_, fre_.sign, fc_re_, fc_re_.sign);
        FixedReal::addsub(fz_im_[c], fim_, fim_.sign, fc_im_, fc_im_.sign);
        if (use_floatexp_) {
            FE fr = fz_re_[c].to_fe(), fi = fz_im_[c].to_fe();
            hZfe_[i].re = fr;
            hZfe_[i].im = fi;
            hZ_[i] = make_double2(fe_to_double(fr), fe_to_double(fi));
        } else {
            hZ_[i] = make_double2(fz_re_[c].to_double(), fz_im_[c].to_double());
        }
    } else {
        mpf_add(t1_, zre_[p], zim_[p]);
        mpf_sub(t2_, zre_[p], zim_[p]);
        MpfMulJob j = {{zim_[c], zre_[c]}, {zre_[p], t1_}, {zim_[p], t2_}};
        ParMul::instance().run(mpf_mul_job, &j, 2);
        mpf_mul_ui(zim_[c], zim_[c], 2);
        mpf_add(zre_[c], zre_[c], ref_re_);
        mpf_add(zim_[c], zim_[c], ref_im_);
        hZ_[i] = make_double2(mpf_ld(zre_[c]), mpf_ld(zim_[c]));
        if (use_floatexp_) {
            hZfe_[i].re = mpf_fe(zre_[c]);
            hZfe_[i].im = mpf_fe(zim_[c]);
        }
    }
    const double zr = hZ_[i].x, zi = hZ_[i].y;
    hzm3_[i] = (zr * zr + zi * zi) / 1000000;
    if (deriv_) {
        if (use_floatexp_) {
            FE a = dfe_r_, b = dfe_i_, xr = hZfe_[i - 1].re, xi = hZfe_[i - 1].im;
            FE re = fe_add(fe_scale2(fe_sub(fe_mul(a, xr), fe_mul(b, xi)), 1), fe_make(1.0, 0));
            FE im = fe_scale2(fe_add(fe_mul(a, xi), fe_mul(b, xr)), 1);
            dfe_r_ = re;
            dfe_i_ = im;
            hD_[i] = make_double2(fe_to_double(re), fe_to_double(im));
        } else {
            double a = hD_[i - 1].x, b = hD_[i - 1].y, xr = hZ_[i - 1].x, xi = hZ_[i - 1].y;
            hD_[i] = make_double2(2.0 * (a * xr - b * xi) + 1.0, 2.0 * (a * xi + b * xr));
        }
    }
    if (std::hypot(zr, zi) > (double)escf_ && !past) return false; // escape(_zf[i]) mp.cpp:2047-2049
    if (i <= pr_it && sa_valid_) sa_update(i);
    return true;
}

// Series-approximation coefficient update (mp.cpp:4273-4303).
void Engine::sa_update(int i) {
    const C2 zprev = c2(hZ_[i - 1].x, hZ_[i - 1].y);
    const C2 dprev = c2(hD_[i - 1].x, hD_[i - 1].y);
    C2 An[kSaTerms], Bn[kSaTerms];
    for (int j = 0; j < kSaTerms; ++j) {
        An[j] = c_mul(c_mul(c2(2, 0), zprev), sa_A_[j]);
        for (int k = 0; k < j / 2; ++k) An[j] = c_add(An[j], c_mul(c_mul(c2(2, 0), sa_A_[k]), sa_A_[j - k - 1]));
        if (j % 2) An[j] = c_add(An[j], c_mul(sa_A_[j / 2], sa_A_[j / 2]));
    }
    if (deriv_) {
        for (int j = 0; j < kSaTerms; ++j) {
            Bn[j] = c_add(c_mul(sa_B_[j], zprev), c_mul(sa_A_[j], dprev));
            for (int k = 0; k < j; ++k) Bn[j] = c_add(Bn[j], c_mul(sa_A_[k], sa_B_[j - k - 1]));
            Bn[j] = c_mul(Bn[j], c2(2, 0));
        }
    }
    An[0] = c_add(An[0], sa_delta_);
    // SACheckMagnitude (mp.cpp:4307-4332): 80-bit gap between a prefix and the tail.
    int pre_mn[kSaTerms], suf_mx[kSaTerms];
    pre_mn[0] = std::min(exp_floor_log2(An[0].re), exp_floor_log2(An[0].im));
    suf_mx[kSaTerms - 1] = std::max(exp_floor_log2(An[kSaTerms - 1].re), exp_floor_log2(An[kSaTerms - 1].im));
    for (int q = 1; q < kSaTerms; ++q) pre_mn[q] = std::max(pre_mn[q - 1], std::min(exp_floor_log2(An[q].re), exp_floor_log2(An[q].im)));
    for (int q = kSaTerms - 2; q >= 0; --q) suf_mx[q] = std::max(suf_mx[q + 1], std::max(exp_floor_log2(An[q].re), exp_floor_log2(An[q].im)));
    int order = -1;
    for (int q = 0; q < kSaTerms - 10; ++q)
        if (pre_mn[q] - suf_mx[q + 1] >= 80) {
            order = std::max(q, 5);
            break;
        }
    if (order < 0) {
        sa_valid_ = false;
        return;
    }
    sa_it_ = i;
    sa_order_ = order;
    for (int j = 0; j < kSaTerms; ++j) sa_A_[j] = An[j];
    if (cm_ & 2)
        for (int j = 0; j < kSaTerms; ++j) sa_B_[j] = Bn[j];
}

void Engine::reset_series() {
    mpf_mul_ui(t1_, dx_, W_);
    mpf_div_ui(t1_, t1_, 2);
    mpf_mul_ui(t2_, dy_, H_);
    mpf_div_ui(t2_, t2_, 2);
    sa_delta_ = c2(mpf_ld(t1_), mpf_ld(t2_));
    for (int i = 0; i < kSaTerms; ++i) sa_A_[i] = sa_B_[i] = c2(0, 0);
    sa_A_[0] = sa_delta_;
}

// Arbitrary-precision per-sample iteration (mp.cpp:719-894), used for the
// reference pixel's own value and the rare floatexp cutoff-sensitive samples.
float Engine::gmp_point(mpf_srcptr c_re, mpf_srcptr c_im, int mxit, int* nout) const {
    if (nout) *nout = -1;
    const mp_bitcnt_t wp = mpf_get_prec(c_re);
    MpfTemp a1(wp), a2(wp), z_re(wp), z_im(wp), d_re(wp), d_im(wp), dc_re(wp), dc_im(wp), e1(wp), e2(wp);
    mpf_set(z_re, c_re);
    mpf_set(z_im, c_im);
    mpf_set_str(d_re, "2", 10);
    const bool ede = (cm_ & 2) != 0;
    // orbit colourings on the arbitrary-precision orbit (mp.cpp:763-770, 819-820)
    const bool sac = (cm_ & 8) != 0, trap = (cm_ & 32) != 0;
    StripeAvg sacc;
    OrbitTrap trapc;
    if (sac) sacc.init();
    if (trap) trapc.init();
    mpf_set_ui(dc_re, 1);
    float res = -2;
    for (int i = 1; i < mxit; ++i) {
        mpf_mul(a1, d_re, z_im);
        mpf_mul(d_re, d_re, z_re);
        mpf_mul(a2, d_im, z_im);
        mpf_mul(d_im, d_im, z_re);
        mpf_sub(d_re, d_re, a2);
        mpf_mul_ui(d_re, d_re, 2);
        mpf_add(d_im, d_im, a1);
        mpf_mul_ui(d_im, d_im, 2);
        if (ede) {
            mpf_mul(e1, dc_re, z_im);
            mpf_mul(e2, dc_im, z_re);
            mpf_add(e2, e1, e2);
            mpf_mul(e1, dc_re, z_re);
            mpf_mul(a2, dc_im, z_im);
            mpf_sub(e1, e1, a2);
            mpf_mul_ui(dc_re, e1, 2);
            mpf_add_ui(dc_re, dc_re, 1);
            mpf_mul_ui(dc_im, e2, 2);
        }
        mpf_mul(a1, z_re, z_im);
        mpf_mul(z_re, z_re, z_re);
        mpf_mul(z_im, z_im, z_im);
        mpf_sub(z_re, z_re, z_im);
        mpf_add(z_re, z_re, c_re);
        mpf_mul_ui(z_im, a1, 2);
        mpf_add(z_im, z_im, c_im);
        if (sac) sacc.push(mpf_get_d(z_re), mpf_get_d(z_im));
        if (trap) trapc.push(mpf_get_d(z_re), mpf_get_d(z_im));
        mpf_mul(a1, z_re, z_re);
        mpf_mul(a2, z_im, z_im);
        mpf_add(a1, a1, a2);
        double rad = mpf_get_d(a1);
        if (rad > ESC2_) {
            if (nout) *nout = i + 1;
            if (ede) {
                mpf_mul(e1, dc_re, dc_re);
                mpf_mul(e2, dc_im, dc_im);
                mpf_add(e1, e1, e2);
                mpf_sqrt(e1, e1);
                mpf_abs(a1, dx_);
                mpf_mul(e1, e1, a1);
                double num = std::isfinite(rad) && rad > 0.0 ? std::sqrt(rad) * std::log(rad) : 0.0;
                mpf_set_d(e2, num);
                if (mpf_sgn(e1) != 0) {
                    mpf_div(e1, e2, e1);
                    res = (float)mpf_get_d(e1);
                } else
                    res = 0.f;
            } else if (sac) { // here the stripe average takes precedence (mp.cpp:851-863)
                res = sacc.value(rad, (double)escf_);
            } else if (trap) {
                res = trapc.value((double)i + 1 - std::log(std::log(rad) / 2 / std::log(2)) / std::log(2));
            } else {
                res = (float)(i + 1 - std::log(std::log(rad) / 2 / std::log(2)) / std::log(2));
            }
            break;
        }
        mpf_mul(a1, d_re, d_re);
        mpf_mul(a2, d_im, d_im);
        mpf_add(a1, a1, a2);
        if (mpf_get_d(a1) < 0.000000001) break;
        if ((i & 255) == 0 && cancel_.load()) return kEmpty;
    }
    if (trap && res == -2.0f) res = trapc.value(0.0); // mp.cpp:882
    return res;
}

float Engine::gmp_sample(const int* a, int mxit, int* nout) const { // mp.cpp:896-919
    const mp_bitcnt_t pr = mpf_get_prec(c0_re_);
    MpfTemp cre(pr), cim(pr), off(pr), soff(pr);
    mpf_set(cre, c0_re_);
    mpf_set(cim, c0_im_);
    mpf_mul_ui(off, dx_, a[1]);
    mpf_add(cre, cre, off);
    mpf_mul_ui(off, dx_, std::abs(a[3]));
    mpf_set(soff, off);
    if (a[3] < 0) mpf_neg(soff, soff);
    mpf_div_ui(soff, soff, SUB_);
    mpf_add(cre, cre, soff);
    mpf_mul_ui(off, dy_, a[0]);
    mpf_add(cim, cim, off);
    mpf_mul_ui(off, dy_, std::abs(a[2]));
    mpf_set(soff, off);
    if (a[2] < 0) mpf_neg(soff, soff);
    mpf_div_ui(soff, soff, SUB_);
    mpf_add(cim, cim, soff);
    return gmp_point(cre, cim, mxit, nout);
}

bool Engine::ref_tail_escapes(int last, int extra) { // mp.cpp:927-957
    const mp_bitcnt_t pr = mpf_get_prec(c0_re_);
    MpfTemp zr(pr), zi(pr), a1(pr), a2(pr);
    if (use_fixed_) {
        fz_re_[last & 1].to_mpf(zr);
        fz_im_[last & 1].to_mpf(zi);
    } else {
        mpf_set(zr, zre_[last & 1]);
        mpf_set(zi, zim_[last & 1]);
    }
    for (int k = 0; k < extra; ++k) {
        mpf_mul(a1, zr, zi);
        mpf_mul(zr, zr, zr);
        mpf_mul(a2, zi, zi);
        mpf_sub(zr, zr, a2);
        mpf_add(zr, zr, ref_re_);
        mpf_mul_ui(zi, a1, 2);
        mpf_add(zi, zi, ref_im_);
        mpf_mul(a1, zr, zr);
        mpf_mul(a2, zi, zi);
        mpf_add(a1, a1, a2);
        if (mpf_get_d(a1) > ESC2_) return true;
    }
    return false;
}

// createRef (mp.cpp:4014-4187). `pick` < 0: view centre; otherwise the
// reference pixel key (already chosen and removed from the pending set).
int Engine::build_reference(const int* pick, bool view_center) {
    zoom_valid_ = false; // the orbit shadows are overwritten
    ref_period_ = 0;
    ref_escaped_ = false;
    ref_escape_it_ = 0;
    ++stats_.references;
    const double t0 = now_ms();
    int p[4] = {H_ / 2, W_ / 2, 0, 0};
    if (view_center) {
        ref_virtual_ = true;
        fe_cutoff_sensitive_ = false;
        ref_x_ = (W_ - 1) * 0.5;
        ref_y_ = (H_ - 1) * 0.5;
        mpf_set(ref_re_, c0_re_);
        mpf_mul_ui(t1_, dx_, W_ - 1);
        mpf_div_ui(t1_, t1_, 2);
        mpf_add(ref_re_, ref_re_, t1_);
        mpf_set(ref_im_, c0_im_);
        mpf_mul_ui(t1_, dy_, H_ - 1);
        mpf_div_ui(t1_, t1_, 2);
        mpf_add(ref_im_, ref_im_, t1_);
    } else {
        ref_virtual_ = false;
        memcpy(p, pick, sizeof(p));
        ref_x_ = p[1] + (double)p[3] / SUB_;
        ref_y_ = p[0] + (double)p[2] / SUB_;
        mpf_set(ref_re_, c0_re_);
        mpf_set(ref_im_, c0_im_);
        mpf_mul_ui(t1_, dx_, p[1]);
        mpf_add(ref_re_, ref_re_, t1_);
        mpf_mul_ui(t1_, dx_, std::abs(p[3]));
        if (p[3] < 0) mpf_neg(t1_, t1_);
        mpf_div_ui(t1_, t1_, SUB_);
        mpf_add(ref_re_, ref_re_, t1_);
        mpf_mul_ui(t1_, dy_, p[0]);
        mpf_add(ref_im_, ref_im_, t1_);
        mpf_mul_ui(t1_, dy_, std::abs(p[2]));
        if (p[2] < 0) mpf_neg(t1_, t1_);
        mpf_div_ui(t1_, t1_, SUB_);
        mpf_add(ref_im_, ref_im_, t1_);
    }
    memcpy(ref_, p, sizeof(p));
    mpf_set(zre_[0], ref_re_);
    mpf_set(zim_[0], ref_im_);
    use_fixed_ = use_floatexp_; // BigFixed auto-enabled on the floatexp path (mp.cpp:4084-4094)
    if (use_fixed_) {
        int prec = (int)mpf_get_prec(ref_re_);
        fixL_ = (prec + 63) / 64 + 2;
        ftmp_.assign((size_t)2 * fixL_ + 8, 0ull);
        ftmp2_.assign((size_t)2 * fixL_ + 8, 0ull);
        fc_re_.from_mpf(ref_re_, fixL_);
        fc_im_.from_mpf(ref_im_, fixL_);
        fz_re_[0] = fc_re_;
        fz_im_[0] = fc_im_;
        ft1_.set_len(fixL_); ft2_.set_len(fixL_); fab_.set_len(fixL_); fre_.set_len(fixL_); fim_.set_len(fixL_);
        fz_re_[1].set_len(fixL_); fz_im_[1].set_len(fixL_);
    }
    hZ_[0] = make_double2(mpf_ld(ref_re_), mpf_ld(ref_im_));
    if (use_floatexp_) {
        hZfe_[0].re = mpf_fe(ref_re_);
        hZfe_[0].im = mpf_fe(ref_im_);
    }
    hD_[0] = make_double2(1.0, 0.0);
    dfe_r_ = fe_make(1.0, 0);
    dfe_i_ = fe_make(0.0, 0);
    reset_series();
    sa_valid_ = true;
    sa_it_ = 0;
    int result = MXIT_;
    bool escaped = false;
    ParSession par(mpf_get_prec(ref_re_) >= kParBits2);
    for (int i = 1; i <= MXIT_; ++i) {
        if (cancel_.load()) break;
        if (!orbit_step(i, MXIT_, false)) {
            ref_escaped_ = true;
            ref_escape_it_ = i;
            if (ref_virtual_ && use_floatexp_ && i >= MXIT_ - 16) fe_cutoff_sensitive_ = true;
            if (!ref_virtual_) {
                if (cm_) {
                    ref_value_ = gmp_point(ref_re_, ref_im_, MXIT_, &ref_n_);
                } else {
                    if (use_fixed_) {
                        fz_re_[i & 1].to_mpf(zre_[i & 1]);
                        fz_im_[i & 1].to_mpf(zim_[i & 1]);
                    }
                    mpf_mul(t1_, zre_[i & 1], zre_[i & 1]);
                    mpf_mul(t2_, zim_[i & 1], zim_[i & 1]);
                    mpf_add(t1_, t1_, t2_);
                    double rad = mpf_get_d(t1_);
                    ref_value_ = (float)(i + 1 - std::log(std::log(rad) / 2 / std::log(2)) / std::log(2));
                    ref_n_ = i + 1;
                }
                ref_value_pending_ = true;
            }
            result = i;
            escaped = true;
            break;
        }
    }
    if (!escaped) {
        if (ref_virtual_ && use_floatexp_) fe_cutoff_sensitive_ = gmp_point(ref_re_, ref_im_, MXIT_ + 64, nullptr) >= 0;
        if (!ref_virtual_) {
            // an orbit trap colours interior samples too: the reference pixel's
            // value from its arbitrary-precision orbit (mp.cpp:4179-4184)
            ref_value_ = (cm_ & 32) ? gmp_point(ref_re_, ref_im_, MXIT_, nullptr) : -2.0f;
            ref_n_ = -1;
            ref_value_pending_ = true;
        }
    }
    stats_.orbit_ms += now_ms() - t0;
    return result;
}

// Ball-arithmetic period and Newton nucleus (mp.cpp:96-223, 1072-1107).
static void sqadd(mpf_ptr zr, mpf_ptr zi, mpf_srcptr cr, mpf_srcptr ci, mpf_ptr s1, mpf_ptr s2, mpf_ptr s3) {
    mpf_add(s1, zr, zi);
    mpf_sub(s2, zr, zi);
    mpf_mul(s3, zr, zi);
    mpf_mul(zr, s1, s2);
    mpf_add(zr, zr, cr);
    mpf_mul_ui(zi, s3, 2);
    mpf_add(zi, zi, ci);
}

// ---------------------------------------------------------------------------
// Pipelined forms of the period search and the Newton orbit for precisions
// where one product takes a fraction of a microsecond (below kParBits6 /
// kParBits4): a parallel round's synchronisation would cost as much as the
// products it overlaps. Instead the loop's independent recurrences run on
// their own threads, linked by ring buffers and progress counters: the orbit
// z -> z^2 + c runs ahead while the derivative (Newton) or the disk radius and
// the containment test (period search) follow it. Every value is produced by
// the same GMP calls, in the same order, into variables of the same precision
// as in the serial loop, so the results are bit for bit the same.
namespace {

constexpr int kRing = 64; // iterates kept between the leading and trailing threads
// Below this a product takes under ~0.2 us and the threads' hand-offs (a
// ~0.28 us round trip between Neoverse V2 cores) cost what the overlap gains;
// measured there: a 1063-bit Newton step 1.31 -> 0.87 us, 1500-bit 2.20 -> 1.06 us,
// 700-bit no gain.
constexpr mp_bitcnt_t kPipeMinBits = 1000;

struct alignas(64) Progress {
    std::atomic<long> v{0};
};
inline void wait_at_least(const Progress& p, long v, const std::atomic<bool>* stop = nullptr) {
    while (p.v.load(std::memory_order_acquire) < v)
        if (stop && stop->load(std::memory_order_relaxed)) return;
}

// Iterates written by one thread and read by others: each variable (its header
// and, through a spacer allocation after it, its limbs) on cache lines of its
// own, so that a writer never invalidates a line another thread is reading.
struct MpfRing {
    struct alignas(64) Slot {
        __mpf_struct v;
    };
    std::vector<Slot> v;
    std::vector<void*> spacers;
    MpfRing(int n, mp_bitcnt_t prec) : v((size_t)n) {
        for (auto& x : v) {
            mpf_init2(&x.v, prec);
            spacers.push_back(malloc(128));
        }
    }
    ~MpfRing() {
        for (auto& x : v) mpf_clear(&x.v);
        for (void* q : spacers) free(q);
    }
    mpf_ptr operator[](long i) { return &v[(size_t)(i % (long)v.size())].v; }
};

// One Newton orbit z_{i+1} = z_i^2 + c, d_{i+1} = 2 z_i d_i + 1 from z_0 = d_0 = 0
// over `period` steps, on three threads: 0 the orbit, 1 Re d, 2 Im d.
struct NewtonPipe {
    mpf_srcptr cr, ci;
    long period;
    mp_bitcnt_t prec;
    MpfRing zr, zi, dr, di; // dr/di: two buffers (step parity)
    Progress z_done, re_done, im_done; // z_0..z_{z_done-1}; d_1..d_{*_done}
    NewtonPipe(mpf_srcptr c_re, mpf_srcptr c_im, long p, mp_bitcnt_t pr)
        : cr(c_re), ci(c_im), period(p), prec(pr), zr(kRing, pr), zi(kRing, pr), dr(2, pr), di(2, pr) {}

    void orbit() {
        MpfTemp t1(prec), t2(prec), e6(prec), f7(prec);
        for (long i = 0; i < period; ++i) {
            // slot i+1 last held z_{i+1-kRing}, read at that step by both followers
            wait_at_least(re_done, i + 2 - kRing);
            wait_at_least(im_done, i + 2 - kRing);
            mpf_srcptr a = zr[i], b = zi[i];
            mpf_add(t1, a, b);
            mpf_sub(t2, a, b);
            mpf_mul(e6, a, b);
            mpf_mul(f7, t1, t2);
            mpf_add(zr[i + 1], f7, cr);
            mpf_mul_ui(zi[i + 1], e6, 2);
            mpf_add(zi[i + 1], zi[i + 1], ci);
            z_done.v.store(i + 2, std::memory_order_release);
        }
    }
    // Re d_{i+1} = 2 (zr dr - zi di) + 1
    void real_part() {
        MpfTemp s1(prec), s2(prec);
        for (long i = 0; i < period; ++i) {
            wait_at_least(z_done, i + 1);
            wait_at_least(im_done, i); // Im d_i, and Im's read of Re d_{i-1} is done
            mpf_mul(s1, zr[i], dr[i]);
            mpf_mul(s2, zi[i], di[i]);
            mpf_ptr out = dr[i + 1];
            mpf_sub(out, s1, s2);
            mpf_mul_ui(out, out, 2);
            mpf_add_ui(out, out, 1);
            re_done.v.store(i + 1, std::memory_order_release);
        }
    }
    // Im d_{i+1} = 2 (zr di + zi dr)
    void imag_part() {
        MpfTemp c4(prec), c5(prec);
        for (long i = 0; i < period; ++i) {
            wait_at_least(z_done, i + 1);
            wait_at_least(re_done, i);
            mpf_mul(c4, zr[i], di[i]);
            mpf_mul(c5, zi[i], dr[i]);
            mpf_ptr out = di[i + 1];
            mpf_add(out, c4, c5);
            mpf_mul_ui(out, out, 2);
            im_done.v.store(i + 1, std::memory_order_release);
        }
    }
    static void run_part(void* ctx, int k) {
        NewtonPipe* p = static_cast<NewtonPipe*>(ctx);
        if (k == 0) p->orbit();
        else if (k == 1) p->real_part();
        else p->imag_part();
    }
    // z_p, d_p into the caller's variables after a full run
    void run(mpf_ptr out_zr, mpf_ptr out_zi, mpf_ptr out_dr, mpf_ptr out_di) {
        mpf_set_ui(zr[0], 0);
        mpf_set_ui(zi[0], 0);
        mpf_set_ui(dr[0], 0);
        mpf_set_ui(di[0], 0);
        z_done.v.store(1);
        re_done.v.store(0);
        im_done.v.store(0);
        ParMul::instance().run(&NewtonPipe::run_part, this, 3);
        mpf_set(out_zr, zr[period]);
        mpf_set(out_zi, zi[period]);
        mpf_set(out_dr, dr[period]);
        mpf_set(out_di, di[period]);
    }
};

// The period search on three threads: 0 the orbit (and |z| as a double), 1 the
// disk radius R, 2 the containment test |z|^2 <= R^2 and the escape test.
struct BallPipe {
    mpf_srcptr cr, ci, r;
    int maxp;
    mp_bitcnt_t prec;
    double cab;
    const std::atomic<bool>* cancel;
    MpfRing zr, zi, R, ru_ring;
    std::vector<double> za; // |z_p| ring
    std::vector<double> Rd; // R_p as a double
    Progress z_done, r_done, q_done; // steps whose z_p / R_p / test are complete
    std::atomic<bool> stop{false};
    int result = 0;
    BallPipe(mpf_srcptr c_re, mpf_srcptr c_im, mpf_srcptr rad, int mp, mp_bitcnt_t pr, const std::atomic<bool>* c)
        : cr(c_re), ci(c_im), r(rad), maxp(mp), prec(pr), cancel(c), zr(kRing, pr), zi(kRing, pr), R(kRing, pr), ru_ring(1, pr),
          za(kRing), Rd(kRing) {}

    void orbit() {
        MpfTemp s1(prec), s2(prec), s3(prec), F(prec);
        for (long p = 1; p <= maxp; ++p) {
            // slot p last held step p - kRing, read by the radius thread at step
            // p - kRing + 1 (its |z|) and by the test at step p - kRing
            wait_at_least(q_done, p - kRing, &stop);
            wait_at_least(r_done, p - kRing + 1, &stop);
            // past escape |z| squares each step: run ahead only while it is
            // moderate, else take step p only once the serial loop would (the
            // test passed step p - 1)
            if (!(za[(size_t)((p - 1) % kRing)] < 1e300)) wait_at_least(q_done, p - 1, &stop);
            if (stop.load(std::memory_order_relaxed)) return;
            mpf_srcptr a = zr[p - 1], b = zi[p - 1];
            mpf_add(s1, a, b);
            mpf_sub(s2, a, b);
            mpf_mul(s3, a, b);
            mpf_mul(F, s1, s2);
            mpf_add(zr[p], F, cr);
            mpf_mul_ui(zi[p], s3, 2);
            mpf_add(zi[p], zi[p], ci);
            za[(size_t)(p % kRing)] = std::hypot(mpf_get_d(zr[p]), mpf_get_d(zi[p]));
            z_done.v.store(p, std::memory_order_release);
        }
    }
    void radius() {
        MpfTemp t(prec), nb(prec), tq(prec);
        mpf_srcptr ru = ru_ring[0];
        for (long p = 1; p <= maxp; ++p) {
            wait_at_least(z_done, p - 1, &stop);     // |z_{p-1}|
            wait_at_least(q_done, p - kRing, &stop); // slot p of R free
            if (stop.load(std::memory_order_relaxed)) return;
            const double a = za[(size_t)((p - 1) % kRing)];
            // a huge |z| (whose square or double would not convert to GMP)
            // is only used when the serial loop reaches this step
            if (!(a < 1e150)) {
                wait_at_least(q_done, p - 1, &stop);
                if (stop.load(std::memory_order_relaxed)) return;
            }
            mpf_set_d(t, 2.0 * a);
            mpf_add(nb, t, R[p - 1]);
            mpf_set_d(tq, a * a + cab + 1.0);
            mpf_mul(nb, nb, R[p - 1]);
            mpf_mul(tq, tq, ru);
            mpf_add(nb, nb, r);
            mpf_add(nb, nb, tq);
            mpf_set(R[p], nb);
            Rd[(size_t)(p % kRing)] = mpf_get_d(R[p]);
            r_done.v.store(p, std::memory_order_release);
        }
    }
    void test() {
        MpfTemp s1(prec), s2(prec), R2m(prec), zabs2(prec);
        for (long p = 1; p <= maxp; ++p) {
            if (cancel && (p & 1023) == 0 && cancel->load()) break;
            wait_at_least(z_done, p);
            wait_at_least(r_done, p);
            mpf_mul(s1, zr[p], zr[p]);
            mpf_mul(s2, zi[p], zi[p]);
            mpf_mul(R2m, R[p], R[p]);
            mpf_add(zabs2, s1, s2);
            if (mpf_cmp(zabs2, R2m) <= 0) {
                result = (int)p;
                break;
            }
            if (za[(size_t)(p % kRing)] > cab + 2.0 + Rd[(size_t)(p % kRing)]) break;
            q_done.v.store(p, std::memory_order_release);
        }
        stop.store(true, std::memory_order_relaxed);
    }
    static void run_part(void* ctx, int k) {
        BallPipe* b = static_cast<BallPipe*>(ctx);
        if (k == 0) b->orbit();
        else if (k == 1) b->radius();
        else b->test();
    }
    int run() {
        mpf_set_ui(zr[0], 0);
        mpf_set_ui(zi[0], 0);
        mpf_set_ui(R[0], 0);
        cab = std::hypot(mpf_get_d(cr), mpf_get_d(ci));
        mpf_ptr ru = ru_ring[0];
        mpf_set_ui(ru, 1);
        mpf_div_2exp(ru, ru, prec > 64 ? prec - 32 : prec / 2);
        za[0] = 0.0;
        ParMul::instance().run(&BallPipe::run_part, this, 3);
        return result;
    }
};

} // namespace

int ball_period(mpf_srcptr cr, mpf_srcptr ci, mpf_srcptr r, int maxp, mp_bitcnt_t prec, const std::atomic<bool>* cancel) {
    if (prec >= kPipeMinBits && prec < kParBits4 && maxp >= 64) {
        ParSession par(true);
        if (ParMul::instance().concurrent(3)) {
            BallPipe b(cr, ci, r, maxp, prec, cancel);
            return b.run();
        }
    }
    MpfTemp s1(prec), s2(prec), s3(prec), zr(prec), zi(prec), R(prec), R2m(prec), zabs2(prec), nb(prec), ru(prec), t(prec), tq(prec), F(prec);
    MpfTemp q1(prec), q2(prec);
    ParSession par(prec >= kParBits4);
    mpf_set_ui(zr, 0);
    mpf_set_ui(zi, 0);
    mpf_set_ui(R, 0);
    const double cab = std::hypot(mpf_get_d(cr), mpf_get_d(ci));
    mpf_set_ui(ru, 1);
    mpf_div_2exp(ru, ru, prec > 64 ? prec - 32 : prec / 2);
    if (prec >= kParBits4 && ParMul::instance().concurrent(7)) {
        // One round of seven products per step: step p's four with the three
        // of step p - 1's containment test (|z_{p-1}|^2 and R_{p-1}^2, values
        // already known), whose verdict is taken before step p's values are
        // used. Step p's products are then only wasted work when step p - 1
        // ends the search, except when |z_{p-1}| is too large for the
        // conversions of step p: that step takes the test on its own first.
        auto test = [&](int p) -> int { // verdict of step p from q1, q2, R2m: p (period), -1 (escaped), 0 (go on)
            mpf_add(zabs2, q1, q2);
            if (mpf_cmp(zabs2, R2m) <= 0) return p;
            const double zb = std::hypot(mpf_get_d(zr), mpf_get_d(zi));
            return zb > cab + 2.0 + mpf_get_d(R) ? -1 : 0;
        };
        for (int p = 1; p <= maxp; ++p) {
            if (cancel && (p & 1023) == 0 && cancel->load()) return 0;
            const double za = std::hypot(mpf_get_d(zr), mpf_get_d(zi));
            const bool pending = p > 1;
            bool tested = !pending;
            if (pending && !(za < 1e150)) {
                MpfMulJob j = {{q1, q2, R2m}, {zr, zi, R}, {zr, zi, R}};
                ParMul::instance().run(mpf_mul_job, &j, 3);
                const int v = test(p - 1);
                if (v > 0) return v;
                if (v < 0) return 0;
                tested = true;
            }
            mpf_set_d(t, 2.0 * za);
            mpf_add(nb, t, R);
            mpf_set_d(tq, za * za + cab + 1.0);
            mpf_add(s1, zr, zi);
            mpf_sub(s2, zr, zi);
            if (tested) {
                MpfMulJob j = {{nb, tq, s3, F}, {nb, tq, zr, s1}, {R, ru, zi, s2}};
                ParMul::instance().run(mpf_mul_job, &j, 4);
            } else {
                MpfMulJob j = {{nb, tq, s3, F, q1, q2, R2m}, {nb, tq, zr, s1, zr, zi, R}, {R, ru, zi, s2, zr, zi, R}};
                ParMul::instance().run(mpf_mul_job, &j, 7);
                const int v = test(p - 1);
                if (v > 0) return v;
                if (v < 0) return 0;
            }
            mpf_add(nb, nb, r);
            mpf_add(nb, nb, tq);
            mpf_set(R, nb);
            mpf_add(zr, F, cr);
            mpf_mul_ui(zi, s3, 2);
            mpf_add(zi, zi, ci);
        }
        MpfMulJob j = {{q1, q2, R2m}, {zr, zi, R}, {zr, zi, R}};
        ParMul::instance().run(mpf_mul_job, &j, 3);
        const int v = test(maxp);
        return v > 0 ? v : 0;
    }
    for (int p = 1; p <= maxp; ++p) {
        if (cancel && (p & 1023) == 0 && cancel->load()) return 0;
        // the serial step's products in two rounds of independent ones:
        // nb = (2|z| + R) R + r + (|z|^2 + |c| + 1) ru, then z <- z^2 + c, then
        // |z|^2 and R^2
        double za = std::hypot(mpf_get_d(zr), mpf_get_d(zi));
        mpf_set_d(t, 2.0 * za);
        mpf_add(nb, t, R);
        mpf_set_d(tq, za * za + cab + 1.0);
        mpf_add(s1, zr, zi);
        mpf_sub(s2, zr, zi);
        {
            MpfMulJob j = {{nb, tq, s3, F}, {nb, tq, zr, s1}, {R, ru, zi, s2}};
            ParMul::instance().run(mpf_mul_job, &j, 4);
        }
        mpf_add(nb, nb, r);
        mpf_add(nb, nb, tq);
        mpf_set(R, nb);
        mpf_add(zr, F, cr);
        mpf_mul_ui(zi, s3, 2);
        mpf_add(zi, zi, ci);
        {
            MpfMulJob j = {{s1, s2, R2m}, {zr, zi, R}, {zr, zi, R}};
            ParMul::instance().run(mpf_mul_job, &j, 3);
        }
        mpf_add(zabs2, s1, s2);
        if (mpf_cmp(zabs2, R2m) <= 0) return p;
        double zb = std::hypot(mpf_get_d(zr), mpf_get_d(zi));
        if (zb > cab + 2.0 + mpf_get_d(R)) break;
    }
    return 0;
}

bool newton_nucleus(mpf_ptr cr, mpf_ptr ci, int period, mp_bitcnt_t prec, int maxit) {
    MpfTemp s1(prec), s2(prec), s3(prec), zr(prec), zi(prec), dr(prec), di(prec), den(prec), nr(prec), ni(prec), tol(prec), step2(prec);
    MpfTemp c4(prec), c5(prec), e6(prec), f7(prec), t1(prec), t2(prec);
    const bool piped = prec >= kPipeMinBits && prec < kParBits6 && period >= 64;
    ParSession par(prec >= kParBits6 || piped);
    std::unique_ptr<NewtonPipe> pipe;
    if (piped && ParMul::instance().concurrent(3)) pipe.reset(new NewtonPipe(cr, ci, period, prec));
    mpf_set_ui(tol, 1);
    mpf_div_2exp(tol, tol, prec > 96 ? prec - 48 : prec / 2);
    mpf_mul(tol, tol, tol);
    for (int it = 0; it < maxit; ++it) {
        mpf_set_ui(zr, 0);
        mpf_set_ui(zi, 0);
        mpf_set_ui(dr, 0);
        mpf_set_ui(di, 0);
        if (pipe) pipe->run(zr, zi, dr, di);
        else for (int i = 0; i < period; ++i) {
            // dz' = 2 z dz + 1 and z' = z^2 + c: six products of the old
            // iterate, one round
            mpf_add(t1, zr, zi);
            mpf_sub(t2, zr, zi);
            MpfMulJob j = {{s1, s2, c4, c5, e6, f7}, {zr, zi, zr, zi, zr, t1}, {dr, di, di, dr, zi, t2}};
            ParMul::instance().run(mpf_mul_job, &j, 6);
            mpf_sub(s3, s1, s2);
            mpf_mul_ui(s3, s3, 2);
            mpf_add_ui(s3, s3, 1);
            mpf_add(di, c4, c5);
            mpf_mul_ui(di, di, 2);
            mpf_set(dr, s3);
            mpf_add(zr, f7, cr);
            mpf_mul_ui(zi, e6, 2);
            mpf_add(zi, zi, ci);
        }
        mpf_mul(s1, dr, dr);
        mpf_mul(s2, di, di);
        mpf_add(den, s1, s2);
        if (mpf_sgn(den) == 0) return false;
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
        if (mpf_cmp(step2, tol) <= 0) return true;
    }
    return false;
}

int Engine::find_nucleus(int maxp) { // mp.cpp:1072-1107 (writes the nucleus into ref_re_/ref_im_)
    const mp_bitcnt_t prec = mpf_get_prec(c0_re_);
    MpfTemp cre(prec), cim(prec), r(prec), dh(prec), dist(prec), dr(prec), di(prec);
    mpf_set_ui(r, 2);
    mpf_div(r, r, scale_);
    mpf_add(cre, c0_re_, r);
    mpf_mul_ui(dh, r, H_);
    mpf_div_ui(dh, dh, W_);
    mpf_add(cim, c0_im_, dh);
    int period = ball_period(cre, cim, r, maxp, prec, &cancel_);
    if (period <= 0) return 0;
    mpf_set(ref_re_, cre);
    mpf_set(ref_im_, cim);
    if (!newton_nucleus(ref_re_, ref_im_, period, prec, 200)) return 0;
    mpf_sub(dr, ref_re_, cre);
    mpf_sub(di, ref_im_, cim);
    mpf_mul(dr, dr, dr);
    mpf_mul(di, di, di);
    mpf_add(dist, dr, di);
    mpf_sqrt(dist, dist);
    return mpf_cmp(dist, r) <= 0 ? period : 0;
}

// The nucleus ref_re_/ref_im_ as the frame's virtual reference: its position in
// pixel units and the pixel it rounds to (mp.cpp:1109-1125).
void Engine::periodic_reference_geometry() {
    ref_escaped_ = false;
    ref_escape_it_ = 0;
    ref_virtual_ = true;
    mpf_sub(t1_, ref_re_, c0_re_);
    mpf_div(t1_, t1_, dx_);
    ref_x_ = mpf_get_d(t1_);
    mpf_sub(t1_, ref_im_, c0_im_);
    mpf_div(t1_, t1_, dy_);
    ref_y_ = mpf_get_d(t1_);
    int px = (int)std::lround(ref_x_), py = (int)std::lround(ref_y_);
    ref_[0] = py;
    ref_[1] = px;
    ref_[2] = 0;
    ref_[3] = 0;
    ref_frac_re_ = (ref_x_ - px) * mpf_ld(dx_);
    ref_frac_im_ = (ref_y_ - py) * mpf_ld(dy_);
}

int Engine::build_periodic_reference(int period) { // mp.cpp:1109-1172
    zoom_valid_ = false; // the orbit shadows are overwritten
    periodic_reference_geometry();
    mpf_set(zre_[0], ref_re_);
    mpf_set(zim_[0], ref_im_);
    use_fixed_ = false;
    hZ_[0] = make_double2(mpf_ld(ref_re_), mpf_ld(ref_im_));
    hZfe_[0].re = mpf_fe(ref_re_);
    hZfe_[0].im = mpf_fe(ref_im_);
    hzm3_[0] = (hZ_[0].x * hZ_[0].x + hZ_[0].y * hZ_[0].y) / 1000000;
    hD_[0] = make_double2(1.0, 0.0);
    dfe_r_ = fe_make(1.0, 0);
    dfe_i_ = fe_make(0.0, 0);
    reset_series();
    sa_valid_ = false;
    sa_it_ = 0;
    sa_order_ = 0;
    const bool save = use_floatexp_;
    use_floatexp_ = true;
    {
        ParSession par(mpf_get_prec(ref_re_) >= kParBits2);
        for (int i = 1; i < period; ++i) orbit_step(i, 0, false);
    }
    use_floatexp_ = save;
    ref_period_ = period;
    return period;
}

FE Engine::nucleus_size() const { // mp.cpp:1195-1219
    const int p = ref_period_;
    if (p < 2) return fe_make(1.0, 1000000);
    FE lr = fe_make(1.0, 0), li = fe_make(0.0, 0), br = fe_make(1.0, 0), bi = fe_make(0.0, 0);
    for (int k = 1; k < p; ++k) {
        FE zr = hZfe_[k - 1].re, zi = hZfe_[k - 1].im;
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
    if (denom.m == 0.0) return fe_make(1.0, 1000000);
    return fe_div(fe_make(1.0, 0), denom);
}

// The request's periodic reference (mbx_request.reference_period > 0; no
// reference counterpart): the given nucleus is the frame's reference whatever
// its size in the frame, on the floatexp path. Its one-period orbit is built
// once and kept (host shadows, device orbit) while the nucleus, period,
// precision and derivative need stay the same, so the frames of a zoom
// sequence toward it share it; per frame only the nucleus's position, the BLA
// table (its validity radii follow the frame's radius) and the mixed form's
// per-frame tables are redone. The lanes rebase, so one orbit serves every
// depth.
int Engine::zoom_reference(int* ref_it) {
    const int p = zoom_period_;
    if (mpf_set_str(ref_re_, zoom_re_.c_str(), 10) != 0 || mpf_set_str(ref_im_, zoom_im_.c_str(), 10) != 0) {
        err_ = "unparsable reference nucleus";
        return MBX_E_INVALID;
    }
    cache_.valid = false; // (the reuse cache and this share the orbit shadows)
    use_floatexp_ = true;
    fe_cutoff_sensitive_ = false;
    ref_subpixel_ = false;
    ref_value_pending_ = false;
    periodic_reference_geometry();
    reset_series();
    sa_valid_ = false;
    sa_it_ = 0;
    sa_order_ = 0;
    ref_period_ = p;
    char kb[96];
    snprintf(kb, sizeof(kb), "|%d|%lu|%d", p, (unsigned long)mpf_get_prec(ref_re_), deriv_ ? 1 : 0);
    const std::string key = zoom_re_ + "|" + zoom_im_ + kb;
    if (zoom_valid_ && zoom_key_ == key) {
        stats_.reused_reference = 1;
    } else {
        zoom_valid_ = false;
        const double t0 = now_ms();
        hZ_.assign((size_t)p + 2, make_double2(0, 0));
        hzm3_.assign((size_t)p + 2, 0.0);
        hD_.assign((size_t)p + 2, make_double2(0, 0));
        hZfe_.assign((size_t)p + 2, FE2{fe_make(0, 0), fe_make(0, 0)});
        mpf_set(zre_[0], ref_re_);
        mpf_set(zim_[0], ref_im_);
        use_fixed_ = false;
        hZ_[0] = make_double2(mpf_ld(ref_re_), mpf_ld(ref_im_));
        hZfe_[0].re = mpf_fe(ref_re_);
        hZfe_[0].im = mpf_fe(ref_im_);
        hzm3_[0] = (hZ_[0].x * hZ_[0].x + hZ_[0].y * hZ_[0].y) / 1000000;
        hD_[0] = make_double2(1.0, 0.0);
        dfe_r_ = fe_make(1.0, 0);
        dfe_i_ = fe_make(0.0, 0);
        {
            ParSession par(mpf_get_prec(ref_re_) >= kParBits2);
            for (int i = 1; i < p; ++i) {
                if (cancel_.load()) return MBX_E_CANCELLED;
                orbit_step(i, 0, false);
            }
        }
        stats_.orbit_ms += now_ms() - t0;
        ++stats_.references;
        const double t1 = now_ms();
        if (!ensure(dZ_, (size_t)p + 2) || !ensure(dzm3_, (size_t)p + 2) || !ensure(dZfe_, (size_t)p + 2) || (deriv_ && !ensure(dD_, (size_t)p + 2)))
            return MBX_E_NOMEM;
        copy_async(dZ_.p, hZ_.data(), sizeof(double2) * p, cudaMemcpyHostToDevice);
        copy_async(dzm3_.p, hzm3_.data(), sizeof(double) * p, cudaMemcpyHostToDevice);
        copy_async(dZfe_.p, hZfe_.data(), sizeof(FE2) * p, cudaMemcpyHostToDevice);
        if (deriv_) copy_async(dD_.p, hD_.data(), sizeof(double2) * p, cudaMemcpyHostToDevice);
        stats_.copy_ms += now_ms() - t1;
        const int rc = cuda_ok("orbit upload");
        if (rc != MBX_OK) return rc;
        zoom_valid_ = true;
        zoom_key_ = key;
    }
    stats_.reference_length = p;
    orbit_len_ = p;
    *ref_it = p;
    int rc = build_bla(p);
    if (rc != MBX_OK) return rc;
    if (mixed_active()) rc = prepare_mixed();
    return rc;
}

// buildReferenceOrbit (mp.cpp:1227-1386).
int Engine::reference_for_frame() {
    int ref_it = 0;
    ref_period_ = 0;
    ref_subpixel_ = false;
    bool periodic_done = false;
    if (mpf_cmp_d(scale_, 1e280) > 0 && use_bla_) {
        const double t0 = now_ms();
        MpfTemp save_re(mpf_get_prec(ref_re_)), save_im(mpf_get_prec(ref_im_));
        mpf_set(save_re, ref_re_);
        mpf_set(save_im, ref_im_);
        int p = find_nucleus(MXIT_);
        stats_.orbit_ms += now_ms() - t0;
        if (p > 2 && p <= MXIT_) {
            const double t1 = now_ms();
            ref_it = build_periodic_reference(p);
            stats_.orbit_ms += now_ms() - t1;
            FE size = nucleus_size();
            ref_subpixel_ = fe_abs_less(size, fe_mul_d(dxfe_, 4.0));
            if (!ref_subpixel_) {
                periodic_done = true;
                if (!use_floatexp_) {
                    double refmin2 = 1e300;
                    bool uf = false;
                    for (int q = 1; q < p; ++q) {
                        double m2 = hzm3_[q] * 1e6;
                        if (m2 <= 0.0) {
                            uf = true;
                            break;
                        }
                        if (m2 < refmin2) refmin2 = m2;
                    }
                    double dcmax = 2.0 / mpf_get_d(scale_);
                    if (uf || std::sqrt(refmin2) * dcmax < 1e-300) use_floatexp_ = true;
                }
            } else {
                mpf_set(ref_re_, save_re);
                mpf_set(ref_im_, save_im);
                ref_period_ = 0;
                ref_virtual_ = false;
            }
        }
    }
    if (!periodic_done) {
        int center[4] = {H_ / 2, W_ / 2, 0, 0};
        (void)rng_.next(); // createRef(random=true) draws once from a one-element set (mp.cpp:4039-4044)
        ref_it = build_reference(center, false);
        if (!use_floatexp_ && mpf_cmp_d(scale_, 1e150) > 0) {
            double refmin2 = 1e300;
            bool underflowed = false;
            for (int q = 1; q <= ref_it; ++q) {
                double m2 = hzm3_[q] * 1e6;
                if (m2 <= 0.0) {
                    underflowed = true;
                    break;
                }
                if (m2 < refmin2) refmin2 = m2;
            }
            double dcmax = 2.0 / mpf_get_d(scale_);
            if (underflowed || std::sqrt(refmin2) * dcmax < 1e-300) {
                use_floatexp_ = true;
                ref_value_pending_ = false;
                ref_it = build_reference(nullptr, true);
            }
        }
        if (use_floatexp_ && (!ref_escaped_ || ref_escape_it_ >= MXIT_ - 16)) {
            bool sensitive = ref_escaped_ || ref_tail_escapes(ref_it, 80);
            if (sensitive) {
                ref_value_pending_ = false;
                ref_it = build_reference(nullptr, true);
            }
        }
    }
    return ref_it;
}

// ---------------------------------------------------------------------------
// Device side of a reference: orbit upload and BLA table (mp.cpp:2613-2709).
int Engine::upload_reference(int ref_it) {
    const int len = (ref_period_ > 0) ? ref_period_ : ref_it + 1;
    orbit_len_ = len;
    const double t0 = now_ms();
    if (!ensure(dZ_, (size_t)MXIT_ + 2) || !ensure(dzm3_, (size_t)MXIT_ + 2)) return MBX_E_NOMEM;
    copy_async(dZ_.p, hZ_.data(), sizeof(double2) * len, cudaMemcpyHostToDevice);
    copy_async(dzm3_.p, hzm3_.data(), sizeof(double) * (MXIT_ + 1), cudaMemcpyHostToDevice);
    if (use_floatexp_) {
        if (!ensure(dZfe_, (size_t)MXIT_ + 2)) return MBX_E_NOMEM;
        copy_async(dZfe_.p, hZfe_.data(), sizeof(FE2) * len, cudaMemcpyHostToDevice);
    }
    if (deriv_) {
        if (!ensure(dD_, (size_t)MXIT_ + 2)) return MBX_E_NOMEM;
        copy_async(dD_.p, hD_.data(), sizeof(double2) * len, cudaMemcpyHostToDevice);
    }
    stats_.copy_ms += now_ms() - t0;
    return cuda_ok("orbit upload");
}

int Engine::build_bla(int reflen) {
    bla_ = BlaView();
    bla_.minlevel = bla_minlevel_;
    bla_.use = 0;
    if (reflen < 3) return MBX_OK;
    const double t0 = now_ms();
    const double eps = std::ldexp(1.0, -53);
    double dxf = std::fabs(mpf_ld(dx_)), dyf = std::fabs(mpf_ld(dy_));
    double mxx = std::max(ref_x_, (double)(W_ - 1) - ref_x_) + 0.5;
    double mxy = std::max(ref_y_, (double)(H_ - 1) - ref_y_) + 0.5;
    double dcmax = std::sqrt(dxf * dxf * mxx * mxx + dyf * dyf * mxy * mxy);
    int off = 0, n = reflen - 1, lev = 0;
    while (n >= 1 && lev < kMaxLevels) {
        bla_.off[lev] = off;
        bla_.size[lev] = n;
        off += n;
        ++lev;
        if (n == 1) break;
        n = n / 2;
    }
    bla_.nlev = lev;
    if (!ensure(dr2_, off) || !ensure(dab_, off) || (deriv_ && !ensure(dce_, off))) return MBX_E_NOMEM;
    hctr_->glitch_min_bits = 0;
    cudaMemsetAsync(&dctr_->glitch_min_bits, 0, sizeof(unsigned long long), st_);
    cudaError_t e = launch_bla_build(dZ_.p, dD_.p, reflen, eps, dcmax, deriv_, dr2_.p, dab_.p, dce_.p, bla_.off, bla_.size, bla_.nlev, &dctr_->glitch_min_bits, st_);
    stats_.kernel_launches += bla_.nlev;
    if (e != cudaSuccess) return fail_cuda("bla build", e);
    unsigned long long bits = 0;
    copy_async(&bits, &dctr_->glitch_min_bits, sizeof(bits), cudaMemcpyDeviceToHost);
    e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return fail_cuda("bla build", e);
    double rmax2;
    memcpy(&rmax2, &bits, 8);
    bla_.rmax2 = rmax2;
    bla_.r2 = dr2_.p;
    bla_.ab = dab_.p;
    bla_.ce = dce_.p;
    bla_.use = 1;
    stats_.bla_ms += now_ms() - t0;
    return MBX_OK;
}

// Per-reference pixel-spacing tables for the double path: dc components are
// mpf products truncated to double (mp.cpp:2300-2312); the real part depends
// only on the column offset and the imaginary part only on the row offset.
int Engine::build_dc_tables() {
    const int xmin = SUB_ * (0 - ref_[1]) + (-(SUB_ / 2) - ref_[3]);
    const int xmax = SUB_ * (W_ - 1 - ref_[1]) + (SUB_ / 2 - ref_[3]);
    const int ymin = SUB_ * (0 - ref_[0]) + (-(SUB_ / 2) - ref_[2]);
    const int ymax = SUB_ * (H_ - 1 - ref_[0]) + (SUB_ / 2 - ref_[2]);
    const int nx = xmax - xmin + 1, ny = ymax - ymin + 1;
    hdcx_.resize(nx);
    hdcy_.resize(ny);
    MpfTemp a(mpf_get_prec(dx_));
    for (int x = xmin; x <= xmax; ++x) {
        mpf_mul_ui(a, dx_, std::abs(x));
        if (x < 0) mpf_neg(a, a);
        if (SUB_ > 1) mpf_div_ui(a, a, SUB_);
        hdcx_[x - xmin] = mpf_ld(a);
    }
    for (int y = ymin; y <= ymax; ++y) {
        mpf_mul_ui(a, dy_, std::abs(y));
        if (y < 0) mpf_neg(a, a);
        if (SUB_ > 1) mpf_div_ui(a, a, SUB_);
        hdcy_[y - ymin] = mpf_ld(a);
    }
    dc_xoff_ = -xmin;
    dc_yoff_ = -ymin;
    if (!ensure(ddcx_, nx) || !ensure(ddcy_, ny)) return MBX_E_NOMEM;
    copy_async(ddcx_.p, hdcx_.data(), sizeof(double) * nx, cudaMemcpyHostToDevice);
    copy_async(ddcy_.p, hdcy_.data(), sizeof(double) * ny, cudaMemcpyHostToDevice);
    return cuda_ok("dc tables");
}

// ---------------------------------------------------------------------------
int Engine::cuda_ok(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(what, e);
    return MBX_OK;
}
cudaError_t Engine::copy_async(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
    if (kind == cudaMemcpyHostToDevice) stats_.h2d_bytes += (long long)bytes;
    else if (kind == cudaMemcpyDeviceToHost) stats_.d2h_bytes += (long long)bytes;
    return cudaMemcpyAsync(dst, src, bytes, kind, st_);
}

int Engine::fail_cuda(const char* what, cudaError_t e) {
    err_ = std::string(what) + ": " + cudaGetErrorString(e);
    return MBX_E_CUDA;
}

DeviceFrame Engine::frame_view() {
    DeviceFrame f;
    f.orbit.Z = dZ_.p;
    f.orbit.Zfe = dZfe_.p;
    f.orbit.D = dD_.p;
    f.orbit.zm3 = dzm3_.p;
    f.bla = bla_;
    f.bla.use = (use_bla_ && bla_.use) ? 1 : 0;
    f.out.iter = out_iter_;
    f.out.normal = out_norm_;
    f.out.escN = out_n_;
    f.out.glitch = dglitch_.p;
    f.out.done = ddone_.p;
    f.out.gmp = dgmp_.p;
    f.ctr = dctr_;
    f.cancel = dcancel_;
    return f;
}

FrameGeom Engine::geom() const {
    FrameGeom g;
    g.W = W_;
    g.H = H_;
    g.sub = SUB_;
    g.mxit = MXIT_;
    g.ESC2 = ESC2_;
    g.dxf = mpf_ld(dx_);
    g.ede = (cm_ & 2) ? 1 : 0;
    g.deovl = (cm_ & 64) ? 1 : 0;
    g.deriv = deriv_ ? 1 : 0;
    g.normal = (cm_ & 16) ? 1 : 0;
    g.oc = ((cm_ & 8) ? kOcStripe : 0) | ((cm_ & 32) ? kOcTrap : 0);
    g.ER = (double)escf_;
    return g;
}

FeParams Engine::fe_params(int mx_ref_it) const {
    FeParams p;
    p.g = geom();
    p.dxfe = dxfe_;
    p.dyfe = dyfe_;
    p.ref_x = ref_x_;
    p.ref_y = ref_y_;
    p.per = ref_period_;
    p.mx_ref_it = mx_ref_it;
    p.use_interior = use_interior_ ? 1 : 0;
    p.int_rep = 1;
    p.interior_confirm = interior_confirm_;
    p.interior_eps2 = interior_eps2_;
    p.fused = 1;
    // the reference's no-BLA lane kernel has no derivative and no orbit colourings (mp.cpp:2148)
    p.no_bla_kernel = (!use_bla_ && !deriv_ && !(cm_ & (8 | 32))) ? 1 : 0;
    p.ref_period_gt0 = ref_period_ > 0 ? 1 : 0;
    p.cutoff_sensitive = fe_cutoff_sensitive_ ? 1 : 0;
    return p;
}

// Mixed-form pass over a pixel set, three lane passes on one stream with no
// host round trip between them: the FP32 pass; the double-float pass over the
// samples whose FP32 error estimate could change the result; the FP64 pass over
// those the double-float estimate still cannot vouch for. Each rerun pass reads
// its queue length on the device. The host then reads three counter blocks; it
// scans flags only when a block left samples behind (orbit staging timed out).
int Engine::run_pass_mixed(std::vector<uint64_t>* keys, const PixelSet& grid, int mx_ref_it) {
    PixelSet px = grid;
    int n = grid.n;
    std::vector<uint64_t> kept;
    if (keys) {
        n = (int)keys->size();
        if (n == 0) return MBX_OK;
        if (!ensure(dkeys_, n)) return MBX_E_NOMEM;
        copy_async(dkeys_.p, keys->data(), sizeof(uint64_t) * n, cudaMemcpyHostToDevice);
        px.keys = dkeys_.p;
        px.n = n;
        kept.swap(*keys);
    }
    if (n <= 0) return MBX_OK;
    if (!ensure(ddone_, n) || !ensure(drerun_keys_, n) || !ensure(drerun2_keys_, n) || !ensure(drerun_done_, n) || !ensure(drerun_gmp_, n) ||
        !ensure(drerun_flag_, n) || !ensure(dflag_sums_, flag_blocks((unsigned)n) + 1))
        return MBX_E_NOMEM;
    cudaMemsetAsync(ddone_.p, 0, n, st_);
    cudaMemsetAsync(dctr_, 0, 2 * sizeof(Counters), st_);
    ++stats_.passes;
    DeviceFrame f = frame_view();
    f.px = px;
    f.rerun_keys = drerun_keys_.p;
    // the main pass flags its leftovers; they are queued in entry order after
    // it (neighbouring samples in a warp, rather than the order they failed in)
    if (!probe_gate_only_) {
        cudaMemsetAsync(drerun_flag_.p, 0, n, st_);
        f.rerun_flag = drerun_flag_.p;
    }
    const double t0 = now_ms();
    cudaEventRecord(ev0_, st_);
    cudaError_t e = run_mixed_pass(f);
    ++stats_.kernel_launches;
    if (e != cudaSuccess) return fail_cuda("mixed pass launch", e);
    cudaEventRecord(evm_, st_);
    if (probe_gate_only_) {
        // the interior gate's probe: its samples are rendered again by the
        // main pass, so its queue is not rerun; its gate counts the interior
        // decisions the FP32 lane could not vouch for as interior
        copy_async(hctr_, dctr_, sizeof(Counters), cudaMemcpyDeviceToHost);
        e = cudaStreamSynchronize(st_);
        stats_.kernel_ms += now_ms() - t0;
        if (e != cudaSuccess) return fail_cuda("mixed probe pass", e);
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ev0_, evm_) == cudaSuccess) {
            stats_.pass_gpu_ms += ms;
            stats_.fp32_pass_gpu_ms += ms;
        }
        if (cancel_.load()) return MBX_E_CANCELLED;
        stats_.fp32_pass_steps += (long long)hctr_->steps;
        stats_.fp32_pass_bla_applies += (long long)hctr_->bla_applies;
        hctr_->interior += hctr_->interior_flagged;
        stats_.steps += (long long)hctr_->steps;
        stats_.bla_applies += (long long)hctr_->bla_applies;
        stats_.bla_skipped += (long long)hctr_->bla_skipped;
        stats_.samples += n;
        if ((int)hctr_->finished < n) hctr_->interior += 1; // samples left unstarted: keep the detectors on
        return MBX_OK;
    }
    auto queue_frame = [&](uint64_t* q, int ctr_in, uint64_t* next_q, int ctr_out) {
        DeviceFrame r = frame_view();
        r.px = PixelSet();
        r.px.keys = q;
        r.px.n = n;
        r.px.n_dev = &dctr_[ctr_in].rerun_n;
        r.px.grid_w = r.px.grid_h = r.px.grid_step = 1;
        r.px.skip_i = r.px.skip_j = -1;
        r.out.done = drerun_done_.p;
        r.out.gmp = drerun_gmp_.p;
        r.ctr = dctr_ + ctr_out;
        r.rerun_keys = next_q;
        return r;
    };
    e = launch_flag_compact(px, (unsigned)n, drerun_flag_.p, dflag_sums_.p, drerun_keys_.p, st_);
    if (e != cudaSuccess) return fail_cuda("rerun queue compaction", e);
    stats_.kernel_launches += 3;
    e = run_df_pass(queue_frame(drerun_keys_.p, 0, drerun2_keys_.p, 1));
    stats_.kernel_launches += 2; // narrow and wide variants, one of which runs
    if (e != cudaSuccess) return fail_cuda("double-float rerun launch", e);
    cudaEventRecord(ev1_, st_);
    copy_async(hctr_, dctr_, 2 * sizeof(Counters), cudaMemcpyDeviceToHost);
    e = cudaStreamSynchronize(st_);
    stats_.kernel_ms += now_ms() - t0;
    if (e != cudaSuccess) return fail_cuda("mixed pass", e);
    {
        float ms = 0.0f, rms = 0.0f, fms = 0.0f;
        if (cudaEventElapsedTime(&ms, ev0_, ev1_) == cudaSuccess) stats_.pass_gpu_ms += ms;
        if (cudaEventElapsedTime(&rms, evm_, ev1_) == cudaSuccess) stats_.rerun_gpu_ms += rms;
        if (cudaEventElapsedTime(&fms, ev0_, evm_) == cudaSuccess) stats_.fp32_pass_gpu_ms += fms;
        stats_.fp32_pass_steps += (long long)hctr_[0].steps;
        stats_.fp32_pass_bla_applies += (long long)hctr_[0].bla_applies;
        stats_.fp32_unvouched_interior += (long long)hctr_[0].interior_flagged;
        stats_.fp32_unvouched_escape += (long long)hctr_[0].escape_flagged;
    }
    if (cancel_.load()) return MBX_E_CANCELLED;
    if ((hctr_[0].stage_timeouts | hctr_[1].stage_timeouts) >> 16) {
        err_ = "orbit staging copy still in flight when its block finished";
        return MBX_E_CUDA;
    }
    Counters& a = hctr_[0];
    for (int k = 1; k < 2; ++k) {
        const Counters& b = hctr_[k];
        a.steps += b.steps;
        a.bla_applies += b.bla_applies;
        a.bla_skipped += b.bla_skipped;
        a.effective_iters += b.effective_iters;
        a.interior += b.interior; // callers read the pass's interior count from hctr_
    }
    stats_.rebases += (long long)a.rebases;
    stats_.exact_steps += (long long)a.exact_steps;
    stats_.fe_rebases += (long long)a.fe_rebases;
    stats_.steps += (long long)a.steps;
    stats_.bla_applies += (long long)a.bla_applies;
    stats_.bla_skipped += (long long)a.bla_skipped;
    stats_.effective_iterations += (long long)a.effective_iters;
    stats_.interior += (int)a.interior;
    stats_.fp64_reruns += std::min<unsigned>(a.rerun_n, (unsigned)n);
    stats_.fp64_reruns_fp64 += std::min<unsigned>(hctr_[1].rerun_n, (unsigned)n);
    stats_.samples += n;
    const bool unstarted = (int)a.finished < n;
    const unsigned n_exact = std::min<unsigned>(hctr_[1].rerun_n, (unsigned)n);
    if (unstarted) {
        // A block left samples unstarted (orbit staging timed out): scan the
        // flags and take them through the FP64 floatexp pass.
        hdone_.resize(n);
        copy_async(hdone_.data(), ddone_.p, n, cudaMemcpyDeviceToHost);
        e = cudaStreamSynchronize(st_);
        if (e != cudaSuccess) return fail_cuda("pass readback", e);
        std::vector<uint64_t> pending;
        for (int i = 0; i < n; ++i) {
            if (hdone_[i]) continue;
            int arr[4];
            if (keys) key_unpack(kept[i], arr);
            else entry_coords(px, i, arr);
            pending.push_back(key_pack(arr[0], arr[1], arr[2], arr[3]));
        }
        stats_.fp64_reruns += (long long)pending.size();
        exact_rerun_ = true;
        PixelSet g = PixelSet();
        g.grid_w = g.grid_h = g.grid_step = 1;
        g.skip_i = g.skip_j = -1;
        const int rc = run_pass(&pending, g, mx_ref_it, nullptr, nullptr);
        exact_rerun_ = false;
        if (rc != MBX_OK) return rc;
        if (!pending.empty()) {
            err_ = "floatexp pass left samples unfinished";
            return MBX_E_CUDA;
        }
    }
    if (n_exact > 0) {
        // Samples the double-float estimate cannot vouch for either: the exact
        // form (the reference's FP64 floatexp loop with its arbitrary-precision
        // recomputes) finishes them, so every sample carries either a vouched
        // result or the exact form's.
        std::vector<uint64_t> pending(n_exact);
        copy_async(pending.data(), drerun2_keys_.p, sizeof(uint64_t) * n_exact, cudaMemcpyDeviceToHost);
        e = cudaStreamSynchronize(st_);
        if (e != cudaSuccess) return fail_cuda("double-float rerun readback", e);
        stats_.exact_reruns += (long long)n_exact;
        const double gpu0 = stats_.pass_gpu_ms;
        exact_rerun_ = true;
        PixelSet g = PixelSet();
        g.grid_w = g.grid_h = g.grid_step = 1;
        g.skip_i = g.skip_j = -1;
        const int rc = run_pass(&pending, g, mx_ref_it, nullptr, nullptr);
        exact_rerun_ = false;
        stats_.rerun_fp64_gpu_ms += stats_.pass_gpu_ms - gpu0;
        if (rc != MBX_OK) return rc;
        if (!pending.empty()) {
            err_ = "floatexp pass left samples unfinished";
            return MBX_E_CUDA;
        }
    }
    return MBX_OK;
}

// One delta pass over a pixel set (stepParallel, mp.cpp:2092-2607). On return
// `keys` (if any) holds the still-pending entries in order and `new_ref` the
// minimum-glitch-score entry (first in set order on ties), if any.
int Engine::run_pass(std::vector<uint64_t>* keys, const PixelSet& grid, int mx_ref_it, bool* have_new_ref, int* new_ref) {
    if (use_floatexp_ && mixed_active() && !exact_rerun_) {
        if (have_new_ref) *have_new_ref = false;
        return run_pass_mixed(keys, grid, mx_ref_it);
    }
    PixelSet px = grid;
    int n = grid.n;
    if (keys) {
        n = (int)keys->size();
        px.keys = nullptr;
        px.n = n;
        if (n == 0) return MBX_OK;
        if (!ensure(dkeys_, n)) return MBX_E_NOMEM;
        copy_async(dkeys_.p, keys->data(), sizeof(uint64_t) * n, cudaMemcpyHostToDevice);
        px.keys = dkeys_.p;
    }
    if (n <= 0) return MBX_OK;
    if (!ensure(ddone_, n) || !ensure(dglitch_, n) || !ensure(dgmp_, n)) return MBX_E_NOMEM;
    cudaMemsetAsync(ddone_.p, 0, n, st_);
    cudaMemsetAsync(dgmp_.p, 0, n, st_);
    cudaMemsetAsync(dctr_, 0, sizeof(Counters), st_);
    ++stats_.passes;
    DeviceFrame f = frame_view();
    f.px = px;
    const int threads = 128;
    const double t0 = now_ms();
    cudaError_t e;
    cudaEventRecord(ev0_, st_);
    if (use_floatexp_) {
        FeParams p = fe_params(mx_ref_it);
        int blocks = std::min((n + threads - 1) / threads, nsm_ * 8);
        if (exact_rerun_) {
            // the mixed form's leftovers: few samples with long dependency
            // chains, spread over every SM's four schedulers, a one-warp block
            // each, with as few lanes per warp as hold them all, so that
            // neither divergence nor a shared FP64 pipe serialises them
            // (measured on the minibrot frame's 1,270 leftovers: full warps
            // on 10 SMs 40.3 ms, spread 34.9 ms)
            const int warps = nsm_ * 4;
            const int lpw = std::max(1, std::min(32, (n + warps - 1) / warps));
            p.lanes_per_warp = lpw;
            e = launch_fe_pass(f, p, (n + lpw - 1) / lpw, 32, st_);
        } else {
            e = launch_fe_pass(f, p, blocks, threads, st_);
        }
    } else {
        Fp64Params p;
        p.g = geom();
        memcpy(p.ref, ref_, sizeof(ref_));
        p.xoff = dc_xoff_;
        p.yoff = dc_yoff_;
        p.dcx = ddcx_.p;
        p.dcy = ddcy_.p;
        p.frac_re = ref_frac_re_;
        p.frac_im = ref_frac_im_;
        p.per = ref_period_;
        for (int q = 0; q < kSaTerms; ++q) {
            p.A[q] = sa_A_[q];
            p.B[q] = sa_B_[q];
        }
        p.sa_delta = sa_delta_;
        p.sa_order = sa_order_;
        p.sa_it = sa_it_;
        p.mx_ref_it = mx_ref_it;
        p.use_interior = use_interior_ ? 1 : 0;
        p.int_rep = 1;
        p.interior_confirm = interior_confirm_;
        p.interior_eps2 = interior_eps2_;
        int blocks = std::min((n + threads - 1) / threads, nsm_ * 8);
        e = launch_fp64_pass(f, p, blocks, threads, st_);
    }
    ++stats_.kernel_launches;
    if (e != cudaSuccess) return fail_cuda("delta pass launch", e);
    cudaEventRecord(ev1_, st_);
    copy_async(hctr_, dctr_, sizeof(Counters), cudaMemcpyDeviceToHost);
    e = cudaStreamSynchronize(st_);
    stats_.kernel_ms += now_ms() - t0;
    if (e != cudaSuccess) return fail_cuda("delta pass", e);
    {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ev0_, ev1_) == cudaSuccess) {
            stats_.pass_gpu_ms += ms;
            if (exact_rerun_) stats_.rerun_gpu_ms += ms;
        }
    }
    stats_.rebases += (long long)hctr_->rebases;
    if (cancel_.load()) return MBX_E_CANCELLED;
    stats_.steps += (long long)hctr_->steps;
    stats_.bla_applies += (long long)hctr_->bla_applies;
    stats_.bla_skipped += (long long)hctr_->bla_skipped;
    stats_.effective_iterations += (long long)hctr_->effective_iters;
    stats_.interior += (int)hctr_->interior;
    stats_.samples += n;
    // Pending entries, arbitrary-precision recomputes and the next reference.
    hdone_.resize(n);
    hgmp_.resize(n);
    copy_async(hdone_.data(), ddone_.p, n, cudaMemcpyDeviceToHost);
    copy_async(hgmp_.data(), dgmp_.p, n, cudaMemcpyDeviceToHost);
    const bool glitches = !use_floatexp_;
    if (glitches) {
        hglitch_.resize(n);
        copy_async(hglitch_.data(), dglitch_.p, sizeof(double) * n, cudaMemcpyDeviceToHost);
    }
    e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return fail_cuda("pass readback", e);
    auto key_of = [&](int i, int* a) {
        if (keys) {
            key_unpack((*keys)[i], a);
            return;
        }
        int cols = (px.grid_w + px.grid_step - 1) / px.grid_step;
        int q = i;
        if (px.skip_i >= 0) {
            int sq = (px.skip_i / px.grid_step) * cols + px.skip_j / px.grid_step;
            if (q >= sq) ++q;
        }
        a[0] = (q / cols) * px.grid_step;
        a[1] = (q % cols) * px.grid_step;
        a[2] = 0;
        a[3] = 0;
    };
    // mp.cpp:2173-2183: EMPTY / cutoff-sensitive floatexp samples in arbitrary precision.
    std::vector<int> gmp_list;
    for (int i = 0; i < n; ++i)
        if (hgmp_[i]) gmp_list.push_back(i);
    if (!gmp_list.empty()) {
        int r = recompute_gmp(gmp_list, key_of);
        if (r != MBX_OK) return r;
    }
    if (have_new_ref) *have_new_ref = false;
    std::vector<uint64_t> pending;
    double min_orbit = 1e100;
    for (int i = 0; i < n; ++i) {
        if (hdone_[i]) continue;
        int a[4];
        key_of(i, a);
        pending.push_back(key_pack(a[0], a[1], a[2], a[3]));
        if (glitches && hglitch_[i] >= 0 && hglitch_[i] < min_orbit) {
            min_orbit = hglitch_[i];
            if (have_new_ref) {
                *have_new_ref = true;
                memcpy(new_ref, a, sizeof(a));
            }
        }
    }
    if (use_floatexp_ && !pending.empty()) {
        err_ = "floatexp pass left samples unfinished";
        return MBX_E_CUDA;
    }
    if (keys) keys->swap(pending);
    else if (!pending.empty()) {
        // Grid passes feed the caller through `grid_pending_`.
        grid_pending_.swap(pending);
    }
    return MBX_OK;
}

int Engine::recompute_gmp(const std::vector<int>& list, const std::function<void(int, int*)>& key_of) {
    const int n = (int)list.size();
    std::vector<float> vals(n);
    std::vector<int32_t> ns(n);
    std::vector<int> idx(n);
    int W2 = W_ * SUB_;
    for (int q = 0; q < n; ++q) {
        int a[4];
        key_of(list[q], a);
        idx[q] = (a[0] * SUB_ + SUB_ / 2 + a[2]) * W2 + (a[1] * SUB_ + SUB_ / 2 + a[3]);
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int q = 0; q < n; ++q) {
        int a[4];
        key_of(list[q], a);
        vals[q] = gmp_sample(a, MXIT_, &ns[q]);
    }
    if (cancel_.load()) return MBX_E_CANCELLED;
    stats_.gmp_pixels += n;
    for (int q = 0; q < n; ++q) {
        copy_async(out_iter_ + idx[q], &vals[q], sizeof(float), cudaMemcpyHostToDevice);
        if (out_n_) copy_async(out_n_ + idx[q], &ns[q], sizeof(int32_t), cudaMemcpyHostToDevice);
    }
    cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return fail_cuda("gmp writeback", e);
    return MBX_OK;
}

int Engine::write_sample(const int* a, float v, int32_t n) {
    const int idx = (a[0] * SUB_ + SUB_ / 2 + a[2]) * W_ * SUB_ + (a[1] * SUB_ + SUB_ / 2 + a[3]);
    copy_async(out_iter_ + idx, &v, sizeof(float), cudaMemcpyHostToDevice);
    if (out_n_) copy_async(out_n_ + idx, &n, sizeof(int32_t), cudaMemcpyHostToDevice);
    return cuda_ok("sample write");
}

int Engine::flush_ref_value() {
    if (!ref_value_pending_) return MBX_OK;
    ref_value_pending_ = false;
    float v = ref_value_;
    int32_t n = ref_n_;
    // Values stored into host temporaries must outlive the async copy.
    ref_value_store_ = v;
    ref_n_store_ = n;
    const int idx = (ref_[0] * SUB_ + SUB_ / 2 + ref_[2]) * W_ * SUB_ + (ref_[1] * SUB_ + SUB_ / 2 + ref_[3]);
    copy_async(out_iter_ + idx, &ref_value_store_, sizeof(float), cudaMemcpyHostToDevice);
    if (out_n_) copy_async(out_n_ + idx, &ref_n_store_, sizeof(int32_t), cudaMemcpyHostToDevice);
    cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return fail_cuda("reference value", e);
    return MBX_OK;
}

// ---------------------------------------------------------------------------
// Mandel::Compute (mp.cpp:1388-2028) for the Mandelbrot mode.
void Engine::fill_batch_slot() {
    ViewDesc d{};
    d.f = frame_view();
    if (!(bla_.use && dbla32_.p)) d.f.bla.use = 0;
    d.p = mixed_params();
    d.bla32 = dbla32_.p;
    d.orb32 = dZf_.p;
    d.bladf = dbladf_.p;
    d.orbdf = dZdf_.p;
    d.interior_gate = 0;
    d.base = 0;
    // probe on the 1/8 grid with interior detection on (mp.cpp:1668-1720)
    ViewDesc pr = d;
    pr.f.px = PixelSet();
    pr.f.px.keys = nullptr;
    pr.f.px.grid_w = W_;
    pr.f.px.grid_h = H_;
    pr.f.px.grid_step = 8;
    pr.f.px.skip_i = pr.f.px.skip_j = -1;
    pr.f.px.n = ((H_ + 7) / 8) * ((W_ + 7) / 8);
    pr.p.use_interior = 1;
    pr.p.g.ede = pr.p.g.deovl = pr.p.g.normal = pr.p.g.deriv = 0; // the probe needs no DE values
    pr.count = (unsigned)pr.f.px.n;
    // main pass over the frame minus the reference pixel
    ViewDesc mn = d;
    mn.f.px = PixelSet();
    mn.f.px.keys = nullptr;
    mn.f.px.grid_w = W_;
    mn.f.px.grid_h = H_;
    mn.f.px.grid_step = 1;
    mn.f.px.skip_i = ref_virtual_ ? -1 : H_ / 2;
    mn.f.px.skip_j = ref_virtual_ ? -1 : W_ / 2;
    mn.f.px.n = W_ * H_ - (ref_virtual_ ? 0 : 1);
    mn.p.use_interior = 1;
    mn.interior_gate = 1;
    mn.count = (unsigned)mn.f.px.n;
    pr.f.out.cost = mn.f.out.cost = nullptr;
    pr.f.out.bla = mn.f.out.bla = nullptr;
    pr.pgrid = mn.pgrid = nullptr;
    pr.pgw = mn.pgw = (W_ + 7) / 8;
    pr.pgh = mn.pgh = (H_ + 7) / 8;
    pr.tw = mn.tw = (W_ + 15) / 16;
    pr.th = mn.th = (H_ + 15) / 16;
    pr.tile_base = mn.tile_base = 0; // set by the batch
    if (batch_slot_->want_cost && ensure(dcost_, (size_t)W_ * H_) && ensure(dblac_, (size_t)W_ * H_) && ensure(dpgrid_, (size_t)mn.pgw * mn.pgh)) {
        pr.f.out.cost = mn.f.out.cost = dcost_.p;
        pr.f.out.bla = mn.f.out.bla = dblac_.p;
        pr.pgrid = mn.pgrid = dpgrid_.p;
    }
    batch_slot_->probe = pr;
    batch_slot_->main = mn;
    batch_slot_->deferred = true;
    stats_.passes += 2;
    stats_.samples += pr.count + mn.count;
}

int Engine::compute_deferred(const mbx_request& r, BatchSlot* slot, mbx_stats* out_stats) {
    slot->deferred = false;
    batch_slot_ = slot;
    const int rc = compute(r, out_stats);
    batch_slot_ = nullptr;
    return rc;
}

int Engine::batch_exact_rerun(std::vector<uint64_t>& keys, bool interior_seen) {
    if (keys.empty()) return MBX_OK;
    stats_.exact_reruns += (long long)keys.size();
    stats_.fp64_reruns_fp64 += (long long)keys.size();
    // interior detection as the single-frame render's gate leaves it
    const bool interior = use_interior_;
    if (!interior_seen) use_interior_ = false;
    exact_rerun_ = true;
    PixelSet g = PixelSet();
    g.grid_w = g.grid_h = g.grid_step = 1;
    g.skip_i = g.skip_j = -1;
    const int rc = run_pass(&keys, g, batch_ref_it_, nullptr, nullptr);
    exact_rerun_ = false;
    use_interior_ = interior;
    if (rc != MBX_OK) return rc;
    if (!keys.empty()) {
        err_ = "floatexp pass left samples unfinished";
        return MBX_E_CUDA;
    }
    return MBX_OK;
}

// The adaptive supersampling of a batched frame (mp.cpp:1789-2006), after the
// batch's shared passes gave it its centre samples; interior detection as the
// frame's probe left it.
int Engine::batch_supersample(bool interior_seen) {
    if (!(SUB_ > 1 && (cm_ & 1))) return MBX_OK;
    const bool interior = use_interior_;
    if (!interior_seen) use_interior_ = false;
    const int rc = supersample(batch_ref_it_);
    use_interior_ = interior;
    return rc;
}

int Engine::batch_finish(const mbx_request& r, mbx_stats* out_stats) {
    const size_t nsamp = (size_t)r.width * r.height * r.sub * r.sub;
    const double t0 = now_ms();
    if (!r.outputs_on_device) {
        copy_async(r.iterations, out_iter_, sizeof(float) * nsamp, cudaMemcpyDeviceToHost);
        if (r.normal) copy_async(r.normal, out_norm_, sizeof(float) * nsamp, cudaMemcpyDeviceToHost);
        if (r.escape_iteration) copy_async(r.escape_iteration, out_n_, sizeof(int32_t) * nsamp, cudaMemcpyDeviceToHost);
        cudaError_t e = cudaStreamSynchronize(st_);
        stats_.copy_ms += now_ms() - t0;
        if (e != cudaSuccess) return fail_cuda("output readback", e);
    }
    if (r.progress) *r.progress = 1.0f;
    if (out_stats) *out_stats = stats_;
    return MBX_OK;
}

int Engine::compute(const mbx_request& r, mbx_stats* out_stats) {
    bool expected = false;
    if (!active_.compare_exchange_strong(expected, true)) return MBX_E_BUSY;
    struct Release {
        std::atomic<bool>& a;
        ~Release() { a.store(false); }
    } release{active_};
    if (cancel_.load()) return MBX_E_CANCELLED;
    stats_ = mbx_stats();
    rng_.seed(1);
    const double t_begin = now_ms();
    int rc = compute_frame(r);
    stats_.total_ms = now_ms() - t_begin;
    stats_.method = method_;
    stats_.used_floatexp = use_floatexp_ ? 1 : 0;
    stats_.period = ref_period_;
    if (out_stats) *out_stats = stats_;
    return rc;
}

int Engine::compute_frame(const mbx_request& r) {
    W_ = r.width;
    H_ = r.height;
    SUB_ = r.sub;
    MXIT_ = r.max_iterations;
    cm_ = r.coloring_method;
    mode_ = r.precision_mode;
    deriv_ = (cm_ & (2 | 16 | 64)) != 0; // EDE, normal map, DE overlay (mp.cpp:4190-4192)
    zoom_period_ = r.reference_period > 0 ? r.reference_period : 0;
    if (zoom_period_ > 0) {
        zoom_re_ = r.reference_re;
        zoom_im_ = r.reference_im;
    }
    escf_ = (float)(r.bailout > 0 ? r.bailout : 1e8);
    ESC2_ = (double)(escf_ * escf_);
    const int full_h = r.full_height > 0 ? r.full_height : 0;
    const int row_base = r.row_base;
    std::string sdig = r.scale;
    int prec = r.precision_bits;
    if (prec <= 0) {
        size_t digits = 0;
        for (char ch : sdig)
            if (ch >= '0' && ch <= '9') ++digits;
        prec = (int)(digits * std::log(10) / std::log(2)) + 64;
    }
    // Every mpf value of a frame takes this precision explicitly (the library
    // never relies on GMP's process-wide default), so engines may build their
    // references concurrently.
    set_precision(prec);
    {
        char buf[256];
        snprintf(buf, sizeof(buf), "|%d|%d|%d|%d|%d|%d|%d|%d|%.17g|%d|", prec, W_, H_, full_h, row_base, SUB_, MXIT_, cm_, (double)escf_, mode_);
        frame_key_ = std::string(r.center_re) + "|" + r.center_im + "|" + r.scale + buf;
        reuse_ = r.reuse_reference && cache_.valid && cache_.key == frame_key_;
        if (!reuse_) cache_.valid = false;
    }
    MpfTemp cre(prec), cim(prec), msc(prec);
    if (mpf_set_str(cre, r.center_re, 10) != 0 || mpf_set_str(cim, r.center_im, 10) != 0 || mpf_set_str(msc, r.scale, 10) != 0 || mpf_sgn(msc) <= 0) {
        err_ = "unparsable centre or scale";
        return MBX_E_INVALID;
    }
    // Device outputs.
    const size_t nsamp = (size_t)W_ * H_ * SUB_ * SUB_;
    float* out_iter = nullptr;
    float* out_norm = nullptr;
    int32_t* out_n = nullptr;
    if (r.outputs_on_device) {
        out_iter = r.iterations;
        out_norm = r.normal;
        out_n = r.escape_iteration;
    } else {
        if (!ensure(diter_own_, nsamp)) return MBX_E_NOMEM;
        out_iter = diter_own_.p;
        if (r.normal) {
            if (!ensure(dnormal_own_, nsamp)) return MBX_E_NOMEM;
            out_norm = dnormal_own_.p;
        }
        if (r.escape_iteration) {
            if (!ensure(descN_own_, nsamp)) return MBX_E_NOMEM;
            out_n = descN_own_.p;
        }
    }
    out_iter_ = out_iter;
    out_norm_ = out_norm;
    out_n_ = out_n;
    cudaError_t e = launch_fill(out_iter, out_norm, out_n, nsamp, st_);
    if (e != cudaSuccess) return fail_cuda("fill", e);
    int rc;
    if (r.compute_mode == MBX_MODE_JULIA) {
        reuse_ = false;
        rc = render_julia(cre, cim, msc, r.fixed_c_re, r.fixed_c_im, full_h, row_base);
    } else {
        rc = render(cre, cim, msc, full_h, row_base, r.progress);
    }
    if (batch_slot_ && batch_slot_->deferred) return rc; // passes and readback follow in the batch
    if (rc == MBX_OK && !r.outputs_on_device) {
        const double t0 = now_ms();
        copy_async(r.iterations, out_iter, sizeof(float) * nsamp, cudaMemcpyDeviceToHost);
        if (r.normal) copy_async(r.normal, out_norm, sizeof(float) * nsamp, cudaMemcpyDeviceToHost);
        if (r.escape_iteration) copy_async(r.escape_iteration, out_n, sizeof(int32_t) * nsamp, cudaMemcpyDeviceToHost);
        e = cudaStreamSynchronize(st_);
        stats_.copy_ms += now_ms() - t0;
        if (e != cudaSuccess) return fail_cuda("output readback", e);
    }
    if (rc == MBX_OK && cancel_.load()) rc = MBX_E_CANCELLED;
    if (rc == MBX_OK && r.progress) *r.progress = 1.0f;
    return rc;
}

int Engine::render(mpf_ptr c_re, mpf_ptr c_im, mpf_ptr scale, int full_h, int row_base, volatile float* progress) {
    mpf_set(scale_, scale);
    const int rows = (full_h > 0) ? full_h : H_;
    {
        const mp_bitcnt_t pr = mpf_get_prec(c0_re_);
        MpfTemp dw(pr), dh(pr);
        mpf_set_ui(dw, 2);
        mpf_div(dw, dw, scale);
        mpf_set(dh, dw);
        mpf_div_ui(dh, dh, W_);
        mpf_mul_ui(dh, dh, rows);
        mpf_sub(c0_re_, c_re, dw);
        mpf_sub(c0_im_, c_im, dh);
        mpf_div_ui(dx_, dw, W_ - 1);
        mpf_mul_ui(dx_, dx_, 2);
        mpf_div_ui(dy_, dh, rows - 1);
        mpf_mul_ui(dy_, dy_, 2);
        if (row_base > 0) {
            MpfTemp off(pr);
            mpf_mul_ui(off, dy_, row_base);
            mpf_add(c0_im_, c0_im_, off);
        }
    }
    method_ = mpf_cmp_d(scale, 1e6) > 0 ? 1 : 0;
    ref_value_pending_ = false;
    if (method_ == 0) return render_shallow(progress);
    use_bla_ = true;
    bla_minlevel_ = 3; // MANDEL_BLA_MINSKIP default 8 -> level 3 (mp.cpp:1542-1547)
    use_interior_ = true;
    interior_eps2_ = 3e-9 * 3e-9;
    interior_confirm_ = 4;
    use_floatexp_ = mpf_cmp_d(scale, 1e280) > 0;
    // The mixed form's lanes rebase (a delta whose |z| falls below |dz| restarts
    // from the start of the reference), so one floatexp reference serves frames
    // of any depth: its frames below the reference's floatexp gate (mp.cpp:
    // 1573-1576) take the floatexp path too, with no glitch re-reference passes.
    if (mixed_active()) use_floatexp_ = true;
    fe_cutoff_sensitive_ = false;
    dxfe_ = mpf_fe(dx_);
    dyfe_ = mpf_fe(dy_);
    int ref_it = 0;
    int rc = MBX_OK;
    refs_built_in_frame_ = 0;
    if (zoom_period_ > 0) {
        rc = zoom_reference(&ref_it);
        if (rc != MBX_OK) return rc;
    } else if (reuse_ && restore_cache(&ref_it)) {
        stats_.reused_reference = 1; // the host orbit shadows still hold this reference
    } else {
        zoom_valid_ = false; // the orbit shadows are rebuilt below
        // host orbit shadows, up to maxiter + 1 entries (tens of MB at maxiter
        // 1e6): cleared only when a reference is built
        hZ_.assign((size_t)MXIT_ + 2, make_double2(0, 0));
        hzm3_.assign((size_t)MXIT_ + 2, 0.0);
        hD_.assign((size_t)MXIT_ + 2, make_double2(0, 0));
        hZfe_.assign((size_t)MXIT_ + 2, FE2{fe_make(0, 0), fe_make(0, 0)});
        ref_it = reference_for_frame();
        if (cancel_.load()) return MBX_E_CANCELLED;
        stats_.reference_length = ref_period_ > 0 ? ref_period_ : ref_it;
        if (ref_subpixel_) use_bla_ = false;
        rc = upload_reference(ref_it);
        if (rc != MBX_OK) return rc;
        if (use_bla_) {
            rc = build_bla(ref_period_ > 0 ? ref_period_ : ref_it);
            if (rc != MBX_OK) return rc;
        }
        if (!use_floatexp_) {
            rc = build_dc_tables();
            if (rc != MBX_OK) return rc;
        }
        if (mixed_active() && use_floatexp_) {
            rc = prepare_mixed();
            if (rc != MBX_OK) return rc;
        }
        save_cache(ref_it);
    }
    refs_built_in_frame_ = 0;
    rc = flush_ref_value();
    if (rc != MBX_OK) return rc;
    if (progress) *progress = 0.08f;
    // (the learned ordering's per-sample costs assume sub 1: with it on,
    // supersampled frames render on their own)
    if (batch_slot_ && use_floatexp_ && mixed_active() && (SUB_ == 1 || !batch_slot_->want_cost)) {
        batch_ref_it_ = ref_it;
        fill_batch_slot(); // the probe and main passes run in the batch's launches
        return MBX_OK;
    }
    // Interior auto-gate probe on the 1/8 grid (mp.cpp:1668-1720).
    {
        PixelSet g;
        g.keys = nullptr;
        g.grid_w = W_;
        g.grid_h = H_;
        g.grid_step = 8;
        g.skip_i = g.skip_j = -1;
        g.n = ((H_ + 7) / 8) * ((W_ + 7) / 8);
        grid_pending_.clear();
        probe_gate_only_ = true;
        rc = run_pass(nullptr, g, ref_it, nullptr, nullptr);
        probe_gate_only_ = false;
        if (rc != MBX_OK) return rc;
        if (hctr_->interior == 0) use_interior_ = false;
    }
    // Main passes with glitch re-referencing (mp.cpp:1724-1761).
    std::vector<uint64_t> pending;
    {
        PixelSet g;
        g.keys = nullptr;
        g.grid_w = W_;
        g.grid_h = H_;
        g.grid_step = 1;
        g.skip_i = ref_virtual_ ? -1 : H_ / 2;
        g.skip_j = ref_virtual_ ? -1 : W_ / 2;
        g.n = W_ * H_ - (ref_virtual_ ? 0 : 1);
        grid_pending_.clear();
        bool have = false;
        int nr[4];
        rc = run_pass(nullptr, g, ref_it, &have, nr);
        if (rc != MBX_OK) return rc;
        pending.swap(grid_pending_);
        rc = glitch_loop(pending, ref_it, have, nr, progress);
        if (rc != MBX_OK) return rc;
    }
    const bool is_ss = (SUB_ > 1) && (cm_ & 1);
    if (!is_ss) return MBX_OK;
    return supersample(ref_it);
}

int Engine::glitch_loop(std::vector<uint64_t>& pending, int& ref_it, bool have, int* nr, volatile float* progress) {
    // Reference pixel: the minimum-score pending pixel; libc rand() picks one
    // when no valid score exists (mp.cpp:4045-4056).
    while (!pending.empty()) {
        if (cancel_.load()) return MBX_E_CANCELLED;
        int pick[4];
        uint64_t want = have ? key_pack(nr[0], nr[1], nr[2], nr[3]) : ~0ull;
        auto it = std::lower_bound(pending.begin(), pending.end(), want);
        if (!have || it == pending.end() || *it != want) it = pending.begin() + (rng_.next() % pending.size());
        key_unpack(*it, pick);
        pending.erase(it);
        cache_.valid = false; // the frame's reference changes
        ref_it = build_reference(pick, false);
        if (cancel_.load()) return MBX_E_CANCELLED;
        int rc = upload_reference(ref_it);
        if (rc != MBX_OK) return rc;
        const bool ss_follows = (SUB_ > 1) && (cm_ & 1);
        if ((!pending.empty() || ss_follows) && use_bla_) {
            rc = build_bla(ref_it);
            if (rc != MBX_OK) return rc;
        }
        rc = build_dc_tables();
        if (rc != MBX_OK) return rc;
        rc = flush_ref_value();
        if (rc != MBX_OK) return rc;
        if (pending.empty()) break;
        PixelSet g;
        g.keys = nullptr;
        g.n = 0;
        g.grid_w = g.grid_h = g.grid_step = 1;
        g.skip_i = g.skip_j = -1;
        have = false;
        rc = run_pass(&pending, g, ref_it, &have, nr);
        if (rc != MBX_OK) return rc;
        if (progress) *progress = 0.9f;
    }
    return MBX_OK;
}

// Adaptive supersampling (mp.cpp:1796-2006).
int Engine::supersample(int ref_it) {
    if (!ensure(dflags_, (size_t)W_ * H_)) return MBX_E_NOMEM;
    const double thresh = std::log((double)MXIT_) / 8.0;
    // EDE: the set boundary; the stripe average: the boundary (palette steps 0);
    // orbit traps: the boundary or more than 3 palette entries per pixel, at the
    // palette density 60 the compute backend leaves (mp.cpp:1810-1838)
    const double density = 60.0;
    const int mode = (cm_ & 2) ? kSsEde : (cm_ & 8) ? kSsStripe : (cm_ & 32) ? kSsTrap : kSsIterations;
    const double gain = mode == kSsStripe ? density * (2048.0 / 20.0) : density / 60.0 * 2048.0;
    const double steps = mode == kSsStripe ? 0.0 : 3.0;
    cudaError_t e = launch_ss_flags(out_iter_, W_, H_, SUB_, mode, thresh, gain, steps, dflags_.p, st_);
    ++stats_.kernel_launches;
    if (e != cudaSuccess) return fail_cuda("ss flags", e);
    std::vector<uint8_t> flags((size_t)W_ * H_);
    copy_async(flags.data(), dflags_.p, flags.size(), cudaMemcpyDeviceToHost);
    e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return fail_cuda("ss flags", e);
    std::vector<uint64_t> samples;
    for (int i = 0; i < H_; ++i)
        for (int j = 0; j < W_; ++j) {
            if (!flags[(size_t)i * W_ + j]) continue;
            for (int yi = -SUB_ / 2; yi <= SUB_ / 2; ++yi)
                for (int xi = -SUB_ / 2; xi <= SUB_ / 2; ++xi) {
                    if (xi == 0 && yi == 0) continue;
                    samples.push_back(key_pack(i, j, yi, xi));
                }
        }
    if (samples.empty()) return MBX_OK;
    if (method_ == 0) return shallow_samples(samples);
    PixelSet g;
    g.keys = nullptr;
    g.n = 0;
    g.grid_w = g.grid_h = g.grid_step = 1;
    g.skip_i = g.skip_j = -1;
    if (use_floatexp_) return run_pass(&samples, g, ref_it, nullptr, nullptr);
    // Double path: first pass with the current BLA table, then glitch passes
    // with BLA off because the table belongs to the previous reference.
    const bool saved_bla = use_bla_;
    bool have = false;
    int nr[4];
    int rc = run_pass(&samples, g, ref_it, &have, nr);
    while (rc == MBX_OK && !samples.empty()) {
        if (cancel_.load()) {
            rc = MBX_E_CANCELLED;
            break;
        }
        int pick[4];
        uint64_t want = have ? key_pack(nr[0], nr[1], nr[2], nr[3]) : ~0ull;
        auto it = std::lower_bound(samples.begin(), samples.end(), want);
        if (!have || it == samples.end() || *it != want) it = samples.begin() + (rng_.next() % samples.size());
        key_unpack(*it, pick);
        samples.erase(it);
        cache_.valid = false;
        ref_it = build_reference(pick, false);
        rc = upload_reference(ref_it);
        if (rc != MBX_OK) break;
        rc = build_dc_tables();
        if (rc != MBX_OK) break;
        rc = flush_ref_value();
        if (rc != MBX_OK) break;
        use_bla_ = false;
        if (samples.empty()) break;
        have = false;
        rc = run_pass(&samples, g, ref_it, &have, nr);
    }
    use_bla_ = saved_bla;
    return rc;
}

// Julia frames: Mandel::ComputeJulia (mp.cpp:992-1044). The geometry is
// ComputeJulia's own (its operation order differs from Compute's), then one
// pass over the grid in double precision.
int Engine::render_julia(mpf_ptr z_re, mpf_ptr z_im, mpf_ptr scale, const char* fcr, const char* fci, int full_h, int row_base) {
    method_ = 0;
    use_floatexp_ = false;
    ref_period_ = 0;
    const int rows = full_h > 0 ? full_h : H_;
    const mp_bitcnt_t pr = mpf_get_prec(c0_re_);
    MpfTemp cr(pr), ci(pr);
    if (mpf_set_str(cr, fcr, 10) != 0 || mpf_set_str(ci, fci, 10) != 0) {
        err_ = "unparsable fixed c";
        return MBX_E_INVALID;
    }
    mpf_set(scale_, scale);
    {
        MpfTemp dw(pr), dh(pr);
        mpf_set_ui(dw, 2);
        mpf_div(dw, dw, scale);
        mpf_set(dh, dw);
        mpf_mul_ui(dh, dh, rows);
        mpf_div_ui(dh, dh, W_);
        mpf_sub(c0_re_, z_re, dw);
        mpf_sub(c0_im_, z_im, dh);
        mpf_mul_ui(dx_, dw, 2);
        mpf_div_ui(dx_, dx_, W_ - 1);
        mpf_mul_ui(dy_, dh, 2);
        mpf_div_ui(dy_, dy_, rows - 1);
        if (row_base != 0) {
            mpf_mul_ui(dw, dy_, (unsigned long)row_base);
            mpf_add(c0_im_, c0_im_, dw);
        }
    }
    JuliaParams p;
    p.g = geom();
    p.z0r = mpf_ld(c0_re_);
    p.z0i = mpf_ld(c0_im_);
    p.dx = mpf_ld(dx_);
    p.dy = mpf_ld(dy_);
    p.cr = mpf_ld(cr);
    p.ci = mpf_ld(ci);
    const int n = W_ * H_;
    cudaMemsetAsync(dctr_, 0, sizeof(Counters), st_);
    DeviceFrame f = frame_view();
    const double t0 = now_ms();
    cudaEventRecord(ev0_, st_);
    cudaError_t e = launch_julia(f, p, std::min((n + 127) / 128, nsm_ * 8), 128, st_);
    cudaEventRecord(ev1_, st_);
    ++stats_.kernel_launches;
    ++stats_.passes;
    if (e != cudaSuccess) return fail_cuda("julia launch", e);
    copy_async(hctr_, dctr_, sizeof(Counters), cudaMemcpyDeviceToHost);
    e = cudaStreamSynchronize(st_);
    stats_.kernel_ms += now_ms() - t0;
    if (e != cudaSuccess) return fail_cuda("julia pass", e);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    stats_.pass_gpu_ms += ms;
    stats_.steps += (long long)hctr_->steps;
    stats_.effective_iterations += (long long)hctr_->effective_iters;
    stats_.interior += (int)hctr_->interior;
    stats_.samples += n;
    return MBX_OK;
}

// Shallow frames (scale <= 1e6, mp.cpp:1444-1519) and their SS sub-samples.
int Engine::render_shallow(volatile float* progress) {
    ShallowParams p;
    p.g = geom();
    p.c0r = mpf_ld(c0_re_);
    p.c0i = mpf_ld(c0_im_);
    p.dx = mpf_ld(dx_);
    p.dy = mpf_ld(dy_);
    p.simd_semantics = (cm_ & (8 | 16 | 32 | 64)) ? 0 : 1; // SAC, the normal map, traps and the DE overlay take the scalar path (mp.cpp:1455-1459)
    PixelSet g;
    g.keys = nullptr;
    g.grid_w = W_;
    g.grid_h = H_;
    g.grid_step = 1;
    g.skip_i = g.skip_j = -1;
    g.n = W_ * H_;
    if (!ensure(ddone_, g.n)) return MBX_E_NOMEM;
    cudaMemsetAsync(dctr_, 0, sizeof(Counters), st_);
    DeviceFrame f = frame_view();
    f.px = g;
    const double t0 = now_ms();
    cudaError_t e = launch_shallow(f, p, std::min((g.n + 127) / 128, nsm_ * 8), 128, st_);
    ++stats_.kernel_launches;
    ++stats_.passes;
    if (e != cudaSuccess) return fail_cuda("shallow launch", e);
    copy_async(hctr_, dctr_, sizeof(Counters), cudaMemcpyDeviceToHost);
    e = cudaStreamSynchronize(st_);
    stats_.kernel_ms += now_ms() - t0;
    if (e != cudaSuccess) return fail_cuda("shallow pass", e);
    stats_.steps += (long long)hctr_->steps;
    stats_.effective_iterations += (long long)hctr_->effective_iters;
    stats_.interior += (int)hctr_->interior;
    stats_.samples += g.n;
    if (progress) *progress = 0.9f;
    if (!((SUB_ > 1) && (cm_ & 1))) return MBX_OK;
    return supersample(0);
}

int Engine::shallow_samples(const std::vector<uint64_t>& samples) {
    const int n = (int)samples.size();
    if (!ensure(dkeys_, n) || !ensure(ddone_, n)) return MBX_E_NOMEM;
    copy_async(dkeys_.p, samples.data(), sizeof(uint64_t) * n, cudaMemcpyHostToDevice);
    ShallowParams p;
    p.g = geom();
    p.g.deovl = 0; // sub-samples carry the smooth/EDE value only (mp.cpp:1936-1967)
    p.g.normal = 0;
    // Up to 128 sub-samples per pixel take the reference's lane kernel, which
    // has no stripe average (a SAC frame's sub-samples take the scalar path)
    // and no orbit traps (a trap frame's sub-samples get the smooth count).
    if (!(cm_ & 8) && (cm_ & 32) && SUB_ * SUB_ <= 128) p.g.oc = 0;
    p.c0r = mpf_ld(c0_re_);
    p.c0i = mpf_ld(c0_im_);
    p.dx = mpf_ld(dx_);
    p.dy = mpf_ld(dy_);
    p.simd_semantics = (SUB_ * SUB_ <= 128) ? 1 : 0;
    PixelSet g;
    g.keys = dkeys_.p;
    g.n = n;
    g.grid_w = g.grid_h = g.grid_step = 1;
    g.skip_i = g.skip_j = -1;
    cudaMemsetAsync(dctr_, 0, sizeof(Counters), st_);
    DeviceFrame f = frame_view();
    f.px = g;
    const double t0 = now_ms();
    cudaError_t e = launch_shallow(f, p, std::min((n + 127) / 128, nsm_ * 8), 128, st_);
    ++stats_.kernel_launches;
    ++stats_.passes;
    if (e != cudaSuccess) return fail_cuda("shallow ss launch", e);
    copy_async(hctr_, dctr_, sizeof(Counters), cudaMemcpyDeviceToHost);
    e = cudaStreamSynchronize(st_);
    stats_.kernel_ms += now_ms() - t0;
    if (e != cudaSuccess) return fail_cuda("shallow ss pass", e);
    stats_.steps += (long long)hctr_->steps;
    stats_.effective_iterations += (long long)hctr_->effective_iters;
    stats_.interior += (int)hctr_->interior;
    stats_.samples += n;
    return MBX_OK;
}

} // namespace mbx

namespace mbx {

// findNucleus for an arbitrary disk (mp.cpp:1072-1107) plus the minibrot size
// estimate of nucleusSizeMag (mp.cpp:1195-1219) evaluated on the nucleus orbit.
int find_nucleus_disk(const char* cre, const char* cim, const char* radius, int maxp, int prec, std::string& nre, std::string& nim, double* size_log10) {
    mpf_set_default_prec((mp_bitcnt_t)prec);
    MpfTemp cr(prec), ci(prec), r(prec), nr(prec), ni(prec), dr(prec), di(prec), dist(prec);
    if (mpf_set_str(cr, cre, 10) || mpf_set_str(ci, cim, 10) || mpf_set_str(r, radius, 10)) return -1;
    int p = ball_period(cr, ci, r, maxp, prec, nullptr);
    if (p <= 0) return 0;
    mpf_set(nr, cr);
    mpf_set(ni, ci);
    if (!newton_nucleus(nr, ni, p, prec, 200)) return 0;
    mpf_sub(dr, nr, cr);
    mpf_sub(di, ni, ci);
    mpf_mul(dr, dr, dr);
    mpf_mul(di, di, di);
    mpf_add(dist, dr, di);
    mpf_sqrt(dist, dist);
    if (mpf_cmp(dist, r) > 0) return 0;
    // Size: l = prod 2 z_k, b = 1 + sum 1/l_k over k = 1..p-1, |size| = 1/(|b| |l|^2).
    MpfTemp zr(prec), zi(prec), s1(prec), s2(prec), s3(prec);
    mpf_set_ui(zr, 0);
    mpf_set_ui(zi, 0);
    FE lr = fe_make(1.0, 0), li = fe_make(0.0, 0), br = fe_make(1.0, 0), bi = fe_make(0.0, 0);
    for (int k = 1; k < p; ++k) {
        sqadd(zr, zi, nr, ni, s1, s2, s3);
        FE xr = mpf_fe(zr), xi = mpf_fe(zi);
        FE tr = fe_scale2(fe_sub(fe_mul(xr, lr), fe_mul(xi, li)), 1);
        FE ti = fe_scale2(fe_add(fe_mul(xr, li), fe_mul(xi, lr)), 1);
        lr = tr;
        li = ti;
        FE l2 = fe_add(fe_mul(lr, lr), fe_mul(li, li));
        if (l2.m == 0.0) continue;
        br = fe_add(br, fe_div(lr, l2));
        bi = fe_sub(bi, fe_div(li, l2));
    }
    FE lmag = fe_sqrt(fe_add(fe_mul(lr, lr), fe_mul(li, li)));
    FE bmag = fe_sqrt(fe_add(fe_mul(br, br), fe_mul(bi, bi)));
    FE denom = fe_mul(bmag, fe_mul(lmag, lmag));
    if (size_log10) *size_log10 = denom.m == 0.0 ? 0.0 : -(std::log10(std::fabs(denom.m)) + (double)denom.e * std::log10(2.0));
    auto to_str = [&](mpf_ptr v) {
        mp_exp_t e;
        char* d = mpf_get_str(nullptr, &e, 10, 0, v);
        std::string s(d);
        free(d);
        bool neg = !s.empty() && s[0] == '-';
        if (neg) s.erase(0, 1);
        std::string out = neg ? "-0." : "0.";
        if (e < 0) out += std::string((size_t)(-e), '0');
        else if (e > 0) {
            out = (neg ? "-" : "") + s.substr(0, std::min<size_t>(s.size(), (size_t)e));
            if ((size_t)e > s.size()) out += std::string((size_t)e - s.size(), '0');
            s = s.size() > (size_t)e ? s.substr((size_t)e) : "";
            out += ".";
        }
        out += s.empty() ? "0" : s;
        return out;
    };
    nre = to_str(nr);
    nim = to_str(ni);
    return p;
}

} // namespace mbx

namespace mbx {

void Engine::save_cache(int ref_it) {
    RefCache& c = cache_;
    c.key = frame_key_;
    c.use_floatexp = use_floatexp_;
    c.use_bla = use_bla_;
    c.ref_subpixel = ref_subpixel_;
    c.ref_virtual = ref_virtual_;
    c.fe_cutoff_sensitive = fe_cutoff_sensitive_;
    c.ref_value_pending = ref_value_pending_;
    c.ref_period = ref_period_;
    memcpy(c.ref, ref_, sizeof(ref_));
    c.orbit_len = orbit_len_;
    c.sa_order = sa_order_;
    c.sa_it = sa_it_;
    c.ref_it = ref_it;
    c.dc_xoff = dc_xoff_;
    c.dc_yoff = dc_yoff_;
    c.reference_length = stats_.reference_length;
    c.ref_x = ref_x_;
    c.ref_y = ref_y_;
    c.ref_frac_re = ref_frac_re_;
    c.ref_frac_im = ref_frac_im_;
    for (int q = 0; q < kSaTerms; ++q) {
        c.A[q] = sa_A_[q];
        c.B[q] = sa_B_[q];
    }
    c.delta = sa_delta_;
    c.bla = bla_;
    c.dxfe = dxfe_;
    c.dyfe = dyfe_;
    c.ref_value = ref_value_;
    c.ref_n = ref_n_;
    c.valid = true;
}

bool Engine::restore_cache(int* ref_it) {
    const RefCache& c = cache_;
    if (!c.valid) return false;
    use_floatexp_ = c.use_floatexp;
    use_bla_ = c.use_bla;
    ref_subpixel_ = c.ref_subpixel;
    ref_virtual_ = c.ref_virtual;
    fe_cutoff_sensitive_ = c.fe_cutoff_sensitive;
    ref_value_pending_ = c.ref_value_pending;
    ref_period_ = c.ref_period;
    memcpy(ref_, c.ref, sizeof(ref_));
    orbit_len_ = c.orbit_len;
    sa_order_ = c.sa_order;
    sa_it_ = c.sa_it;
    dc_xoff_ = c.dc_xoff;
    dc_yoff_ = c.dc_yoff;
    stats_.reference_length = c.reference_length;
    ref_x_ = c.ref_x;
    ref_y_ = c.ref_y;
    ref_frac_re_ = c.ref_frac_re;
    ref_frac_im_ = c.ref_frac_im;
    for (int q = 0; q < kSaTerms; ++q) {
        sa_A_[q] = c.A[q];
        sa_B_[q] = c.B[q];
    }
    sa_delta_ = c.delta;
    bla_ = c.bla;
    dxfe_ = c.dxfe;
    dyfe_ = c.dyfe;
    ref_value_ = c.ref_value;
    ref_n_ = c.ref_n;
    *ref_it = c.ref_it;
    return true;
}

} // namespace mbx

// Mixed-precision floatexp pass. The bulk delta iteration runs in FP32 on a
// rescaled delta dz = S * w, with S an FP32-mantissa floatexp (float m, int e)
// and w an O(1) float2; the reference orbit is read as float2 from shared
// memory (staged once per block by a TMA bulk copy) or from L1/L2 when it does
// not fit. On GB300 one FP64 instruction costs as much issue time as ~60 FP32
// ones, so FP64 (and FP64-mantissa floatexp) is used only on rare events:
//   * BLA skips: coefficients and validity radii come from the FP64 table;
//     candidates are screened on integer exponents, decided and applied in FP64;
//   * rebasing near |Z + dz| ~ |dz|: screened in FP32, decided in FP64-floatexp;
//   * escape: screened in FP32 with a relative margin, decided and the smooth
//     value computed from an FP64 reconstruction of z;
//   * interior detection: FP32 screen, FP64 at close returns and saves;
//   * steps where the orbit is below FP32's range (exact floatexp step).
// Semantics follow the reference's rescaled loop (mp.cpp:3287-3618); results
// are validated against the arbitrary-precision oracle, not bit-compared.
#include <cuda_runtime.h>

#include "engine.h"

namespace mbx {

namespace {

constexpr double kLn2m = 0x1.62e42fefa39efp-1;

__device__ __forceinline__ bool mcancelled(const DeviceFrame& f) { return f.cancel && *f.cancel; }

// ---- FP32-mantissa floatexp: m in [0.5,1) (or 0), e int -------------------
struct F32E {
    float m;
    int e;
};
__device__ __forceinline__ F32E f32e_norm(float m, int e) {
    if (m == 0.0f) return F32E{0.0f, 0};
    unsigned b = __float_as_uint(m);
    int ex = (int)((b >> 23) & 0xff);
    if (ex == 0) { // subnormal mantissa: scale up exactly
        m *= 16777216.0f;
        b = __float_as_uint(m);
        ex = (int)((b >> 23) & 0xff) - 24;
    }
    return F32E{__uint_as_float((b & 0x807fffffu) | (126u << 23)), e + ex - 126};
}
__device__ __forceinline__ F32E f32e_mulf(F32E a, float b) { return f32e_norm(a.m * b, a.e); }
// a * 2^k as float, flushing below FP32's normal range to zero.
__device__ __forceinline__ float ldexpf_ftz(float a, int k) {
    if (a == 0.0f) return 0.0f;
    unsigned b = __float_as_uint(a);
    int ex = (int)((b >> 23) & 0xff) + k;
    if (ex <= 0) return 0.0f;
    if (ex >= 255) return __uint_as_float((b & 0x80000000u) | 0x7f7fffffu);
    return __uint_as_float((b & 0x807fffffu) | ((unsigned)ex << 23));
}
__device__ __forceinline__ float f32e_to_float(F32E a) { return ldexpf_ftz(a.m, a.e); }
__device__ __forceinline__ F32E f32e_from_fe(FE a) {
    if (a.m == 0.0) return F32E{0.0f, 0};
    return f32e_norm((float)a.m, (int)a.e);
}
__device__ __forceinline__ FE fe_from_f32e(F32E a) { return a.m == 0.0f ? fe_make(0.0, 0) : fe_make((double)a.m, (int64_t)a.e); }
// x / S for x, S in F32E, as float.
__device__ __forceinline__ float f32e_ratio(F32E x, F32E s) {
    if (x.m == 0.0f) return 0.0f;
    return ldexpf_ftz(__fdividef(x.m, s.m), x.e - s.e);
}
__device__ __forceinline__ int float_exp(float x) { return (int)((__float_as_uint(x) >> 23) & 0xff) - 127; }

// Exact floatexp step for orbit entries below FP32's range (mp.cpp:2794-2835).
__device__ void exact_step(FE Xr, FE Xi, FE dcr, FE dci, FE& S, double& wr, double& wi) {
    const double sm = S.m, sm2 = sm * sm;
    const int64_t se = S.e;
    const int64_t NONE = (int64_t)0x8000000000000000ll;
    int64_t e = NONE;
    const bool has_w = wr != 0.0 || wi != 0.0;
    if (has_w && Xr.m != 0.0) e = max(e, Xr.e + se);
    if (has_w && Xi.m != 0.0) e = max(e, Xi.e + se);
    if (has_w) e = max(e, se + se);
    if (dcr.m != 0.0) e = max(e, dcr.e);
    if (dci.m != 0.0) e = max(e, dci.e);
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

struct MixedState {
    F32E S;        // delta scale
    float wr, wi;  // delta unit
    float s;       // S as float (0 below FP32's range)
    float dr, di;  // dc / S
    F32E dcr, dci; // dc
};

__device__ __forceinline__ void refresh(MixedState& st) {
    st.s = f32e_to_float(st.S);
    st.dr = f32e_ratio(st.dcr, st.S);
    st.di = f32e_ratio(st.dci, st.S);
}

// FP32-floatexp copy of the FP64 BLA table: A and B as float2 mantissas with
// one exponent each, the radius^2 as float mantissa + exponent. Built once per
// reference from the FP64 table (k_bla_to_f32).
__device__ __forceinline__ int dexp_of(double x) { // x = m 2^e, m in [0.5,1)
    int e;
    (void)xfrexp(x, &e);
    return e;
}

__global__ void k_bla_to_f32(const double* r2, const double4* ab, Bla32* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double4 c = ab[i];
    Bla32 b;
    double amax = fmax(fabs(c.x), fabs(c.y)), bmax = fmax(fabs(c.z), fabs(c.w));
    b.ea = amax > 0 ? dexp_of(amax) : 0;
    b.eb = bmax > 0 ? dexp_of(bmax) : 0;
    b.ab = make_float4((float)xldexp(c.x, -b.ea), (float)xldexp(c.y, -b.ea), (float)xldexp(c.z, -b.eb), (float)xldexp(c.w, -b.eb));
    double v = r2[i];
    if (v > 0.0) {
        int e;
        double m = xfrexp(v, &e);
        b.r2m = (float)m;
        b.r2e = e;
        if (b.r2m >= 1.0f) { // mantissa rounded up to 1.0
            b.r2m = 0.5f;
            b.r2e += 1;
        }
    } else {
        b.r2m = 0.0f;
        b.r2e = 0;
    }
    out[i] = b;
}

// BLA skip in FP32-floatexp (mp.cpp:2883-2970 semantics; coefficients and
// radii constructed in FP64). dz = S w, dc = dcm 2^dce (shared exponent).
__device__ int mixed_bla32(const BlaView& b, const Bla32* t, const float2* orb, bool periodic, int s, F32E& S, float& wr, float& wi, float2 dcm, int dce, float ESC2lo, int mx_ref_it) {
    int maxp = b.nlev - 1;
    int startp = (s == 1) ? maxp : __ffs(s - 1) - 1;
    if (startp > maxp) startp = maxp;
    if (startp < b.minlevel) return 0;
    const float wm2 = wr * wr + wi * wi;
    if (wm2 == 0.0f) return 0;
    const F32E dz2 = f32e_norm(S.m * S.m * wm2, 2 * S.e);
    for (int p = startp; p >= b.minlevel; --p) {
        int i = (s - 1) >> p;
        if (i >= b.size[p]) continue;
        const Bla32 e = t[b.off[p] + i];
        if (e.r2m == 0.0f) continue;
        if (!(dz2.e < e.r2e || (dz2.e == e.r2e && dz2.m < e.r2m))) continue; // |dz|^2 < r2
        const int l = 1 << p;
        const int land = s + l;
        if (land >= mx_ref_it - 1) continue;
        // A dz + B dc = A (S.m w) 2^(ea + S.e) + B dcm 2^(eb + dce)
        const float swr = S.m * wr, swi = S.m * wi;
        float t1r = e.ab.x * swr - e.ab.y * swi, t1i = e.ab.x * swi + e.ab.y * swr;
        float t2r = e.ab.z * dcm.x - e.ab.w * dcm.y, t2i = e.ab.z * dcm.y + e.ab.w * dcm.x;
        const int E1 = e.ea + S.e, E2 = e.eb + dce;
        const int E = max(E1, E2);
        const float vr = ldexpf_ftz(t1r, E1 - E) + ldexpf_ftz(t2r, E2 - E);
        const float vi = ldexpf_ftz(t1i, E1 - E) + ldexpf_ftz(t2i, E2 - E);
        const float v2 = vr * vr + vi * vi;
        // Never skip past an escape: z = X_land + dz' (conservative FP32 test).
        const float2 zl = orb[land];
        const float zr = zl.x + ldexpf_ftz(vr, E), zi = zl.y + ldexpf_ftz(vi, E);
        if (zr * zr + zi * zi > ESC2lo) return 0;
        if (v2 == 0.0f) {
            if (!periodic) return 0;
            S = F32E{0.5f, 1};
            wr = wi = 0.0f;
        } else {
            const float vm = sqrtf(v2), inv = 1.0f / vm;
            S = f32e_norm(vm, E);
            wr = vr * inv;
            wi = vi * inv;
        }
        return l;
    }
    return 0;
}

// BLA skip (mp.cpp:2883-2970 semantics): levels screened on integer exponents
// of |dz|^2 against the precomputed exponents of r2; decided and applied in FP64.
__device__ int mixed_bla(const BlaView& b, const int16_t* r2e, const double2* Z, bool periodic, int s, MixedState& st, FE dcr, FE dci, double ESC2, int mx_ref_it) {
    int maxp = b.nlev - 1;
    int startp = (s == 1) ? maxp : __ffs(s - 1) - 1;
    if (startp > maxp) startp = maxp;
    if (startp < b.minlevel) return 0;
    const float wm2 = st.wr * st.wr + st.wi * st.wi;
    if (wm2 == 0.0f) return 0;
    const int edz2 = 2 * st.S.e + float_exp(wm2) + 1; // |dz|^2 < 2^edz2
    for (int p = startp; p >= b.minlevel; --p) {
        int i = (s - 1) >> p;
        if (i >= b.size[p]) continue;
        const int er = r2e[b.off[p] + i];      // r2 >= 2^(er-1), or -32768 when r2 <= 0
        if (er == -32768 || edz2 - 2 > er) continue; // clearly too large (or invalid)
        const double r2 = b.r2[b.off[p] + i];
        const double wr = st.wr, wi = st.wi;
        const FE S = fe_from_f32e(st.S);
        FE dz2 = fe_mul(fe_mul(S, S), fe_from(wr * wr + wi * wi));
        if (!fe_abs_less(dz2, fe_from(r2))) continue;
        int l = 1 << p;
        int land = s + l;
        if (land >= mx_ref_it - 1) continue;
        const double dr = fe_to_double(fe_div(dcr, S)), di = fe_to_double(fe_div(dci, S));
        double4 bc = b.ab[b.off[p] + i];
        double nwr = (bc.x * wr - bc.y * wi) + (bc.z * dr - bc.w * di);
        double nwi = (bc.x * wi + bc.y * wr) + (bc.z * di + bc.w * dr);
        if (!(fabs(nwr) < 1e150 && fabs(nwi) < 1e150)) return 0;
        double2 zl = Z[land];
        double fr = zl.x + fe_to_double(fe_mul_d(S, nwr));
        double fi = zl.y + fe_to_double(fe_mul_d(S, nwi));
        if (fr * fr + fi * fi > ESC2) return 0;
        double wm2d = nwr * nwr + nwi * nwi;
        if (wm2d == 0.0) {
            if (!periodic) return 0;
            st.S = F32E{0.5f, 1};
            st.wr = st.wi = 0.0f;
        } else {
            double wmag = sqrt(wm2d);
            st.S = f32e_from_fe(fe_mul(S, fe_from(wmag)));
            st.wr = (float)(nwr / wmag);
            st.wi = (float)(nwi / wmag);
        }
        return l;
    }
    return 0;
}

// Stage the FP32 orbit into shared memory: bulk TMA copies (cp.async.bulk,
// global -> shared) completing on one mbarrier; the wait is bounded.
__device__ bool stage_orbit(float2* smem, const float2* g, int entries, unsigned long long* mbar) {
    const unsigned bytes = ((unsigned)entries * 8u + 15u) & ~15u;
    const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
        const unsigned chunk = 1u << 15;
        for (unsigned off = 0; off < bytes; off += chunk) {
            unsigned n = bytes - off < chunk ? bytes - off : chunk;
            unsigned dst = (unsigned)__cvta_generic_to_shared((char*)smem + off);
            const char* src = (const char*)g + off;
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst), "l"(src), "r"(n), "r"(mb) : "memory");
        }
    }
    __syncthreads();
    unsigned done = 0;
    for (int spin = 0; spin < (1 << 22) && !done; ++spin) {
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mb)
            : "memory");
    }
    return done != 0;
}

// Per-lane state of the mixed pass.
struct Lane {
    int i, oidx;         // pass entry, output index
    double dpx, dpy;     // sample offset from the reference in pixels (for rare exact steps)
    F32E S;              // delta scale
    float wr, wi, s, dr, di;
    float2 dcm;          // dc mantissas with shared exponent dce
    int dce;
    int m, iter, rm;
    float2 Xc;           // X_m
    // interior detection
    float zsr_f, zsi_f, conf_D2, swr, swi;
    double zsr, zsi, conf_zr, conf_zi;
    F32E sS;
    int save_iter, period_win, conf_P, conf_next, conf_count, conf_giveup, sidx, save_iter2, twin2;
};

__device__ __forceinline__ void lane_refresh(Lane& L) {
    L.s = f32e_to_float(L.S);
    const float inv = __fdividef(1.0f, L.S.m);
    L.dr = ldexpf_ftz(L.dcm.x * inv, L.dce - L.S.e);
    L.di = ldexpf_ftz(L.dcm.y * inv, L.dce - L.S.e);
}

// dz = S w with S <- |v| 2^e and w <- v / |v| for an FP32 vector v scaled by 2^e.
__device__ __forceinline__ void lane_set_delta(Lane& L, float vr, float vi, int e) {
    const float v2 = vr * vr + vi * vi;
    if (v2 == 0.0f) {
        L.S = F32E{0.5f, 1};
        L.wr = L.wi = 0.0f;
        return;
    }
    const float vm = sqrtf(v2), inv = 1.0f / vm;
    L.S = f32e_norm(vm, e);
    L.wr = vr * inv;
    L.wi = vi * inv;
}

__device__ __forceinline__ FE lane_dc_re(const MixedParams& p, const Lane& L) { return fe_mul_d(p.dxfe, L.dpx); }
__device__ __forceinline__ FE lane_dc_im(const MixedParams& p, const Lane& L) { return fe_mul_d(p.dyfe, L.dpy); }

__device__ void lane_setup(Lane& L, int i, const DeviceFrame& f, const MixedParams& p, const F32E dxf, const F32E dyf, const float2* orb) {
    const FrameGeom& g = p.g;
    int arr[4];
    if (f.px.keys) {
        key_unpack(f.px.keys[i], arr);
    } else {
        int cols = (f.px.grid_w + f.px.grid_step - 1) / f.px.grid_step;
        int q = i;
        if (f.px.skip_i >= 0) {
            int sq = (f.px.skip_i / f.px.grid_step) * cols + f.px.skip_j / f.px.grid_step;
            if (q >= sq) ++q;
        }
        arr[0] = (q / cols) * f.px.grid_step;
        arr[1] = (q % cols) * f.px.grid_step;
        arr[2] = arr[3] = 0;
    }
    L.i = i;
    L.oidx = (arr[0] * g.sub + g.sub / 2 + arr[2]) * g.W * g.sub + (arr[1] * g.sub + g.sub / 2 + arr[3]);
    L.dpx = arr[1] + (double)arr[3] / g.sub - p.ref_x;
    L.dpy = arr[0] + (double)arr[2] / g.sub - p.ref_y;
    // dc in FP32 floatexp with one shared exponent.
    const F32E cr = f32e_mulf(dxf, (float)L.dpx), ci = f32e_mulf(dyf, (float)L.dpy);
    int e = (cr.m != 0.0f) ? cr.e : ((ci.m != 0.0f) ? ci.e : 0);
    if (cr.m != 0.0f && ci.m != 0.0f) e = max(cr.e, ci.e);
    L.dce = e;
    L.dcm = make_float2(ldexpf_ftz(cr.m, cr.e - e), ldexpf_ftz(ci.m, ci.e - e));
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
    L.swr = L.swi = 3e38f;
    L.sS = F32E{2.0f, 0};
    L.sidx = -2;
    L.save_iter2 = 1;
    L.twin2 = 1;
}

// z = X_m + S w in FP64 (rare decisions).
__device__ __forceinline__ void lane_z_double(const Lane& L, const double2* Zd, double& zr, double& zi) {
    const double2 Xd = L.m ? Zd[L.rm] : make_double2(0.0, 0.0);
    const double sd = xldexp((double)L.S.m, L.S.e);
    zr = Xd.x + sd * (double)L.wr;
    zi = Xd.y + sd * (double)L.wi;
}

// Advance one lane by up to `budget` iterations. Returns 0 running, 1 escaped,
// 2 interior, 4 cancelled; nesc / zrad_out are set on escape.
__device__ int lane_run(Lane& L, int budget, const DeviceFrame& f, const MixedParams& p, const Bla32* bla32, const float2* orb, int reflen, float ESC2f, int blamask, float& zrad_out, unsigned long long& n_steps, unsigned long long& n_bla, unsigned long long& n_skip, unsigned long long& n_rebase) {
    const FrameGeom& g = p.g;
    const int per = p.per;
    const double2* Zd = f.orbit.Z;
    const FE2* Zfe = f.orbit.Zfe;
    const float ESC2hi = ESC2f * 1.000002f, ESC2lo = ESC2f * 0.999998f;
    for (int b = 0; b < budget; ++b) {
        if (L.iter >= g.mxit) return 2;
        if (p.use_interior) {
            const int idxs = per ? L.rm : L.m;
            if (idxs == L.sidx && L.wr == L.swr && L.wi == L.swi && L.S.m == L.sS.m && L.S.e == L.sS.e) return 2;
            if (L.iter - L.save_iter2 >= L.twin2) {
                L.swr = L.wr;
                L.swi = L.wi;
                L.sS = L.S;
                L.sidx = idxs;
                L.save_iter2 = L.iter;
                L.twin2 += L.twin2;
            }
        }
        if (bla32 && L.m >= 2 && ((L.rm - 1) & blamask) == 0) {
            const int skip = mixed_bla32(f.bla, bla32, orb, per > 0, L.rm, L.S, L.wr, L.wi, L.dcm, L.dce, ESC2lo, per ? per : reflen);
            if (skip > 0) {
                ++n_bla;
                n_skip += skip;
                L.m += skip;
                L.iter += skip;
                L.rm += skip;
                if (per && L.rm >= per) L.rm -= per;
                lane_refresh(L);
                L.Xc = orb[L.rm];
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
        // w' = (2 X_m + s w) w + d
        const bool tiny = L.m != 0 && fabsf(L.Xc.x) < 1e-30f && fabsf(L.Xc.y) < 1e-30f && (Zfe[L.rm].re.m != 0.0 || Zfe[L.rm].im.m != 0.0);
        if (!tiny) {
            const float fR = 2.0f * L.Xc.x + L.s * L.wr;
            const float fI = 2.0f * L.Xc.y + L.s * L.wi;
            const float nwr = fR * L.wr - fI * L.wi + L.dr;
            const float nwi = fR * L.wi + fI * L.wr + L.di;
            L.wr = nwr;
            L.wi = nwi;
        } else {
            double wr = L.wr, wi = L.wi;
            FE S = fe_from_f32e(L.S);
            exact_step(Zfe[L.rm].re, Zfe[L.rm].im, lane_dc_re(p, L), lane_dc_im(p, L), S, wr, wi);
            const double mg = sqrt(wr * wr + wi * wi);
            L.S = f32e_from_fe(S);
            L.wr = (float)wr;
            L.wi = (float)wi;
            (void)mg;
            lane_refresh(L);
        }
        ++L.m;
        ++L.iter;
        ++L.rm;
        if (per && L.rm == per) L.rm = 0;
        L.Xc = orb[L.rm];
        const float zr = L.Xc.x + L.s * L.wr, zi = L.Xc.y + L.s * L.wi;
        const float zrad = zr * zr + zi * zi;
        if (zrad > ESC2lo) {
            if (zrad > ESC2hi) {
                zrad_out = zrad;
                return 1;
            }
            double zdr, zdi;
            lane_z_double(L, Zd, zdr, zdi);
            const double zr2 = zdr * zdr + zdi * zdi;
            if (zr2 > g.ESC2) {
                zrad_out = (float)zr2;
                return 1;
            }
        }
        if (p.use_interior) {
            if (L.conf_P > 0) {
                L.conf_D2 *= 4.0f * zrad;
                if (L.conf_D2 > 1e18f) L.conf_D2 = 1e18f;
                if (L.iter >= L.conf_next) {
                    double zdr, zdi;
                    lane_z_double(L, Zd, zdr, zdi);
                    const double qr = zdr - L.conf_zr, qi = zdi - L.conf_zi;
                    if (qr * qr + qi * qi < p.interior_eps2 * (zdr * zdr + zdi * zdi) && L.conf_D2 < 1.0f) {
                        if (++L.conf_count >= p.interior_confirm) return 2;
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
                const float qr = zr - L.zsr_f, qi = zi - L.zsi_f;
                const bool maybe = qr * qr + qi * qi < 1e-11f * zrad;
                const bool save = L.iter - L.save_iter >= L.period_win;
                if (maybe || save) {
                    double zdr, zdi;
                    lane_z_double(L, Zd, zdr, zdi);
                    if (maybe) {
                        const double dqr = zdr - L.zsr, dqi = zdi - L.zsi;
                        if (dqr * dqr + dqi * dqi < p.interior_eps2 * (zdr * zdr + zdi * zdi)) {
                            L.conf_P = max(L.iter - L.save_iter, 1);
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
                        L.zsr_f = zr;
                        L.zsi_f = zi;
                        L.save_iter = L.iter;
                        L.period_win += L.period_win;
                    }
                }
            }
        }
        // keep |w| ~ 1 (rescale window [1/wmax2, wmax2], autotuned)
        const float wm2 = L.wr * L.wr + L.wi * L.wi;
        if (wm2 > p.wmax2 || (wm2 < p.wmin2 && wm2 > 0.0f)) {
            const float wmag = sqrtf(wm2), inv = 1.0f / wmag;
            L.S = f32e_mulf(L.S, wmag);
            L.wr *= inv;
            L.wi *= inv;
            lane_refresh(L);
        }
        // Rebase (mp.cpp:3584-3615): |z|^2 < |dz|^2 decided on FP32 floatexp
        // with a 1e-4 margin; FP64 floatexp inside the margin, for strong
        // cancellation in X + dz, and at the end of the reference.
        const float w2 = L.wr * L.wr + L.wi * L.wi;
        const F32E dz2 = f32e_norm(L.S.m * L.S.m * w2, 2 * L.S.e);
        int decide = 0; // 0 none, 1 rebase in FP32, 2 FP64 test
        if (!per && L.m >= reflen) decide = 2;
        else if (dz2.m != 0.0f) {
            if (zrad == 0.0f) decide = 2;
            else {
                const F32E z2 = f32e_norm(zrad, 0);
                const float q = ldexpf_ftz(__fdividef(z2.m, dz2.m), max(-120, min(120, z2.e - dz2.e)));
                if (q < 0.9999f) decide = (zrad > 0.25f * (L.Xc.x * L.Xc.x + L.Xc.y * L.Xc.y) && L.s != 0.0f) ? 1 : 2;
                else if (q < 1.0001f) decide = 2;
            }
        }
        if (decide == 1) {
            lane_set_delta(L, zr, zi, 0);
            lane_refresh(L);
            L.m = 0;
            L.rm = -1;
            L.Xc = make_float2(0.0f, 0.0f);
            ++n_rebase;
        } else if (decide == 2) {
            const FE S = fe_from_f32e(L.S);
            FE Xmr = L.m ? Zfe[L.rm].re : fe_make(0.0, 0);
            FE Xmi = L.m ? Zfe[L.rm].im : fe_make(0.0, 0);
            FE Swr = fe_mul_d(S, (double)L.wr), Swi = fe_mul_d(S, (double)L.wi);
            FE zrfe = fe_add(Xmr, Swr), zife = fe_add(Xmi, Swi);
            FE zradfe = fe_add(fe_mul(zrfe, zrfe), fe_mul(zife, zife));
            FE dzfe = fe_add(fe_mul(Swr, Swr), fe_mul(Swi, Swi));
            if ((!per && L.m >= reflen) || fe_abs_less(zradfe, dzfe)) {
                FE Snew = fe_sqrt(zradfe);
                if (Snew.m == 0.0) {
                    L.wr = L.wi = 0.0f;
                } else {
                    L.S = f32e_from_fe(Snew);
                    L.wr = (float)fe_to_double(fe_div(zrfe, Snew));
                    L.wi = (float)fe_to_double(fe_div(zife, Snew));
                    lane_refresh(L);
                }
                L.m = 0;
                L.rm = -1;
                L.Xc = make_float2(0.0f, 0.0f);
                ++n_rebase;
            }
        }
    }
    return 0;
}

template <int MINB>
__global__ void __launch_bounds__(256, MINB) k_mixed_pass(DeviceFrame f, MixedParams p, const int16_t* r2e, const Bla32* bla32) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ unsigned long long mbar;
    __shared__ int stage_ok;
    (void)r2e;
    const FrameGeom& g = p.g;
    const float2* orb = p.Zf;
    if (p.orbit_in_smem) {
        float2* so = reinterpret_cast<float2*>(smem_raw);
        bool ok = stage_orbit(so, p.Zf, p.smem_entries, &mbar);
        if (threadIdx.x == 0) stage_ok = ok ? 1 : 0;
        __syncthreads();
        if (!stage_ok) {
            if (threadIdx.x == 0) atomicAdd(&f.ctr->rescales, 1ull); // staging timed out: this block leaves its share to the others
            return;
        }
        orb = so;
    }
    const int reflen = p.mx_ref_it + 1;
    const float ESC2f = (float)g.ESC2;
    const int blamask = (1 << f.bla.minlevel) - 1;
    const Bla32* bt = f.bla.use ? bla32 : nullptr;
    const F32E dxf = f32e_from_fe(p.dxfe), dyf = f32e_from_fe(p.dyfe);
    const unsigned lane_id = threadIdx.x & 31;
    unsigned long long n_steps = 0, n_bla = 0, n_skip = 0, n_eff = 0, n_rebase = 0;
    unsigned int n_int = 0;
    Lane L;
    bool live = false, exhausted = false, stop = false;
    unsigned rounds = 0;
    for (;;) {
        // Warp-synchronous refill: every idle lane takes a new sample together,
        // so the per-sample setup runs once for all of them.
        const unsigned idle = __ballot_sync(0xffffffffu, !live);
        if (idle && !exhausted) {
            int base = 0;
            const int leader = __ffs(idle) - 1;
            if ((int)lane_id == leader) base = (int)atomicAdd(&f.ctr->next, (unsigned)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base >= f.px.n) exhausted = true;
            if (!live) {
                const int i = base + __popc(idle & ((1u << lane_id) - 1u));
                if (i < f.px.n && !stop) {
                    lane_setup(L, i, f, p, dxf, dyf, orb);
                    live = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, live) == 0) break;
        if (live) {
            float zrad = 0.0f;
            const int st = lane_run(L, 32, f, p, bt, orb, reflen, ESC2f, blamask, zrad, n_steps, n_bla, n_skip, n_rebase);
            if (st == 1) {
                // smooth value N - log2(log2|z|) in FP32 (the output is FP32)
                const float lg = log2f(zrad);
                f.out.iter[L.oidx] = (float)L.iter - log2f(0.5f * lg);
                if (f.out.escN) f.out.escN[L.oidx] = L.iter;
                f.out.done[L.i] = 1;
                n_eff += (unsigned long long)L.iter;
                live = false;
            } else if (st == 2) {
                f.out.iter[L.oidx] = -2.0f;
                if (f.out.escN) f.out.escN[L.oidx] = -1;
                f.out.done[L.i] = 1;
                n_eff += (unsigned long long)g.mxit;
                ++n_int;
                live = false;
            }
        }
        if (((++rounds & 255u) == 0) && mcancelled(f)) {
            stop = true;
            exhausted = true;
            live = false;
        }
    }
    atomicAdd(&f.ctr->steps, n_steps);
    atomicAdd(&f.ctr->bla_applies, n_bla);
    atomicAdd(&f.ctr->bla_skipped, n_skip);
    atomicAdd(&f.ctr->effective_iters, n_eff);
    atomicAdd(&f.ctr->rebases, n_rebase);
    atomicAdd(&f.ctr->interior, n_int);
}

__global__ void k_orbit_to_float(const double2* Z, float2* Zf, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) Zf[i] = make_float2((float)Z[i].x, (float)Z[i].y);
}

// Exponent of each BLA radius^2 (r2 in [2^(e-1), 2^e)), -32768 for r2 <= 0.
__global__ void k_bla_exponents(const double* r2, int16_t* e, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = r2[i];
    if (!(v > 0.0)) {
        e[i] = -32768;
        return;
    }
    int ex;
    (void)xfrexp(v, &ex);
    e[i] = (int16_t)max(-32767, min(32767, ex));
}

__global__ void k_fma_probe_f32(float* out, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = __fmaf_rn(x0, a, b); x1 = __fmaf_rn(x1, a, b); x2 = __fmaf_rn(x2, a, b); x3 = __fmaf_rn(x3, a, b);
        x4 = __fmaf_rn(x4, a, b); x5 = __fmaf_rn(x5, a, b); x6 = __fmaf_rn(x6, a, b); x7 = __fmaf_rn(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_fma_probe_f64(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = __fma_rn(x0, a, b); x1 = __fma_rn(x1, a, b); x2 = __fma_rn(x2, a, b); x3 = __fma_rn(x3, a, b);
        x4 = __fma_rn(x4, a, b); x5 = __fma_rn(x5, a, b); x6 = __fma_rn(x6, a, b); x7 = __fma_rn(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

} // namespace

int Engine::measure_fma_peak(int fp64, double* tflops) {
    const int blocks = nsm_ * 8, threads = 256;
    const int iters = fp64 ? 2000 : 40000;
    void* buf = nullptr;
    if (cudaMalloc(&buf, (size_t)blocks * threads * 8) != cudaSuccess) return MBX_E_NOMEM;
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(ev0_, st_);
        if (fp64) k_fma_probe_f64<<<blocks, threads, 0, st_>>>((double*)buf, iters, 0.999999, 1e-7);
        else k_fma_probe_f32<<<blocks, threads, 0, st_>>>((float*)buf, iters, 0.999999f, 1e-7f);
        cudaEventRecord(ev1_, st_);
        cudaError_t e = cudaEventSynchronize(ev1_);
        if (e != cudaSuccess) {
            cudaFree(buf);
            return fail_cuda("fma probe", e);
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, ev0_, ev1_);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaFree(buf);
    *tflops = 2.0 * 8.0 * (double)blocks * threads * iters / (best * 1e-3) / 1e12;
    return MBX_OK;
}

cudaError_t launch_mixed_pass(const DeviceFrame& f, const MixedParams& p, int blocks, int threads, size_t smem, cudaStream_t st) {
    (void)f;
    (void)p;
    (void)blocks;
    (void)threads;
    (void)smem;
    (void)st;
    return cudaErrorNotSupported; // launched through Engine::run_mixed_pass (needs the exponent table)
}

int Engine::prepare_mixed() {
    const int len = orbit_len_;
    if (!ensure(dZf_, (size_t)len + 4)) return MBX_E_NOMEM;
    k_orbit_to_float<<<(len + 255) / 256, 256, 0, st_>>>(dZ_.p, dZf_.p, len);
    ++stats_.kernel_launches;
    if (bla_.use && bla_.nlev > 0) {
        int n = bla_.off[bla_.nlev - 1] + bla_.size[bla_.nlev - 1];
        if (!ensure(dr2e_, (size_t)n)) return MBX_E_NOMEM;
        k_bla_exponents<<<(n + 255) / 256, 256, 0, st_>>>(dr2_.p, dr2e_.p, n);
        ++stats_.kernel_launches;
        if (!ensure(dbla32_, (size_t)n)) return MBX_E_NOMEM;
        k_bla_to_f32<<<(n + 255) / 256, 256, 0, st_>>>(dr2_.p, dab_.p, dbla32_.p, n);
        ++stats_.kernel_launches;
    }
    return cuda_ok("mixed preparation");
}

cudaError_t Engine::run_mixed_pass(const DeviceFrame& f) {
    MixedParams p;
    p.g = geom();
    p.dxfe = dxfe_;
    p.dyfe = dyfe_;
    p.ref_x = ref_x_;
    p.ref_y = ref_y_;
    p.per = ref_period_;
    p.mx_ref_it = ref_period_ > 0 ? ref_period_ : orbit_len_ - 1;
    p.use_interior = use_interior_ ? 1 : 0;
    p.interior_eps2 = interior_eps2_;
    p.interior_confirm = interior_confirm_;
    p.Zf = dZf_.p;
    p.Zsmall = nullptr;
    const size_t bytes = ((size_t)orbit_len_ * 8 + 15) & ~(size_t)15;
    p.orbit_in_smem = (bytes <= (size_t)smem_orbit_limit_) ? 1 : 0;
    p.smem_entries = orbit_len_;
    const int threads = mixed_threads_;
    const int blocks = std::max(1, std::min((f.px.n + threads - 1) / threads, nsm_ * mixed_blocks_per_sm_));
    const size_t smem = p.orbit_in_smem ? bytes : 0;
    p.wmax2 = mixed_wmax2_;
    p.wmin2 = 1.0f / mixed_wmax2_;
    DeviceFrame g = f;
    if (!(bla_.use && dr2e_.p)) g.bla.use = 0;
    const Bla32* bt = mixed_bla32_ ? dbla32_.p : nullptr;
    auto launch = [&](auto kern) -> cudaError_t {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        kern<<<blocks, threads, smem, st_>>>(g, p, dr2e_.p, bt);
        return cudaGetLastError();
    };
    if (mixed_blocks_per_sm_ >= 4) return launch(k_mixed_pass<4>);
    if (mixed_blocks_per_sm_ == 3) return launch(k_mixed_pass<3>);
    return launch(k_mixed_pass<2>);
    return cudaGetLastError();
}

} // namespace mbx

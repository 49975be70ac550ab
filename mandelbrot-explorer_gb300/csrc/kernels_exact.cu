// Exact-form CUDA passes of the perturbation renderer (compiled with
// -fmad=false so that every double operation below is the IEEE operation the
// reference executes, in the reference's order). Each kernel is persistent:
// every thread pulls sample indices from a global work counter, so lanes whose
// pixel finished are refilled immediately (the GPU form of the reference's
// AVX2 lane refill, mp.cpp:416-532) instead of idling behind slow lanes.
//
// Reference: cbotx/Mandelbrot-Explorer src/engine/mandel_perturbation.cpp
// ("mp.cpp"); the per-pixel semantics are those of its scalar loops.
#include "kernels.h"
#include "orbit_color.h"

namespace mbx {

static constexpr double kLn2 = 0x1.62e42fefa39efp-1; // log(2.0), correctly rounded

__device__ __forceinline__ int sample_index(const FrameGeom& g, const int* a) { // mp.cpp:4334-4340
    return (a[0] * g.sub + g.sub / 2 + a[2]) * g.W * g.sub + (a[1] * g.sub + g.sub / 2 + a[3]);
}

// Resolve list entry `i` of the pass to its {row, col, subrow, subcol}.
__device__ __forceinline__ void entry_key(const PixelSet& px, int i, int* a) { entry_coords(px, i, a); }

__device__ __forceinline__ bool cancelled(const DeviceFrame& f) { return f.cancel && *f.cancel; }

__device__ __forceinline__ double smooth_value(int n, double zrad) {
    return (double)n - log(log(zrad) / 2 / kLn2) / kLn2;
}

// ---------------------------------------------------------------------------
// Double path (mp.cpp:2290-2585, tryBLA mp.cpp:2714-2755).
__device__ __forceinline__ int bla_try_fp64(const BlaView& b, const double2* Z, int s, double& dzr, double& dzi, double& ddr, double& ddi, double dcr, double dci, bool ede, double ESC2, int mx_ref_it) {
    if (s < 1 || b.nlev == 0) return 0;
    double zmag2 = dzr * dzr + dzi * dzi;
    int maxp = b.nlev - 1;
    int startp = (s == 1) ? maxp : __ffs(s - 1) - 1;
    if (startp > maxp) startp = maxp;
    if (startp < b.minlevel) return 0;
    for (int p = startp; p >= b.minlevel; --p) {
        int i = (s - 1) >> p;
        if (i >= b.size[p]) continue;
        double r2 = b.r2[b.off[p] + i];
        if (r2 <= 0 || zmag2 >= r2) continue;
        int l = 1 << p;
        int land = s + l;
        if (land >= mx_ref_it - 1) continue;
        double4 bc = b.ab[b.off[p] + i];
        double nzr = bc.x * dzr - bc.y * dzi + bc.z * dcr - bc.w * dci;
        double nzi = bc.x * dzi + bc.y * dzr + bc.z * dci + bc.w * dcr;
        double2 zl = Z[land];
        double fr = zl.x + nzr, fi = zl.y + nzi;
        if (fr * fr + fi * fi > ESC2) return 0;
        if (ede) {
            double4 bd = b.ce[b.off[p] + i];
            double nddr = (bd.x * dzr - bd.y * dzi) + (bc.x * ddr - bc.y * ddi) + (bd.z * dcr - bd.w * dci);
            double nddi = (bd.x * dzi + bd.y * dzr) + (bc.x * ddi + bc.y * ddr) + (bd.z * dci + bd.w * dcr);
            ddr = nddr;
            ddi = nddi;
        }
        dzr = nzr;
        dzi = nzi;
        return l;
    }
    return 0;
}

// OC: the orbit colourings (orbit_color.h): their accumulators take every
// iteration's z; a trap turns BLA and the state-repetition detector off
// (mp.cpp:2121, 2388), a BLA skip restarts the stripe window (:2422-2427).
template <int OC>
__global__ void __launch_bounds__(128) k_fp64_pass(DeviceFrame f, Fp64Params p) {
    const FrameGeom& g = p.g;
    const double2* Z = f.orbit.Z;
    const double2* D = f.orbit.D;
    unsigned long long n_steps = 0, n_bla = 0, n_skip = 0, n_eff = 0;
    unsigned int n_int = 0;
    for (;;) {
        if (cancelled(f)) break;
        int i = (int)atomicAdd(&f.ctr->next, 1u);
        if (i >= f.px.n) break;
        int arr[4];
        entry_key(f.px, i, arr);
        // Per-pixel dc (mp.cpp:2300-2315) from the host-built mpf spacing tables.
        int xpix = g.sub * (arr[1] - p.ref[1]) + (arr[3] - p.ref[3]);
        int ypix = g.sub * (arr[0] - p.ref[0]) + (arr[2] - p.ref[2]);
        C2 dc = c2(p.dcx[xpix + p.xoff], p.dcy[ypix + p.yoff]);
        if (p.per) dc = c2(dc.re - p.frac_re, dc.im - p.frac_im);
        // Series-approximation seed (mp.cpp:2317-2330).
        C2 dz = c2(0, 0), dd = c2(0, 0);
        for (int x = p.sa_order; x >= 0; --x) {
            dz = c_add(dz, p.A[x]);
            dz = c_mul(dz, dc);
            dz = c_div(dz, p.sa_delta);
        }
        if (g.deriv) {
            for (int x = p.sa_order; x >= 0; --x) {
                dd = c_add(dd, p.B[x]);
                dd = c_mul(dd, dc);
                dd = c_div(dd, p.sa_delta);
            }
        }
        int j = p.sa_it + 1;
        double dzr = dz.re, dzi = dz.im, dcr = dc.re, dci = dc.im, ddr = dd.re, ddi = dd.im;
        double tmp, zr = 0, zi = 0, dr = 0, di = 0, zrad = 0;
        int k = j;
        const int per = p.per;
        int rk = k, rkm1 = k - 1;
        double zsr = 1e30, zsi = 1e30;
        int save_j = j, period_win = 1;
        int conf_P = 0, conf_next = 0, conf_count = 0, conf_giveup = 0;
        double conf_D2 = 0, conf_zr = 0, conf_zi = 0;
        const bool detect = p.use_interior != 0;
        const bool int_rep = p.int_rep && detect && !(OC & kOcTrap);
        OrbitColor<OC> oc;
        oc.init();
        double sdzr = 1e300, sdzi = 1e300;
        int sk = -1, save_j2 = j, twin2 = 1;
        int outcome = 0; // 0 running, 1 escaped, 2 interior, 3 glitch
        double gscore = -1.0;
        int tick = 0;
        while (j < g.mxit) {
            if (((++tick) & 4095) == 0 && cancelled(f)) {
                outcome = 4;
                break;
            }
            if (int_rep) {
                if (k == sk && dzr == sdzr && dzi == sdzi) {
                    outcome = 2;
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
            if (f.bla.use && !(OC & kOcTrap) && dzr * dzr + dzi * dzi < f.bla.rmax2) {
                int skip = bla_try_fp64(f.bla, Z, rkm1, dzr, dzi, ddr, ddi, dcr, dci, g.deriv, g.ESC2, p.mx_ref_it);
                if (skip > 0) {
                    ++n_bla;
                    n_skip += skip;
                    k += skip;
                    j += skip;
                    rk += skip;
                    if (per && rk >= per) rk -= per;
                    rkm1 = (per && rk == 0) ? per - 1 : rk - 1;
                    oc.skipped();
                    zsr = 1e30;
                    zsi = 1e30;
                    save_j = j;
                    period_win = 1;
                    conf_P = 0;
                    conf_giveup = 0;
                    continue;
                }
            }
            ++n_steps;
            if (g.deriv) {
                if (k == 0) {
                    tmp = (dzr * (1 + ddr) - dzi * (1 + ddi)) * 2;
                    ddi = (dzr * (1 + ddi) + dzi * (1 + ddr)) * 2;
                } else {
                    double2 zk = Z[k - 1], dk = D[k - 1];
                    tmp = (ddr * zk.x - ddi * zk.y + dzr * (dk.x + ddr) - dzi * (dk.y + ddi)) * 2;
                    ddi = (ddr * zk.y + ddi * zk.x + dzr * (dk.y + ddi) + dzi * (dk.x + ddr)) * 2;
                }
                ddr = tmp;
                double2 dk1 = D[k];
                dr = ddr + dk1.x;
                di = ddi + dk1.y;
            }
            double dzr2 = dzr * dzr;
            double dzi2 = dzi * dzi;
            if (k == 0) {
                tmp = dzr2 - dzi2 + dcr;
                dzi = dzr * dzi * 2 + dci;
            } else {
                double2 zp = Z[rkm1];
                tmp = (dzr * zp.x - dzi * zp.y) * 2 + dzr2 - dzi2 + dcr;
                dzi = (dzr * zp.y + dzi * zp.x) * 2 + dzr * dzi * 2 + dci;
            }
            dzr = tmp;
            double2 zc = Z[rk];
            zr = dzr + zc.x;
            zi = dzi + zc.y;
            zrad = zr * zr + zi * zi;
            oc.push(zr, zi);
            ++k;
            rkm1 = rk;
            if (per) {
                if (++rk == per) rk = 0;
            } else
                rk = k;
            if (zrad > g.ESC2) {
                outcome = 1;
                break;
            }
            if (detect) {
                if (conf_P > 0) {
                    conf_D2 *= 4 * zrad;
                    if (conf_D2 > 1e18) conf_D2 = 1e18;
                    if (j >= conf_next) {
                        double pr = zr - conf_zr, pi = zi - conf_zi;
                        bool ret = (pr * pr + pi * pi < p.interior_eps2 * zrad);
                        if (ret && conf_D2 < 1.0) {
                            if (++conf_count >= p.interior_confirm) {
                                outcome = 2;
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
                    if (pr * pr + pi * pi < p.interior_eps2 * zrad) {
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
            if (zrad < dzr * dzr + dzi * dzi || (!per && k == p.mx_ref_it)) {
                if ((dzr * dzr + dzi * dzi) / zrad > 10000000) {
                    gscore = zrad / f.orbit.zm3[per ? j % per : j];
                    outcome = 3;
                    break;
                }
                dzr = zr;
                dzi = zi;
                if (g.deriv) {
                    ddr = dr - 1;
                    ddi = di;
                }
                k = 0;
                rk = 0;
                rkm1 = per ? per - 1 : -1;
            }
            if (!per && k == p.mx_ref_it) {
                gscore = (double)zrad / f.orbit.zm3[j];
                outcome = 3;
                break;
            }
            ++j;
        }
        if (outcome == 4) break;
        if (outcome == 0 && j >= g.mxit) outcome = 2;
        const int idx = sample_index(g, arr);
        if (outcome == 1) {
            float v;
            if (g.ede) {
                v = (float)(sqrt(zrad) / g.dxf * log(zrad) / sqrt(dr * dr + di * di));
            } else {
                v = (float)smooth_value(j + 1, zrad);
                if (g.normal) {
                    // normal angle arg(z) - arg(dz/dc) (mp.cpp:2489-2492)
                    if (f.out.normal) f.out.normal[idx] = (float)(atan2(zi, zr) - atan2(di, dr));
                } else if (g.deovl) {
                    if (f.out.normal) f.out.normal[idx] = (float)(sqrt(zrad) / g.dxf * log(zrad) / sqrt(dr * dr + di * di));
                } else if (OC) { // trap, else stripe average (mp.cpp:2497-2500)
                    v = oc.escaped(smooth_value(j + 1, zrad), zrad, g.ER);
                }
            }
            f.out.iter[idx] = v;
            if (f.out.escN) f.out.escN[idx] = j + 1;
            f.out.done[i] = 1;
            n_eff += (unsigned long long)(j + 1);
        } else if (outcome == 2) {
            f.out.iter[idx] = oc.interior();
            if (f.out.escN) f.out.escN[idx] = -1;
            f.out.done[i] = 1;
            n_eff += (unsigned long long)g.mxit;
            ++n_int;
        } else {
            f.out.glitch[i] = gscore;
            if (gscore >= 0 && gscore < 1e100) atomicMin(&f.ctr->glitch_min_bits, (unsigned long long)__double_as_longlong(gscore));
        }
    }
    atomicAdd(&f.ctr->steps, n_steps);
    atomicAdd(&f.ctr->bla_applies, n_bla);
    atomicAdd(&f.ctr->bla_skipped, n_skip);
    atomicAdd(&f.ctr->effective_iters, n_eff);
    atomicAdd(&f.ctr->interior, n_int);
}

// ---------------------------------------------------------------------------
// Floatexp path helpers (mp.cpp:2770-2970).
__device__ void bla_rerescale_underflow(FE& S, double& wr, double& wi, double nwr, double nwi) { // mp.cpp:2770-2781
    if (nwr == 0.0 && nwi == 0.0) {
        S = fe_make(1.0, 0);
        wr = wi = 0.0;
        return;
    }
    FE wmag = fe_sqrt(fe_add(fe_mul(fe_from(nwr), fe_from(nwr)), fe_mul(fe_from(nwi), fe_from(nwi))));
    S = fe_mul(S, wmag);
    double inv = 1.0 / fe_to_double(wmag);
    wr = nwr * inv;
    wi = nwi * inv;
}

__device__ void fe_step_underflow(FE Xr, FE Xi, FE dcr, FE dci, FE& S, double& wr, double& wi) { // mp.cpp:2794-2835
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
    const double mag2 = nr * nr + ni * ni;
    const double mag = mag2 > 0.0 ? sqrt(mag2) : hypot(nr, ni);
    if (mag == 0.0) {
        S = fe_make(1.0, 0);
        wr = wi = 0.0;
        return;
    }
    S = fe_renorm(mag, e);
    wr = nr / mag;
    wi = ni / mag;
}

__device__ void fe_deriv_underflow(FE zr, FE zi, FE& SJ, double& jr, double& ji, double& invSJd) { // mp.cpp:2842-2876
    double im = 0.5 / SJ.m;
    int64_t ie = 1 - SJ.e;
    if (im >= 1.0) {
        im *= 0.5;
        ++ie;
    }
    FE invSJ = fe_make(im, ie);
    int64_t e = invSJ.e;
    if (zr.m != 0.0) e = max(e, zr.e);
    if (zi.m != 0.0) e = max(e, zi.e);
    auto align = [e](FE x) -> double {
        if (x.m == 0.0) return 0.0;
        int64_t d = x.e - e;
        if (d < -54) return 0.0;
        return x.m * pow2i((int)d);
    };
    double azr = align(zr), azi = align(zi);
    double ar = 2.0 * (azr * jr - azi * ji) + align(invSJ);
    double ai = 2.0 * (azr * ji + azi * jr);
    double mag = sqrt(ar * ar + ai * ai);
    if (mag == 0.0) {
        SJ = fe_make(1.0, 0);
        jr = ji = 0.0;
        invSJd = 1.0;
        return;
    }
    SJ = fe_mul(SJ, fe_renorm(mag, e));
    jr = ar / mag;
    ji = ai / mag;
    invSJd = 1.0 / fe_to_double(SJ);
}

// tryBLAfe (mp.cpp:2883-2970).
// wm2: wr * wr + wi * wi when the caller has it (else a negative value)
__device__ int bla_try_fe(const BlaView& b, const double2* Z, bool periodic, int s, FE& S, FE S2, double& wr, double& wi, double dr, double di, double ESC2, int mx_ref_it, double* ab,
                          double wm2 = -1.0) {
    if (s < 1 || b.nlev == 0) return 0;
    int maxp = b.nlev - 1;
    int startp = (s == 1) ? maxp : __ffs(s - 1) - 1;
    if (startp > maxp) startp = maxp;
    if (startp < b.minlevel) return 0;
    double w2 = wm2;
    if (dbits(wm2) >> 63) w2 = wr * wr + wi * wi; // (not known)
    FE dz2 = fe_mul(S2, fe_from(w2));
    if (b.rmax2 <= 0.0 || !fe_abs_less(dz2, fe_from(b.rmax2))) return 0;
    for (int p = startp; p >= b.minlevel; --p) {
        int i = (s - 1) >> p;
        if (i >= b.size[p]) continue;
        double r2 = b.r2[b.off[p] + i];
        if (d_le_zero(r2) || !fe_abs_less(dz2, fe_from(r2))) continue;
        int l = 1 << p;
        int land = s + l;
        if (land >= mx_ref_it - 1) continue;
        double4 bc = b.ab[b.off[p] + i];
        double nwr = (bc.x * wr - bc.y * wi) + (bc.z * dr - bc.w * di);
        double nwi = (bc.x * wi + bc.y * wr) + (bc.z * di + bc.w * dr);
        const double BIG = 1e150;
        double2 zl = Z[land];
        if (d_abs_less(nwr, BIG) && d_abs_less(nwi, BIG)) { // (finite, below 1e150)
            double fr = zl.x + fe_to_double(fe_mul_d(S, nwr));
            double fi = zl.y + fe_to_double(fe_mul_d(S, nwi));
            if (d_abs_less(ESC2, fr * fr + fi * fi)) return 0; // > ESC2
            double wm2 = nwr * nwr + nwi * nwi;
            if (d_is_zero(wm2)) {
                if (periodic)
                    bla_rerescale_underflow(S, wr, wi, nwr, nwi);
                else
                    return 0;
            } else {
                double wmag = sqrt(wm2);
                S = fe_mul(S, fe_from(wmag));
                double inv = 1.0 / wmag;
                wr = nwr * inv;
                wi = nwi * inv;
            }
        } else {
            FE dzr = fe_mul_d(S, wr), dzi = fe_mul_d(S, wi);
            FE dcrfe = fe_mul_d(S, dr), dcife = fe_mul_d(S, di);
            FE nzr = fe_add(fe_sub(fe_mul_d(dzr, bc.x), fe_mul_d(dzi, bc.y)), fe_sub(fe_mul_d(dcrfe, bc.z), fe_mul_d(dcife, bc.w)));
            FE nzi = fe_add(fe_add(fe_mul_d(dzr, bc.y), fe_mul_d(dzi, bc.x)), fe_add(fe_mul_d(dcrfe, bc.w), fe_mul_d(dcife, bc.z)));
            double fr = zl.x + fe_to_double(nzr), fi = zl.y + fe_to_double(nzi);
            if (fr * fr + fi * fi > ESC2) return 0;
            FE Snew = fe_sqrt(fe_add(fe_mul(nzr, nzr), fe_mul(nzi, nzi)));
            if (Snew.m == 0.0) {
                S = fe_make(1.0, 0);
                wr = wi = 0.0;
            } else {
                S = Snew;
                wr = fe_to_double(fe_div(nzr, S));
                wi = fe_to_double(fe_div(nzi, S));
            }
        }
        if (ab) {
            ab[0] = bc.x;
            ab[1] = bc.y;
            ab[2] = bc.z;
            ab[3] = bc.w;
        }
        return l;
    }
    return 0;
}

struct PixOut {
    float value;
    float nrm;
    int n;
    int state; // 1 escaped, 2 interior, 4 cancelled
};

// The plain delta step of pixelRescaled: w' = (2 X + s w) w + d in the fused
// form, 2 (X w) + s w^2 + d otherwise. On GB300 each FP64 instruction holds
// its SM quarter's FP64 unit for 64 cycles, independent operands or not, so
// the exact form's loops are bound by their count of FP64 instructions: the
// doubling X + X (exact) is formed on the bit pattern, and the tests below
// compare bit patterns (floatexp.h d_is_zero, d_abs_less, d_eq), with the
// IEEE results.
__device__ __forceinline__ void fe_plain_step(bool fused, double Xr, double Xi, double s, double wr, double wi, double dr, double di, double& nwr, double& nwi) {
    if (fused) {
        const double fR = d_twice(Xr) + s * wr;
        const double fI = d_twice(Xi) + s * wi;
        nwr = fR * wr - fI * wi + dr;
        nwi = fR * wi + fI * wr + di;
    } else {
        double w2r = wr * wr - wi * wi, w2i = 2.0 * wr * wi;
        nwr = 2.0 * (Xr * wr - Xi * wi) + s * w2r + dr;
        nwi = 2.0 * (Xr * wi + Xi * wr) + s * w2i + di;
    }
}
// |x| < 2^-1056 (the subnormal 2^18 * 2^-1074): the step's underflow test, on
// the bit pattern
__device__ __forceinline__ bool below_step_floor(double x) { return (dbits(x) & 0x7fffffffffffffffull) < 0x40000ull; }

// pixelRescaled (mp.cpp:3287-3618), smooth / EDE / DE-overlay.
// OC: the orbit colourings, as in k_fp64_pass (mp.cpp:3338-3346, 3389-3397,
// 3503-3504, 3524-3529); a trap turns BLA off.
template <int OC>
__device__ PixOut pixel_fe(const DeviceFrame& f, const FeParams& p, FE dcr, FE dci, unsigned long long& n_steps, unsigned long long& n_bla, unsigned long long& n_skip) {
    const FrameGeom& g = p.g;
    const double2* Z = f.orbit.Z;
    const FE2* Zfe = f.orbit.Zfe;
    const int reflen = p.mx_ref_it + 1;
    const int per = p.per;
    int rm = 0;
    FE S = fe_sqrt(fe_add(fe_mul(dcr, dcr), fe_mul(dci, dci)));
    double wr, wi, dr, di;
    if (S.m == 0.0) {
        S = fe_make(1.0, 0);
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
    const bool deriv = g.deriv != 0;
    FE SJ = fe_make(1.0, 0);
    double jr = 1.0, ji = 0.0, invSJd = 1.0;
    const bool detect = p.use_interior != 0;
    const bool int_rep = p.int_rep && detect && !(OC & kOcTrap);
    OrbitColor<OC> oc;
    oc.init();
    double swr = 1e300, swi = 1e300;
    FE sS = fe_make(1e300, 0);
    int sm = -1, save_iter2 = 1, twin2r = 1;
    PixOut o;
    o.nrm = 0.0f;
    o.n = -1;
    int tick = 0;
    // |w|^2 of the current state when the previous iteration formed it (a
    // step with no rescale or rebase after it), else -1
    double wm2_known = -1.0;
    while (iter < g.mxit) {
        const double wm2_now = wm2_known;
        wm2_known = -1.0;
        if (((++tick) & 4095) == 0 && cancelled(f)) {
            o.state = 4;
            return o;
        }
        if (int_rep) {
            if (m == sm && d_eq(wr, swr) && d_eq(wi, swi) && d_eq(S.m, sS.m) && S.e == sS.e) {
                o.value = -2.0f;
                o.state = 2;
                return o;
            }
            if (iter - save_iter2 >= twin2r) {
                swr = wr;
                swi = wi;
                sS = S;
                sm = m;
                save_iter2 = iter;
                twin2r += twin2r;
            }
        }
        if (f.bla.use && !(OC & kOcTrap) && m >= 2) {
            double ab[4];
            int skip = bla_try_fe(f.bla, Z, p.ref_period_gt0, rm, S, S2, wr, wi, dr, di, g.ESC2, per ? per : reflen, deriv ? ab : nullptr, wm2_now);
            if (skip > 0) {
                ++n_bla;
                n_skip += skip;
                oc.skipped();
                if (deriv) {
                    FE Jr = fe_mul_d(SJ, jr), Ji = fe_mul_d(SJ, ji);
                    FE nJr = fe_add(fe_sub(fe_mul_d(Jr, ab[0]), fe_mul_d(Ji, ab[1])), fe_from(ab[2]));
                    FE nJi = fe_add(fe_add(fe_mul_d(Jr, ab[1]), fe_mul_d(Ji, ab[0])), fe_from(ab[3]));
                    SJ = fe_sqrt(fe_add(fe_mul(nJr, nJr), fe_mul(nJi, nJi)));
                    if (SJ.m == 0.0) {
                        SJ = fe_make(1.0, 0);
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
        ++n_steps;
        double2 X = m ? Z[rm] : make_double2(0.0, 0.0);
        double Xr = X.x, Xi = X.y;
        // the pre-step z (DE colourings only)
        double zmr = 0.0, zmi = 0.0;
        bool deriv_underflow = false;
        if (deriv) {
            zmr = Xr + s * wr;
            zmi = Xi + s * wi;
            deriv_underflow = d_is_zero(zmr) && d_is_zero(zmi) && d_is_zero(invSJd);
        }
        FE zmrfe = fe_make(0, 0), zmife = fe_make(0, 0);
        if (deriv_underflow) {
            FE Xrfe = m ? Zfe[rm].re : fe_make(0.0, 0);
            FE Xife = m ? Zfe[rm].im : fe_make(0.0, 0);
            zmrfe = fe_add(Xrfe, fe_mul_d(S, wr));
            zmife = fe_add(Xife, fe_mul_d(S, wi));
        }
        double nwr, nwi;
        fe_plain_step(p.fused, Xr, Xi, s, wr, wi, dr, di, nwr, nwi);
        const bool step_underflow = below_step_floor(nwr) && below_step_floor(nwi);
        if (step_underflow && !(d_is_zero(nwr) && d_is_zero(nwi) && d_is_zero(wr) && d_is_zero(wi) && d_is_zero(dcr.m) && d_is_zero(dci.m))) {
            FE Xrfe = m ? Zfe[rm].re : fe_make(0.0, 0);
            FE Xife = m ? Zfe[rm].im : fe_make(0.0, 0);
            fe_step_underflow(Xrfe, Xife, dcr, dci, S, wr, wi);
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
                fe_deriv_underflow(zmrfe, zmife, SJ, jr, ji, invSJd);
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
        X = m ? Z[rm] : make_double2(0.0, 0.0);
        Xr = X.x;
        Xi = X.y;
        double zr = Xr + s * wr, zi = Xi + s * wi;
        double zrad = zr * zr + zi * zi;
        const double wmag2 = wr * wr + wi * wi;
        bool keep = true;
        oc.push(zr, zi);
        if (d_abs_less(g.ESC2, zrad)) { // zrad > ESC2
            o.n = iter;
            o.state = 1;
            if (g.ede) {
                double num = sqrt(zrad) * log(zrad);
                FE Jmag = fe_mul_d(SJ, sqrt(jr * jr + ji * ji));
                o.value = (float)fe_to_double(fe_div(fe_from(num), fe_mul(p.dxfe, Jmag)));
                return o;
            }
            if (g.normal) {
                // normal angle arg(z) - arg(J); SJ > 0 (mp.cpp:3512-3515)
                o.nrm = (float)(atan2(zi, zr) - atan2(ji, jr));
            } else if (g.deovl) {
                double num = sqrt(zrad) * log(zrad);
                FE Jmag = fe_mul_d(SJ, sqrt(jr * jr + ji * ji));
                o.nrm = (float)fe_to_double(fe_div(fe_from(num), fe_mul(p.dxfe, Jmag)));
            } else if (OC) { // trap, else stripe average
                o.value = oc.escaped((double)iter - log(log(zrad) / 2.0 / kLn2) / kLn2, zrad, g.ER);
                return o;
            }
            o.value = (float)((double)iter - log(log(zrad) / 2.0 / kLn2) / kLn2);
            return o;
        }
        if (detect) {
            if (conf_P > 0) {
                conf_D2 *= 4.0 * zrad;
                if (d_abs_less(1e18, conf_D2)) conf_D2 = 1e18; // conf_D2 >= +0 or NaN
                if (iter >= conf_next) {
                    double pr = zr - conf_zr, pi = zi - conf_zi;
                    if (d_abs_less(pr * pr + pi * pi, p.interior_eps2 * zrad) && d_abs_less(conf_D2, 1.0)) {
                        if (++conf_count >= p.interior_confirm) {
                            o.value = oc.interior();
                            o.state = 2;
                            return o;
                        }
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
                if (d_abs_less(pr * pr + pi * pi, p.interior_eps2 * zrad)) {
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
        // |w|^2 > 1e16, or 0 < |w|^2 < 1e-16 (|w|^2 >= +0 or NaN)
        if (d_abs_less(1e16, wmag2) || (d_abs_less(wmag2, 1e-16) && !d_is_zero(wmag2))) {
            FE wmag = fe_sqrt(fe_from(wmag2));
            S = fe_mul(S, wmag);
            s = fe_to_double(S);
            S2 = fe_mul(S, S);
            double inv = 1.0 / fe_to_double(wmag);
            wr *= inv;
            wi *= inv;
            dr = fe_to_double(fe_div(dcr, S));
            di = fe_to_double(fe_div(dci, S));
            keep = false;
        }
        double dzmag2 = s * s * (keep ? wmag2 : wr * wr + wi * wi);
        if (d_abs_less(zrad, 1e-8) || d_abs_less(zrad, dzmag2) || (!per && m >= reflen)) { // zrad, dzmag2 >= +0 or NaN
            FE Xmr = m ? Zfe[rm].re : fe_make(0.0, 0);
            FE Xmi = m ? Zfe[rm].im : fe_make(0.0, 0);
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
                keep = false;
            }
        }
        if (keep) wm2_known = wmag2;
    }
    o.value = oc.interior();
    o.state = 2;
    return o;
}

// solveRescaledSimd8NoBla semantics for one lane (mp.cpp:3620-3816).
__device__ PixOut pixel_fe_nobla(const DeviceFrame& f, const FeParams& p, FE dcr, FE dci, unsigned long long& n_steps) {
    const FrameGeom& g = p.g;
    const double2* Z = f.orbit.Z;
    const FE2* Zfe = f.orbit.Zfe;
    const int mx_ref_it = p.mx_ref_it;
    const int referenceLength = mx_ref_it + 1;
    double wr = 0, wi = 0, sd, dr = 0, di = 0;
    FE scale;
    const FE s0 = fe_sqrt(fe_add(fe_mul(dcr, dcr), fe_mul(dci, dci)));
    if (s0.m == 0.0) {
        scale = fe_make(1.0, 0);
    } else {
        scale = s0;
        wr = fe_to_double(fe_div(dcr, s0));
        wi = fe_to_double(fe_div(dci, s0));
        dr = wr;
        di = wi;
    }
    sd = fe_to_double(scale);
    int index = 1, iteration = 1;
    PixOut o;
    o.nrm = 0.0f;
    o.n = -1;
    int tick = 0;
    for (;;) {
        if (iteration >= g.mxit) {
            o.value = -2.0f;
            o.state = 2;
            return o;
        }
        if (((++tick) & 4095) == 0 && cancelled(f)) {
            o.state = 4;
            return o;
        }
        ++n_steps;
        double pr = 0, pi = 0;
        if (index > 0) {
            double2 zp = Z[index - 1];
            pr = zp.x;
            pi = zp.y;
        }
        const int current = index > mx_ref_it ? mx_ref_it : index;
        double2 zc = Z[current];
        double nwr, nwi;
        if (p.fused) {
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
        const double aR = zc.x + (sd * nwr), aI = zc.y + (sd * nwi);
        double actual = (aR * aR) + (aI * aI);
        double delta = (nwr * nwr) + (nwi * nwi);
        if (delta == 0.0 && (nwr != 0.0 || nwi != 0.0 || wr != 0.0 || wi != 0.0 || dcr.m != 0.0 || dci.m != 0.0)) {
            const FE rR = index ? Zfe[index - 1].re : fe_make(0.0, 0);
            const FE rI = index ? Zfe[index - 1].im : fe_make(0.0, 0);
            fe_step_underflow(rR, rI, dcr, dci, scale, wr, wi);
            sd = fe_to_double(scale);
            dr = fe_to_double(fe_div(dcr, scale));
            di = fe_to_double(fe_div(dci, scale));
            const FE ar = fe_add(Zfe[current].re, fe_mul_d(scale, wr));
            const FE ai = fe_add(Zfe[current].im, fe_mul_d(scale, wi));
            actual = fe_to_double(fe_add(fe_mul(ar, ar), fe_mul(ai, ai)));
            delta = wr * wr + wi * wi;
        } else {
            wr = nwr;
            wi = nwi;
        }
        ++index;
        ++iteration;
        if (actual > g.ESC2) {
            o.n = iteration;
            o.state = 1;
            o.value = (float)((double)iteration - log(log(actual) / 2.0 / kLn2) / kLn2);
            return o;
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
            const FE rR = index ? Zfe[index - 1].re : fe_make(0.0, 0);
            const FE rI = index ? Zfe[index - 1].im : fe_make(0.0, 0);
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

template <int OC>
__global__ void __launch_bounds__(128) k_fe_pass(DeviceFrame f, FeParams p) {
    if (p.lanes_per_warp && (int)(threadIdx.x & 31u) >= p.lanes_per_warp) return;
    const FrameGeom& g = p.g;
    unsigned long long n_steps = 0, n_bla = 0, n_skip = 0, n_eff = 0;
    unsigned int n_int = 0;
    const int n = f.px.n_dev ? min((int)*f.px.n_dev, f.px.n) : f.px.n;
    for (;;) {
        if (cancelled(f)) break;
        // plain read first: threads past the end leave without an atomic
        if ((int)*(volatile unsigned int*)&f.ctr->next >= n) break;
        int i = (int)atomicAdd(&f.ctr->next, 1u);
        if (i >= n) break;
        int arr[4];
        entry_key(f.px, i, arr);
        // dc in floatexp (mp.cpp:2160-2163).
        double px = arr[1] + (double)arr[3] / g.sub;
        double py = arr[0] + (double)arr[2] / g.sub;
        FE Dcr = fe_mul_d(p.dxfe, px - p.ref_x);
        FE Dci = fe_mul_d(p.dyfe, py - p.ref_y);
        // (the no-BLA lane kernel has no orbit colourings, mp.cpp:2148)
        PixOut o = (OC == 0 && p.no_bla_kernel) ? pixel_fe_nobla(f, p, Dcr, Dci, n_steps) : pixel_fe<OC>(f, p, Dcr, Dci, n_steps, n_bla, n_skip);
        if (o.state == 4) break;
        const int idx = sample_index(g, arr);
        // mp.cpp:2173-2183: EMPTY or cutoff-sensitive results go to the
        // arbitrary-precision recompute, flagged here for the host.
        const float v = o.value;
        if (v == kEmpty || (p.cutoff_sensitive && (v < 0 || v > g.mxit - 16))) {
            f.out.gmp[i] = 1;
            atomicAdd(&f.ctr->gmp_flags, 1u);
        }
        f.out.iter[idx] = v;
        if ((g.deovl || g.normal) && f.out.normal) f.out.normal[idx] = o.nrm;
        if (f.out.escN) f.out.escN[idx] = o.state == 1 ? o.n : -1;
        f.out.done[i] = 1;
        if (o.state == 1) {
            n_eff += (unsigned long long)o.n;
        } else {
            n_eff += (unsigned long long)g.mxit;
            ++n_int;
        }
    }
    atomicAdd(&f.ctr->steps, n_steps);
    atomicAdd(&f.ctr->bla_applies, n_bla);
    atomicAdd(&f.ctr->bla_skipped, n_skip);
    atomicAdd(&f.ctr->effective_iters, n_eff);
    atomicAdd(&f.ctr->interior, n_int);
}

// ---------------------------------------------------------------------------
// Shallow direct loop: floatPointCompute (mp.cpp:330-399) and the lane-refill
// kernel's per-lane arithmetic (mp.cpp:416-532).
template <int OC>
__device__ double shallow_scalar(double c_re, double c_im, int mxit, const FrameGeom& g, double* nrm, int* nout) {
    double z_re = c_re, z_im = c_im, d_re = 2, d_im = 0, dc_re = 1, dc_im = 0, tmp;
    const bool deriv = g.ede || g.deovl || g.normal;
    OrbitColor<OC> oc; // mp.cpp:347-369
    oc.init();
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
        oc.push(z_re, z_im);
        tmp = z_re * z_re + z_im * z_im;
        if (tmp > g.ESC2) {
            *nout = i + 1;
            if (g.ede) return sqrt(tmp) * log(tmp) / sqrt(dc_re * dc_re + dc_im * dc_im);
            if (g.normal) { // mp.cpp:375-378
                if (nrm) *nrm = atan2(z_im, z_re) - atan2(dc_im, dc_re);
                return (i + 1 - log(log(tmp) / 2 / kLn2) / kLn2);
            }
            if (g.deovl) {
                if (nrm) *nrm = sqrt(tmp) * log(tmp) / sqrt(dc_re * dc_re + dc_im * dc_im);
                return (i + 1 - log(log(tmp) / 2 / kLn2) / kLn2);
            }
            if (OC) return oc.escaped(i + 1 - log(log(tmp) / 2 / kLn2) / kLn2, tmp, g.ER); // mp.cpp:383-389
            return (i + 1 - log(log(tmp) / 2 / kLn2) / kLn2);
        }
        tmp = d_re * d_re + d_im * d_im;
        if (tmp < 0.000000001) return oc.interior();
        ++i;
    }
    return oc.interior();
}

__device__ float shallow_lane(double cr, double ci, int mxit, const FrameGeom& g, int* nout) {
    double zr = cr, zi = ci, dr = 2, di = 0, dcr = 1, dci = 0, jv = 1;
    for (;;) {
        double ndr = 2.0 * ((dr * zr) - (di * zi));
        double ndi = 2.0 * ((dr * zi) + (di * zr));
        double ndcr = (2.0 * ((dcr * zr) - (dci * zi))) + 1.0;
        double ndci = 2.0 * ((dcr * zi) + (dci * zr));
        double nzr = ((zr * zr) - (zi * zi)) + cr;
        double nzi = (2.0 * (zr * zi)) + ci;
        zr = nzr;
        zi = nzi;
        dr = ndr;
        di = ndi;
        dcr = ndcr;
        dci = ndci;
        double zrad = (zr * zr) + (zi * zi);
        double dmag = (dr * dr) + (di * di);
        double jnext = jv + 1.0;
        if (zrad > g.ESC2) {
            *nout = (int)jv + 1;
            if (g.ede) return (float)(sqrt(zrad) * log(zrad) / sqrt(dcr * dcr + dci * dci));
            return (float)(jv + 1 - log(log(zrad) / 2 / kLn2) / kLn2);
        }
        if (dmag < 1e-9) return -2.0f;
        if (jnext >= (double)mxit) return -2.0f;
        jv = jnext;
    }
}

// One Julia sample with the per-lane arithmetic of solveJuliaShallowSimdList
// (mp.cpp:534-636): z0 the sample, c fixed, D_0 = 1 and D' = 2 z D under EDE.
// nout: escape index (0 when z0 is already outside), -1 interior.
__device__ float julia_lane(double zr, double zi, double cr, double ci, int mxit, const FrameGeom& g, int* nout) {
    double zrad = (zr * zr) + (zi * zi);
    *nout = -1;
    if (zrad > g.ESC2) {
        *nout = 0;
        return g.ede ? (float)(sqrt(zrad) * log(zrad)) : (float)(-log(log(zrad) / 2 / kLn2) / kLn2);
    }
    double dr = 1.0, di = 0.0, jv = 0.0;
    for (;;) {
        double ndr = dr, ndi = di;
        if (g.ede) {
            ndr = 2.0 * ((dr * zr) - (di * zi));
            ndi = 2.0 * ((dr * zi) + (di * zr));
        }
        const double nzr = ((zr * zr) - (zi * zi)) + cr;
        const double nzi = (2.0 * (zr * zi)) + ci;
        zr = nzr;
        zi = nzi;
        dr = ndr;
        di = ndi;
        zrad = (zr * zr) + (zi * zi);
        const double jnext = jv + 1.0;
        if (zrad > g.ESC2) {
            *nout = (int)jv + 1;
            if (g.ede) {
                const double denom = sqrt((dr * dr) + (di * di));
                return denom > 0.0 ? (float)(sqrt(zrad) * log(zrad) / denom) : 0.0f;
            }
            return (float)(jv + 1 - log(log(zrad) / 2 / kLn2) / kLn2);
        }
        if (jnext >= (double)mxit) return -2.0f;
        jv = jnext;
    }
}

// ComputeJulia's frame (mp.cpp:1019-1041): every sample of the grid, the EDE
// value divided by (float)dx.
__global__ void __launch_bounds__(128) k_julia(DeviceFrame f, JuliaParams p) {
    const FrameGeom& g = p.g;
    unsigned long long n_eff = 0, n_steps = 0;
    unsigned int n_int = 0;
    const int n = g.W * g.H;
    for (;;) {
        if (cancelled(f)) break;
        const int s = (int)atomicAdd(&f.ctr->next, 1u);
        if (s >= n) break;
        const int i = s / g.W, j = s - i * g.W;
        const double imag = p.z0i + p.dy * i;
        int nout = -1;
        float v = julia_lane(p.z0r + p.dx * j, imag, p.cr, p.ci, g.mxit, g, &nout);
        if (g.ede && v >= 0.0f) v /= (float)p.dx;
        f.out.iter[s] = v;
        if (f.out.escN) f.out.escN[s] = nout;
        if (nout >= 0) {
            n_eff += (unsigned long long)nout;
            n_steps += (unsigned long long)nout;
        } else {
            n_eff += (unsigned long long)g.mxit;
            n_steps += (unsigned long long)g.mxit;
            ++n_int;
        }
    }
    atomicAdd(&f.ctr->effective_iters, n_eff);
    atomicAdd(&f.ctr->steps, n_steps);
    atomicAdd(&f.ctr->interior, n_int);
}

// Base pass (mp.cpp:1483-1519) in grid mode, or adaptive-SS sub-samples
// (mp.cpp:1920-1969) from a key list.
template <int OC>
__global__ void __launch_bounds__(128) k_shallow(DeviceFrame f, ShallowParams p) {
    const FrameGeom& g = p.g;
    unsigned long long n_eff = 0, n_steps = 0;
    unsigned int n_int = 0;
    for (;;) {
        if (cancelled(f)) break;
        int i = (int)atomicAdd(&f.ctr->next, 1u);
        if (i >= f.px.n) break;
        int arr[4];
        entry_key(f.px, i, arr);
        double cr, ci;
        if (arr[2] == 0 && arr[3] == 0 && !f.px.keys) {
            ci = p.c0i + p.dy * arr[0];
            cr = p.c0r + p.dx * arr[1];
        } else {
            cr = p.c0r + p.dx * arr[1] + p.dx * arr[3] / g.sub;
            ci = p.c0i + p.dy * arr[0] + p.dy * arr[2] / g.sub;
        }
        const int idx = sample_index(g, arr);
        int nout = -1;
        double val;
        if (OC == 0 && p.simd_semantics) { // (no orbit colourings in the lane kernel, mp.cpp:1459)
            val = (double)shallow_lane(cr, ci, g.mxit, g, &nout);
            if (g.ede && val >= 0) val /= p.dx;
            f.out.iter[idx] = (float)val;
        } else {
            double de = 0.0;
            val = shallow_scalar<OC>(cr, ci, g.mxit, g, &de, &nout);
            if (g.normal) { // mp.cpp:1504-1507 (with EDE also set: the raw distance, angle 0)
                f.out.iter[idx] = (float)val;
                if (f.out.normal) f.out.normal[idx] = (float)de;
            } else if (g.deovl) {
                float v = (float)val;
                f.out.iter[idx] = v;
                if (f.out.normal) f.out.normal[idx] = (v < 0) ? 0.0f : (float)(de / p.dx);
            } else { // the value is stored as float before the EDE division (mp.cpp:1512-1515)
                float v = (float)val;
                if (g.ede && v >= 0) v = (float)((double)v / p.dx);
                f.out.iter[idx] = v;
            }
        }
        if (f.out.escN) f.out.escN[idx] = nout;
        f.out.done[i] = 1;
        if (nout > 0) {
            n_eff += (unsigned long long)nout;
            n_steps += (unsigned long long)nout;
        } else {
            n_eff += (unsigned long long)g.mxit;
            ++n_int;
        }
    }
    atomicAdd(&f.ctr->effective_iters, n_eff);
    atomicAdd(&f.ctr->steps, n_steps);
    atomicAdd(&f.ctr->interior, n_int);
}

// ---------------------------------------------------------------------------
// BLA table construction (mp.cpp:2613-2709): level 0 from the orbit, then one
// launch per merge level; every entry of a level is independent.
__global__ void k_bla_level0(const double2* Z, const double2* D, int reflen, double eps, double dcmax, int ede, double* r2, double4* ab, double4* ce, unsigned long long* rmax2_bits) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int s = t + 1;
    if (s >= reflen) return;
    double2 z = Z[s];
    double zr = z.x, zi = z.y;
    double Zmag = sqrt(zr * zr + zi * zi);
    double ar = 2.0 * zr, ai = 2.0 * zi;
    double Amag = 2.0 * Zmag;
    double R = eps * (Zmag - dcmax) / (Amag + 1.0);
    double rr = R > 0 ? R * R : 0.0;
    r2[t] = rr;
    ab[t] = make_double4(ar, ai, 1.0, 0.0);
    if (ede) {
        double2 d = D[s];
        ce[t] = make_double4(2.0 * d.x, 2.0 * d.y, 0.0, 0.0);
    }
    if (rr > 0) atomicMax(rmax2_bits, (unsigned long long)__double_as_longlong(rr));
}

__global__ void k_bla_merge(double dcmax, int ede, double* r2, double4* ab, double4* ce, int src_off, int dst_off, int dst_size) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dst_size) return;
    const int xi = src_off + 2 * i, yi = xi + 1;
    double4 xc = ab[xi], yc = ab[yi];
    double4 zc;
    zc.x = yc.x * xc.x - yc.y * xc.y;
    zc.y = yc.x * xc.y + yc.y * xc.x;
    zc.z = yc.x * xc.z - yc.y * xc.w + yc.z;
    zc.w = yc.x * xc.w + yc.y * xc.z + yc.w;
    if (ede) {
        double4 xd = ce[xi], yd = ce[yi];
        double4 zd;
        zd.x = (yd.x * xc.x - yd.y * xc.y) + (yc.x * xd.x - yc.y * xd.y);
        zd.y = (yd.x * xc.y + yd.y * xc.x) + (yc.x * xd.y + yc.y * xd.x);
        zd.z = (yd.x * xc.z - yd.y * xc.w) + (yc.x * xd.z - yc.y * xd.w) + yd.z;
        zd.w = (yd.x * xc.w + yd.y * xc.z) + (yc.x * xd.w + yc.y * xd.z) + yd.w;
        ce[dst_off + i] = zd;
    }
    double Rx = sqrt(r2[xi]), Ry = sqrt(r2[yi]);
    double Axmag = sqrt(xc.x * xc.x + xc.y * xc.y);
    double Bxmag = sqrt(xc.z * xc.z + xc.w * xc.w);
    double cand = Axmag > 0 ? (Ry - Bxmag * dcmax) / Axmag : 0.0;
    double R = (cand < Rx) ? cand : Rx; // std::min(Rx, cand)
    r2[dst_off + i] = R > 0 ? R * R : 0.0;
    ab[dst_off + i] = zc;
}

// ---------------------------------------------------------------------------
// Adaptive-SS flags over the base samples (mp.cpp:1838-1884).
// Adaptive-SS selection (mp.cpp:1796-1879). mode: kSsIterations (the
// iteration difference against thresh), kSsEde (a sign change: the set
// boundary), kSsStripe / kSsTrap (the stripe average and orbit traps store a
// value, not a count: the set boundary, or a colour change of more than
// `steps` palette entries per pixel, `gain` entries per unit of value; the
// stripe average's steps default to 0, the boundary only).
__global__ void k_ss_flags(const float* iter, int W, int H, int sub, int mode, double thresh, double gain, double steps, uint8_t* flags) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= W * H) return;
    int i = q / W, j = q % W;
    auto at = [&](int r, int c) { return iter[(r * sub + sub / 2) * W * sub + (c * sub + sub / 2)]; };
    bool need = false;
    if (mode == kSsEde) {
        float cv = at(i, j);
        for (int xi = -1; xi <= 1 && !need; ++xi)
            for (int yi = -1; yi <= 1; ++yi) {
                if (xi == 0 && yi == 0) continue;
                int ny = i + yi, nx = j + xi;
                if (nx >= 0 && nx < W && ny >= 0 && ny < H && cv * at(ny, nx) < 0) {
                    need = true;
                    break;
                }
            }
    } else {
        float cv = at(i, j);
        float diff = 0;
        bool boundary = false;
        for (int xi = -1; xi <= 1; ++xi)
            for (int yi = -1; yi <= 1; ++yi) {
                if (xi == 0 && yi == 0) continue;
                int ny = i + yi, nx = j + xi;
                if (nx >= 0 && nx < W && ny >= 0 && ny < H) {
                    const float nv = at(ny, nx);
                    diff = fmaxf(diff, fabsf(cv - nv));
                    if (cv * nv < 0) boundary = true; // interior / exterior edge
                }
            }
        if (mode == kSsStripe)
            need = boundary || (steps > 0 && diff * gain > steps);
        else if (mode == kSsTrap)
            need = boundary || (diff * gain > steps);
        else
            need = log((double)diff) > thresh;
    }
    flags[q] = need ? 1 : 0;
}

__global__ void k_fill(float* iter, float* normal, int32_t* escN, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n; i += stride) {
        iter[i] = kEmpty;
        if (normal) normal[i] = 0.0f;
        if (escN) escN[i] = -10;
    }
}

// ---------------------------------------------------------------------------
cudaError_t launch_fill(float* iter, float* normal, int32_t* escN, size_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_fill<<<blocks, 256, 0, st>>>(iter, normal, escN, n);
    return cudaGetLastError();
}
cudaError_t launch_fp64_pass(const DeviceFrame& f, const Fp64Params& p, int blocks, int threads, cudaStream_t st) {
    switch (p.g.oc) {
    case 0: k_fp64_pass<0><<<blocks, threads, 0, st>>>(f, p); break;
    case kOcStripe: k_fp64_pass<kOcStripe><<<blocks, threads, 0, st>>>(f, p); break;
    case kOcTrap: k_fp64_pass<kOcTrap><<<blocks, threads, 0, st>>>(f, p); break;
    default: k_fp64_pass<kOcStripe | kOcTrap><<<blocks, threads, 0, st>>>(f, p); break;
    }
    return cudaGetLastError();
}
cudaError_t launch_fe_pass(const DeviceFrame& f, const FeParams& p, int blocks, int threads, cudaStream_t st) {
    switch (p.g.oc) {
    case 0: k_fe_pass<0><<<blocks, threads, 0, st>>>(f, p); break;
    case kOcStripe: k_fe_pass<kOcStripe><<<blocks, threads, 0, st>>>(f, p); break;
    case kOcTrap: k_fe_pass<kOcTrap><<<blocks, threads, 0, st>>>(f, p); break;
    default: k_fe_pass<kOcStripe | kOcTrap><<<blocks, threads, 0, st>>>(f, p); break;
    }
    return cudaGetLastError();
}
cudaError_t launch_julia(const DeviceFrame& f, const JuliaParams& p, int blocks, int threads, cudaStream_t st) {
    k_julia<<<blocks, threads, 0, st>>>(f, p);
    return cudaGetLastError();
}

cudaError_t launch_shallow(const DeviceFrame& f, const ShallowParams& p, int blocks, int threads, cudaStream_t st) {
    switch (p.g.oc) {
    case 0: k_shallow<0><<<blocks, threads, 0, st>>>(f, p); break;
    case kOcStripe: k_shallow<kOcStripe><<<blocks, threads, 0, st>>>(f, p); break;
    case kOcTrap: k_shallow<kOcTrap><<<blocks, threads, 0, st>>>(f, p); break;
    default: k_shallow<kOcStripe | kOcTrap><<<blocks, threads, 0, st>>>(f, p); break;
    }
    return cudaGetLastError();
}
cudaError_t launch_bla_build(const double2* Z, const double2* D, int reflen, double eps, double dcmax, bool ede, double* r2, double4* ab, double4* ce, const int* off, const int* size, int nlev, unsigned long long* rmax2_bits, cudaStream_t st) {
    int n0 = reflen - 1;
    if (n0 <= 0) return cudaSuccess;
    k_bla_level0<<<(n0 + 255) / 256, 256, 0, st>>>(Z, D, reflen, eps, dcmax, ede ? 1 : 0, r2, ab, ce, rmax2_bits);
    for (int p = 1; p < nlev; ++p) {
        int n = size[p];
        if (n <= 0) break;
        k_bla_merge<<<(n + 255) / 256, 256, 0, st>>>(dcmax, ede ? 1 : 0, r2, ab, ce, off[p - 1], off[p], n);
    }
    return cudaGetLastError();
}
cudaError_t launch_ss_flags(const float* iter, int W, int H, int sub, int mode, double thresh, double gain, double steps, uint8_t* flags, cudaStream_t st) {
    int n = W * H;
    k_ss_flags<<<(n + 255) / 256, 256, 0, st>>>(iter, W, H, sub, mode, thresh, gain, steps, flags);
    return cudaGetLastError();
}

} // namespace mbx

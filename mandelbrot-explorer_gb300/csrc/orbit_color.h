// Orbit colourings of the delta loops (host and device): the stripe average
// (ColoringMethod::STRIPE_AVERAGE, "SAC") and the orbit traps
// (ColoringMethod::ORBIT_TRAP), as src/engine/orbit_coloring.h:21-132 defines
// them and the loops use them (mp.cpp:338-398 shallow, 2359-2378, 2422-2427,
// 2471-2472, 2497-2500 double path, 3338-3346, 3389-3397, 3503-3504, 3524-3529
// floatexp path, 764-882 arbitrary-precision point).
//
// Stripe average: every iteration's z adds the term t = 1/2 + sin(7 arg z) / 2;
// the value is the average of the last W terms under a triangular weight (the
// newest weighs W, the oldest 1), interpolated at escape between the average
// with and without the last term by the smooth-iteration fraction. A BLA skip
// breaks the run of terms, so it restarts the window. W = 256, the
// reference's default window.
// Orbit traps: the orbit's closest approach to the point 0 (|z|), the cross
// (min(|Re z|, |Im z|), weighted 1.5) and the circle |z| = 1/2; the value is
// 0.17 (-log10 distance) + 0.025 mu, mu the smooth escape count (0 interior).
// Operation order follows the reference's, in double; sin, atan2, log and
// log10 are the platform's (CUDA's on the device).
#pragma once
#include <math.h>

#ifndef MBX_OC_HD
#ifdef __CUDACC__
#define MBX_OC_HD __host__ __device__ __forceinline__
#else
#define MBX_OC_HD inline
#endif
#endif

namespace mbx {

// coloring bits of the orbit colourings (mbx_request.coloring_method)
constexpr int kOcStripe = 1, kOcTrap = 2;
constexpr int kStripeWindow = 256;

struct StripeAvg {
    double ring[kStripeWindow];
    double run;     // sum of the window's terms
    double tri;     // triangular-weighted sum (newest term weight W)
    double last;    // the latest term
    int pos, fill;

    MBX_OC_HD void init() {
        run = tri = last = 0.0;
        pos = fill = 0;
    }
    MBX_OC_HD void restart() { // a BLA skip: the window starts again
        run = tri = 0.0;
        pos = fill = 0;
    }
    MBX_OC_HD void push(double zr, double zi) {
        const double t = 0.5 + 0.5 * sin(7.0 * atan2(zi, zr));
        last = t;
        double out = 0.0;
        if (fill == kStripeWindow) out = ring[pos];
        else ++fill;
        // every older term loses one unit of weight, the new one enters at W
        tri += (double)kStripeWindow * t - run;
        run += t - out;
        ring[pos] = t;
        pos = pos + 1 == kStripeWindow ? 0 : pos + 1;
    }
    // value at escape: |z|^2 = zrad, escape radius R
    MBX_OC_HD float value(double zrad, double R) const {
        double frac = 1.0 - log(log(zrad) * 0.5 / log(R)) / log(2.0);
        const double weight = (double)fill * kStripeWindow - (double)fill * (fill - 1) / 2.0;
        const double with_last = weight > 0.0 ? tri / weight : 0.0;
        const double wl = (double)kStripeWindow;
        const double without_last = weight > wl ? (tri - wl * last) / (weight - wl) : with_last;
        frac -= floor(frac);
        return (float)(without_last + (with_last - without_last) * frac);
    }
};

struct OrbitTrap {
    double point2;  // min |z|^2
    double cross;   // min min(|Re z|, |Im z|)
    double circle;  // min ||z| - 1/2|

    MBX_OC_HD void init() { point2 = cross = circle = 1e300; }
    MBX_OC_HD void push(double zr, double zi) {
        const double m2 = zr * zr + zi * zi;
        if (m2 < point2) point2 = m2;
        const double c = fmin(fabs(zr), fabs(zi));
        if (c < cross) cross = c;
        const double r = fabs(sqrt(m2) - 0.5);
        if (r < circle) circle = r;
    }
    // mu: the smooth escape count (0 for interior samples)
    MBX_OC_HD float value(double mu) const {
        double d = fmin(fmin(sqrt(point2), cross * 1.5), circle);
        if (d > 1.0) d = 1.0;
        const double trap = -log10(fmax(d, 1e-14));
        if (mu < 0.0) mu = 0.0;
        return (float)(0.17 * trap + 0.025 * mu);
    }
};

// The accumulators of one sample; OC selects which exist (kOcStripe, kOcTrap).
template <int OC>
struct OrbitColor {
    StripeAvg sac;
    OrbitTrap trap;
    MBX_OC_HD void init() {
        if (OC & kOcStripe) sac.init();
        if (OC & kOcTrap) trap.init();
    }
    MBX_OC_HD void push(double zr, double zi) {
        if (OC & kOcStripe) sac.push(zr, zi);
        if (OC & kOcTrap) trap.push(zr, zi);
    }
    MBX_OC_HD void skipped() {
        if (OC & kOcStripe) sac.restart();
    }
    // escape value when no DE / normal-map / overlay colouring takes precedence
    MBX_OC_HD float escaped(double mu, double zrad, double R) const {
        if (OC & kOcTrap) return trap.value(mu);
        return sac.value(zrad, R);
    }
    MBX_OC_HD float interior() const { return (OC & kOcTrap) ? trap.value(0.0) : -2.0f; }
};
template <>
struct OrbitColor<0> { // no orbit colouring: nothing to carry
    MBX_OC_HD void init() {}
    MBX_OC_HD void push(double, double) {}
    MBX_OC_HD void skipped() {}
    MBX_OC_HD float escaped(double, double, double) const { return 0.0f; }
    MBX_OC_HD float interior() const { return -2.0f; }
};

} // namespace mbx

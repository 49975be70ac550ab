// Host build of the device colour math (mandelbrot-explorer_gb300/csrc/
// color_math.cuh), compiled by tests/test_color.py with -ffp-contract=off:
// the same IEEE operations the kernel executes. Checks, over log-uniform
// values v in [0, 1e7], that log(v+2) and the palette coordinate
// pow(L, L^2*density/3600) round exactly as the FP64 functions rounded to
// float whenever the pair-of-floats result is accepted, and reports how often
// the FP64 path is taken and the largest relative errors seen.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../mandelbrot-explorer_gb300/csrc/color_math.cuh"

using namespace mbx::cm;

int main(int argc, char** argv) {
    const long n = argc > 1 ? atol(argv[1]) : 1000000;
    const float density = argc > 2 ? (float)atof(argv[2]) : 60.0f;
    Exp2Table tab;
    make_exp2_table(tab);
    std::mt19937_64 g(12345);
    std::uniform_real_distribution<double> u(0.0, 7.0);
    long bad_log = 0, bad_pow = 0;
    int fb_log = 0, fb_pow = 0;
    double max_log = 0, max_pow = 0;
    for (long i = 0; i < n; ++i) {
        const float v = (float)(std::pow(10.0, u(g)) - 1.0);
        const float x = v + 2.0f;
        const ff l = log_ff(x);
        const long double tl = logl((long double)x);
        const double el = (double)fabsl(((long double)l.hi + l.lo - tl) / tl);
        if (el > max_log) max_log = el;
        const float L = logf_cr(x, fb_log);
        if (L != (float)std::log((double)x)) ++bad_log;
        const float e = L * L * density / 3600.0f;
        const ff p = exp_ff(ff_mul_f(log_ff(L), e), tab);
        const long double tp = powl((long double)L, (long double)e);
        const double ep = (double)fabsl(((long double)p.hi + p.lo - tp) / tp);
        if (ep > max_pow) max_pow = ep;
        const float P = powf_cr(L, e, tab, fb_pow);
        if (P != (float)std::pow((double)L, (double)e)) ++bad_pow;
    }
    printf("%ld %ld %ld %d %d %.6g %.6g\n", n, bad_log, bad_pow, fb_log, fb_pow, max_log, max_pow);
    return 0;
}

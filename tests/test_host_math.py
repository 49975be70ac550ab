"""Host-side arithmetic the device shares: the floatexp frexp/ldexp, the
restated libgcc complex division used for series-approximation seeding, and the
replica of glibc's rand() sequence. Compiled and checked against the C library
of the machine running the tests."""
import os
import subprocess
import tempfile

from conftest import PKG

PROGRAM = r"""
#include "floatexp.h"
#include "engine.h"
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <random>
using namespace mbx;
int main() {
    std::mt19937_64 g(11);
    std::uniform_real_distribution<double> u(-1, 1);
    std::uniform_int_distribution<int> ue(-1080, 1080), uk(-2200, 2200);
    long bad = 0;
    for (long i = 0; i < 3000000; ++i) {
        double x = std::ldexp(u(g), ue(g));
        int k = uk(g);
        if (dbits(std::ldexp(x, k)) != dbits(xldexp(x, k))) ++bad;
        int e1, e2;
        double f1 = std::frexp(x, &e1), f2 = xfrexp(x, &e2);
        if (dbits(f1) != dbits(f2) || (x != 0 && e1 != e2)) ++bad;
        double a = std::ldexp(u(g), ue(g) / 4), b = std::ldexp(u(g), ue(g) / 4), c = std::ldexp(u(g), ue(g) / 4), d = std::ldexp(u(g), ue(g) / 4);
        std::complex<double> z(a, b), w(c, d);
        z /= w;
        C2 q = c_div(c2(a, b), c2(c, d));
        double zr = z.real(), zi = z.imag();
        if (std::isfinite(zr) && std::isfinite(zi) && (dbits(zr) != dbits(q.re) || dbits(zi) != dbits(q.im))) ++bad;
    }
    // the exact loop's tests on bit patterns (d_is_zero, d_abs_less, d_eq,
    // d_le_zero) and its doubling (d_twice) give the IEEE results, NaN,
    // infinities, signed zeros and subnormals included
    const double sp[] = {0.0, -0.0, 1.0, -1.0, 5e-324, -5e-324, 2.2250738585072014e-308, 8.98846567431158e307, 1.7976931348623157e308,
                         -1.7976931348623157e308, INFINITY, -INFINITY, NAN, -NAN, 1e-8, 1e16, 1e-16, 0.5, 0.9999999999999999};
    std::uniform_int_distribution<uint64_t> ub;
    for (long i = 0; i < 4000000; ++i) {
        double a, b;
        if (i < 19 * 19) {
            a = sp[i / 19];
            b = sp[i % 19];
        } else {
            uint64_t x = ub(g), y = ub(g);
            if (i & 1) y = x ^ (ub(g) & 0xff); // near neighbours
            a = bitsd(x);
            b = bitsd(y);
            if (i & 2) b = std::fabs(b);
        }
        if (d_is_zero(a) != (a == 0.0)) ++bad;
        if (d_abs_less(a, b) != (std::fabs(a) < std::fabs(b))) ++bad;
        if (d_eq(a, b) != (a == b)) ++bad;
        if (d_le_zero(a) != (a <= 0.0)) ++bad;
        const double t = a + a;
        if (!std::isnan(a) && dbits(d_twice(a)) != dbits(t)) ++bad;
    }
    LibcRand r;
    r.seed(1);
    srand(1);
    for (int i = 0; i < 100000; ++i)
        if (r.next() != rand()) { ++bad; break; }
    printf("%ld\n", bad);
    return bad != 0;
}
"""


def test_floatexp_complex_and_rand_match_libc():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        open(src, "w").write(PROGRAM)
        csrc = os.path.join(PKG, "csrc")
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + csrc, "-I/usr/local/cuda/include", src, "-o", exe]
        subprocess.check_call(cmd)
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr


SPLIT_PROGRAM = r"""
#include "mixed_lane.cuh"
#include <cmath>
#include <cstdio>
#include <random>
using namespace mbx;
int main() {
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> u(0.5, 1.0);
    long bad = 0;
    for (long i = 0; i < 2000000; ++i) {
        const double m = u(g) * ((i & 1) ? -1.0 : 1.0);
        const int e = (int)(g() % 2001) - 1000;
        const TE<df32> t = te_from_fe_df(fe_make(m, e));
        const double v = ((double)t.m.hi + (double)t.m.lo) * std::ldexp(1.0, t.e - e);
        if (std::fabs(v - m) > std::ldexp(std::fabs(m), -48)) ++bad;               // the pair's 48 bits
        if (std::fabs(t.m.lo) > std::ldexp(std::fabs(t.m.hi), -24)) ++bad;         // a normalised pair
        if (std::fabs(t.m.hi) < 0.5f || std::fabs(t.m.hi) > 1.0f) ++bad;           // mantissa range
    }
    if (te_from_fe_df(fe_make(0.0, 7)).m.hi != 0.0f) ++bad;
    printf("%ld\n", bad);
    return bad != 0;
}
"""


def test_floatexp_to_double_float_split():
    """The double-float lane's orbit-entry steps read FE orbit entries as
    double-float floatexp (mixed_lane.cuh te_from_fe_df: the 53-bit mantissa
    split on its bit pattern, no FP64 instruction): the pair must hold the
    mantissa to the double-float's 48 bits, normalised, with the exponent
    carried."""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        open(src, "w").write(SPLIT_PROGRAM)
        csrc = os.path.join(PKG, "csrc")
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wno-deprecated-declarations", "-I" + csrc, "-I/usr/local/cuda/include", src, "-o", exe]
        subprocess.check_call(cmd)
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout + out.stderr


def test_threaded_nucleus_search_matches_serial_oracle():
    """mbx_find_nucleus runs the period search and the Newton orbit on three
    threads between 1000 and 1600/2000 bits (ring-buffered recurrences), and
    above as parallel rounds of products (seven per period-search step, its
    containment test one step behind); the nucleus must equal, digit for digit,
    the serial reference algorithm's (oracle: mp.cpp:116-223), and so must a
    search whose Newton leaves the disk."""
    import mbx
    import oracle
    import views

    v = views.deep_view(1000)
    for digits, radius, prec in ((500, "1e-330", 1300), (400, "1e-300", 1200), (700, "1e-500", 2200)):
        cx, cy = v["center_re"][:digits], v["center_im"][:digits]
        got = mbx.find_nucleus(cx, cy, radius, 100000, prec)
        want = oracle.nucleus(cx, cy, radius, 100000, prec)
        if want is None:
            assert got is None
            continue
        from decimal import Decimal

        assert got is not None and got[0] == want[0]
        assert Decimal(got[1]) == want[1] and Decimal(got[2]) == want[2]

// Frame dumper around the reference engine, compiled only in the build
// container by oracle/ref_build/Makefile (the reference sources are read in
// place and never copied). It runs Mandel::Compute exactly as the reference's
// own verify/render tools do and writes the raw float32 iteration buffer
// (plus the DE-overlay buffer when requested) for parity fixtures.
//
// usage: mbx_refdump <cx> <cy> <scale-digits> <W> <H> <mxit> <sub> <cmethod>
//                    <out.f32> [full_h row_base] [--time trials] [--julia <cre> <cim>]
// With --julia the frame is Mandel::ComputeJulia for the fixed c (cre, cim).
// Precision rule of src/tools/verify.cpp:runCase: bits = digits*log2(10)+64.
#include <gmp.h>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mandel_perturbation.h"

int main(int argc, char** argv) {
    if (argc < 10) {
        fprintf(stderr, "usage: mbx_refdump cx cy scale W H mxit sub cmethod out [full_h row_base] [--time trials]\n");
        return 2;
    }
    const char* cx = argv[1];
    const char* cy = argv[2];
    std::string scale = argv[3];
    int W = atoi(argv[4]), H = atoi(argv[5]), mxit = atoi(argv[6]), sub = atoi(argv[7]);
    int cmethod = atoi(argv[8]);
    const char* out = argv[9];
    int full_h = 0, row_base = 0, trials = 0;
    int a = 10;
    if (argc > 11 && strncmp(argv[10], "--", 2) != 0) {
        full_h = atoi(argv[10]);
        row_base = atoi(argv[11]);
        a = 12;
    }
    if (argc > a + 1 && strcmp(argv[a], "--time") == 0) {
        trials = atoi(argv[a + 1]);
        a += 2;
    }
    const char* jre = nullptr;
    const char* jim = nullptr;
    if (argc > a + 2 && strcmp(argv[a], "--julia") == 0) {
        jre = argv[a + 1];
        jim = argv[a + 2];
    }
    int precision = (int)(scale.size() * log(10) / log(2)) + 64;
    if (const char* e = getenv("MANDEL_PREC")) precision = (int)(atol(e) * 3.3219281 + 64.0);
    mpf_set_default_prec(precision);
    mpf_t mcx, mcy, msc;
    mpf_init_set_str(mcx, cx, 10);
    mpf_init_set_str(mcy, cy, 10);
    mpf_init_set_str(msc, scale.c_str(), 10);
    const size_t n = (size_t)W * H * sub * sub;
    std::vector<float> iter(n, EMPTYPIXEL), normal(n, 0.0f);
    double best = 1e300;
    int runs = trials > 0 ? trials : 1;
    for (int t = 0; t < runs; ++t) {
        std::fill(iter.begin(), iter.end(), EMPTYPIXEL);
        std::fill(normal.begin(), normal.end(), 0.0f);
        Mandel m(W, H, mxit, sub, iter.data());
        m.setPrecision(precision);
        if (cmethod & (ColoringMethod::DE_OVERLAY | ColoringMethod::NORMAL_MAP)) m.setNormalBuffer(normal.data());
        auto t0 = std::chrono::steady_clock::now();
        if (jre) {
            mpf_t fr, fi;
            mpf_init_set_str(fr, jre, 10);
            mpf_init_set_str(fi, jim, 10);
            m.ComputeJulia(mcx, mcy, msc, fr, fi, mxit, cmethod, full_h, row_base);
            mpf_clear(fr);
            mpf_clear(fi);
        } else {
            m.Compute(mcx, mcy, msc, mxit, cmethod, full_h, row_base);
        }
        double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (s < best) best = s;
    }
    if (trials > 0) fprintf(stderr, "MBX_REF_TIME %.6f\n", best);
    FILE* f = fopen(out, "wb");
    if (!f) return 3;
    fwrite(iter.data(), sizeof(float), n, f);
    if (cmethod & (ColoringMethod::DE_OVERLAY | ColoringMethod::NORMAL_MAP)) fwrite(normal.data(), sizeof(float), n, f);
    fclose(f);
    mpf_clear(mcx);
    mpf_clear(mcy);
    mpf_clear(msc);
    return 0;
}

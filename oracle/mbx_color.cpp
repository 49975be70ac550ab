// ORACLE — test infrastructure only. CPU restatement of the reference's image
// epilogue (cbotx/Mandelbrot-Explorer src/tools/render.cpp with
// src/engine/interpolate.cpp): palette from six control points by monotone
// cubic interpolation, the value-to-palette mappings, linear-light box
// downsample of a supersampled frame, relief / normal-map / distance-overlay
// shading, gamma encode and the 24-bit BMP writer. Only tests/ and the CPU legs
// of bench.py may load it; the product never does.
//
// Pinning: tests/golden/make_color_golden.py runs the reference's own render
// tool (compiled in place by oracle/ref_build) and keeps its BMP files next to
// the engine values it coloured; tests require this file to reproduce every
// BMP byte for byte. Compiled with -ffp-contract=off, so the operation order
// written below is the order executed; float/double promotions are spelled out
// where the reference relies on C++'s usual arithmetic conversions.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int kPalette = 2048; // render.cpp:20 colP

// interpolate.cpp:7-60 mono_cubic_interpolate: segment slopes, tangents that
// vanish at slope sign changes (harmonic-type blend elsewhere), cubic Hermite
// coefficients per segment, evaluated at i / m for i in [0, m).
void mono_cubic(const float* xs, const float* ys, int n, float* out, int m) {
    std::vector<float> dx(n - 1), slope(n - 1), tan(n), q2(n - 1), q3(n - 1);
    for (int k = 0; k + 1 < n; ++k) {
        dx[k] = xs[k + 1] - xs[k];
        const float dy = ys[k + 1] - ys[k];
        slope[k] = dy / dx[k];
    }
    tan[0] = slope[0];
    for (int k = 0; k + 2 < n; ++k) {
        const float s0 = slope[k], s1 = slope[k + 1];
        if (s0 * s1 <= 0) {
            tan[k + 1] = 0;
        } else {
            const float span = dx[k] + dx[k + 1];
            tan[k + 1] = 3 * span / ((span + dx[k + 1]) / s0 + (span + dx[k]) / s1);
        }
    }
    tan[n - 1] = slope[n - 2];
    for (int k = 0; k + 1 < n; ++k) {
        const float inv = 1 / dx[k];
        const float c = tan[k] + tan[k + 1] - slope[k] - slope[k];
        q2[k] = (slope[k] - tan[k] - c) * inv;
        q3[k] = c * inv * inv;
    }
    for (int i = 0; i < m; ++i) {
        const float x = 1.f * i / m;
        float y;
        if (x == xs[n - 1]) {
            y = ys[n - 1];
        } else {
            int lo = 0, hi = n - 2, hit = -1;
            while (lo <= hi) {
                const int mid = (lo + hi) / 2;
                if (xs[mid] < x) lo = mid + 1;
                else if (xs[mid] > x) hi = mid - 1;
                else {
                    hit = mid;
                    break;
                }
            }
            if (hit >= 0) {
                y = ys[hit];
            } else {
                const int k = hi > 0 ? hi : 0;
                const float d = x - xs[k], d2 = d * d;
                y = ys[k] + tan[k] * d + q2[k] * d2 + q3[k] * d * d2;
            }
        }
        out[i] = y;
    }
}

// render.cpp:23-29: Ultra-Fractal-style control points per channel.
void palette(float* map /* [3][kPalette] */) {
    static const float pos[6] = {0.0f, 0.16f, 0.42f, 0.6425f, 0.8575f, 1.0f};
    static const float col[3][6] = {{0, 32, 237, 255, 0, 0}, {70, 107, 255, 170, 2, 70}, {100, 203, 255, 0, 0, 100}};
    for (int c = 0; c < 3; ++c) mono_cubic(pos, col[c], 6, map + c * kPalette, kPalette);
}

struct Params {
    int ss, mapping, shading;
    float density;
    double az, el, relief, de_k;
};
enum { MAP_LOG_POWER = 0, MAP_EDE = 1, MAP_SAC = 2, MAP_TRAP = 3 };
enum { SHADE_NONE = 0, SHADE_RELIEF = 1, SHADE_NORMAL = 2, SHADE_DE_OVERLAY = 3 };

// render.cpp:71-92 getColor (with color_func, render.cpp:31-33).
void lookup(const float* map, const Params& p, float v, float& r, float& g, float& b) {
    if (v < 0) {
        r = g = b = 0;
        return;
    }
    float f;
    if (p.mapping == MAP_SAC) {
        f = v * (p.density / 20.0f);
    } else if (p.mapping == MAP_EDE) {
        f = tanhf(v * p.density / 3600.0f * 5.0f);
    } else if (p.mapping == MAP_TRAP) {
        f = v;
    } else {
        const float l = logf(v + 2);
        f = powf(l, logf(v + 2) * logf(v + 2) * p.density / 3600.0f);
    }
    int x = (int)(f * kPalette) % kPalette;
    if (x < 0) x += kPalette;
    r = map[x];
    g = map[kPalette + x];
    b = map[2 * kPalette + x];
}

inline float to_linear(float c) { return powf(c / 255.f, 2.2f); }                      // render.cpp:94-96
inline float to_gamma(float l) { return 255.f * powf(l < 0 ? 0 : l, 1.f / 2.2f); }     // render.cpp:97-99

// render.cpp:47-69 reliefShadeAt: screen-space gradient of the value, Lambert
// against the light direction, ambient 0.25 + diffuse 0.85.
float relief_shade(const float* v, int y, int x, int ws, int hs, const Params& p) {
    const float c = v[(size_t)y * ws + x];
    if (c < 0) return 1.0f;
    auto at = [&](int yy, int xx) -> float {
        if (xx < 0 || xx >= ws || yy < 0 || yy >= hs) return c;
        const float q = v[(size_t)yy * ws + xx];
        return q < 0 ? c : q;
    };
    const float sx = (at(y, x + 1) - at(y, x - 1)) * 0.5f;
    const float sy = (at(y + 1, x) - at(y - 1, x)) * 0.5f;
    const double nx = (double)(-sx) * p.relief, ny = (double)(-sy) * p.relief, nz = 1.0;
    const double inv = 1.0 / std::sqrt(nx * nx + ny * ny + nz * nz);
    const double lx = std::cos(p.el) * std::cos(p.az);
    const double ly = std::cos(p.el) * std::sin(p.az);
    const double lz = std::sin(p.el);
    double d = (nx * lx + ny * ly + nz * lz) * inv;
    if (d < 0) d = 0;
    return (float)(0.25 + 0.85 * d);
}

// render.cpp:276-287: Lambert shade from the normal-map angle.
float normal_shade(float ang, const Params& p) {
    const double nx = std::cos((double)ang), ny = std::sin((double)ang), nz = 1.0;
    const double inv = 1.0 / std::sqrt(nx * nx + ny * ny + nz * nz);
    const double lx = std::cos(p.el) * std::cos(p.az);
    const double ly = std::cos(p.el) * std::sin(p.az);
    const double lz = std::sin(p.el);
    double d = (nx * lx + ny * ly + nz * lz) * inv;
    if (d < 0) d = 0;
    return (float)(0.3 + 0.8 * d);
}

// The float-to-byte store of render.cpp:297-299 on the reference's platform:
// truncation to a 32-bit integer, low byte kept.
inline uint8_t to_byte(float x) { return (uint8_t)(int32_t)x; }

} // namespace

extern "C" {

// Palette as three 2048-entry float channels (render.cpp:23-29).
void mbx_oracle_palette(float* map) { palette(map); }

// render.cpp:248-300: colour each of the (width*ss) x (height*ss) values,
// average ss x ss blocks in linear light, gamma-encode into rgb[height][width][3].
// aux: the normal-map angles (shading 2) or the distance-overlay buffer (shading 3).
int mbx_oracle_colorize(const float* values, const float* aux, int width, int height, int ss, int mapping, int shading, float density,
                        double light_az, double light_el, double relief_strength, double de_k, uint8_t* rgb) {
    if (width < 1 || height < 1 || ss < 1 || mapping < 0 || mapping > 3 || shading < 0 || shading > 3) return -1;
    if ((shading == SHADE_NORMAL || shading == SHADE_DE_OVERLAY) && !aux) return -1;
    const Params p = {ss, mapping, shading, density, light_az, light_el, relief_strength, de_k};
    std::vector<float> map(3 * kPalette);
    palette(map.data());
    const int ws = width * ss, hs = height * ss;
#pragma omp parallel for schedule(dynamic, 8)
    for (int i = 0; i < height; ++i)
        for (int j = 0; j < width; ++j) {
            float lr = 0, lg = 0, lb = 0;
            for (int a = 0; a < ss; ++a)
                for (int b = 0; b < ss; ++b) {
                    const int yy = i * ss + a, xx = j * ss + b;
                    const size_t k = (size_t)yy * ws + xx;
                    float r, g, bl;
                    lookup(map.data(), p, values[k], r, g, bl);
                    const double cr = to_linear(r), cg = to_linear(g), cb = to_linear(bl);
                    if (shading == SHADE_DE_OVERLAY) {
                        const double de = aux[k];
                        const double bw = de / (de + p.de_k);
                        const double gray = bw, cw = bw * bw;
                        lr = (float)((double)lr + (cr * cw + gray * (1.0 - cw)));
                        lg = (float)((double)lg + (cg * cw + gray * (1.0 - cw)));
                        lb = (float)((double)lb + (cb * cw + gray * (1.0 - cw)));
                        continue;
                    }
                    float sh = 1.0f;
                    if (shading == SHADE_NORMAL) sh = normal_shade(aux[k], p);
                    else if (shading == SHADE_RELIEF) sh = relief_shade(values, yy, xx, ws, hs, p);
                    lr = (float)((double)lr + cr * (double)sh);
                    lg = (float)((double)lg + cg * (double)sh);
                    lb = (float)((double)lb + cb * (double)sh);
                }
            const int n = ss * ss;
            uint8_t* px = rgb + ((size_t)i * width + j) * 3;
            px[0] = to_byte(to_gamma(lr / n) + 0.5f);
            px[1] = to_byte(to_gamma(lg / n) + 0.5f);
            px[2] = to_byte(to_gamma(lb / n) + 0.5f);
        }
    return 0;
}

// The integer the reference's byte store sees for a linear value l
// (render.cpp:97-99, 297): (int)(255 powf(l, 1/2.2) + 0.5).
void mbx_oracle_gamma_value(const float* l, int n, int32_t* out) {
    for (int i = 0; i < n; ++i) out[i] = (int32_t)(to_gamma(l[i]) + 0.5f);
}

// render.cpp:101-137 writeBMP into a buffer: 14-byte file header, 40-byte
// BITMAPINFOHEADER, bottom-up BGR rows padded to 4 bytes. Returns the size;
// out may be NULL to query it.
long mbx_oracle_bmp(const uint8_t* rgb, int width, int height, uint8_t* out) {
    const long row = (width * 3 + 3) & ~3;
    const long size = 54 + row * height;
    if (!out) return size;
    memset(out, 0, (size_t)size);
    auto put32 = [&](long at, uint32_t v) { memcpy(out + at, &v, 4); };
    auto put16 = [&](long at, uint16_t v) { memcpy(out + at, &v, 2); };
    out[0] = 'B';
    out[1] = 'M';
    put32(2, (uint32_t)size);
    put32(10, 54);
    put32(14, 40);
    put32(18, (uint32_t)width);
    put32(22, (uint32_t)height);
    put16(26, 1);
    put16(28, 24);
    put32(34, (uint32_t)(row * height));
    for (int y = 0; y < height; ++y) {
        uint8_t* line = out + 54 + (long)(height - 1 - y) * row;
        for (int x = 0; x < width; ++x) {
            const uint8_t* px = rgb + ((size_t)y * width + x) * 3;
            line[x * 3 + 0] = px[2];
            line[x * 3 + 1] = px[1];
            line[x * 3 + 2] = px[0];
        }
    }
    return size;
}

} // extern "C"

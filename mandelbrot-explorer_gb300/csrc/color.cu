// Image epilogue on the device (color.h). One thread per output pixel walks
// its ss x ss values: palette coordinate (render.cpp:71-92), linear-light
// palette entry, per-sample shade, running float sum in the reference's
// promotion order, then the gamma-encoded byte (render.cpp:248-300).
//
// Exactness: every float and double operation below is the reference's
// operation on the same operands, written with round-to-nearest intrinsics so
// that nothing is contracted. The libm calls of the reference become: the
// correctly rounded pair-of-floats log/pow of color_math.cuh (the reference's
// logf/powf are correctly rounded on all but ~1e-4 of inputs); tables built on
// the host with the host's libm for the functions of the palette entry
// (powf(c/255, 2.2)) and of the final byte (a monotone step function of the
// linear value, stored as its 352 step positions); the FP64 library tanh, cos,
// sin and sqrt for the distance mapping and the two shadings.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "color.h"

namespace mbx {

namespace {

// interpolate.cpp:7-60 (monotone cubic through the control points, sampled at
// i / m), written out with the reference's float operation order.
void mono_cubic(const float* xs, const float* ys, int n, float* out, int m) {
    std::vector<float> dx(n - 1), slope(n - 1), tan(n), q2(n - 1), q3(n - 1);
    for (int k = 0; k + 1 < n; ++k) {
        dx[k] = xs[k + 1] - xs[k];
        slope[k] = (ys[k + 1] - ys[k]) / dx[k];
    }
    tan[0] = slope[0];
    for (int k = 0; k + 2 < n; ++k) {
        if (slope[k] * slope[k + 1] <= 0) {
            tan[k + 1] = 0;
        } else {
            const float span = dx[k] + dx[k + 1];
            tan[k + 1] = 3 * span / ((span + dx[k + 1]) / slope[k] + (span + dx[k]) / slope[k + 1]);
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
        if (x == xs[n - 1]) {
            out[i] = ys[n - 1];
            continue;
        }
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
            out[i] = ys[hit];
        } else {
            const int k = hi > 0 ? hi : 0;
            const float d = x - xs[k], d2 = d * d;
            out[i] = ys[k] + tan[k] * d + q2[k] * d2 + q3[k] * d * d2;
        }
    }
}

int32_t gamma_value(float l) { return (int32_t)(255.f * powf(l < 0 ? 0 : l, 1.f / 2.2f) + 0.5f); } // render.cpp:97-99, 297

float bits_to_float(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

} // namespace

void build_palette(float* map) { // render.cpp:23-29
    static const float pos[6] = {0.0f, 0.16f, 0.42f, 0.6425f, 0.8575f, 1.0f};
    static const float col[3][6] = {{0, 32, 237, 255, 0, 0}, {70, 107, 255, 170, 2, 70}, {100, 203, 255, 0, 0, 100}};
    for (int c = 0; c < 3; ++c) mono_cubic(pos, col[c], 6, map + c * kPaletteSize, kPaletteSize);
}

void build_color_tables(ColorTables& t) {
    std::vector<float> map(3 * kPaletteSize);
    build_palette(map.data());
    for (int i = 0; i < kPaletteSize; ++i)
        t.lin[i] = make_float4(powf(map[i] / 255.f, 2.2f), powf(map[kPaletteSize + i] / 255.f, 2.2f), powf(map[2 * kPaletteSize + i] / 255.f, 2.2f), 0.0f);
    // Least l in [0, 4] (ordered as its bit pattern) with gamma_value(l) >= k.
    const uint32_t top = 0x40800000u; // 4.0f
    for (int k = 1; k <= kGammaSteps; ++k) {
        uint32_t lo = 0, hi = top;
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (gamma_value(bits_to_float(mid)) >= k) hi = mid;
            else lo = mid + 1;
        }
        t.gamma[k - 1] = bits_to_float(lo);
    }
    cm::make_exp2_table(t.exp2);
}

namespace {

// (int) of a float as the reference's x86-64 build converts it: out-of-range
// and NaN give INT_MIN (render.cpp:89 on values past 2^31 / 2048).
__device__ __forceinline__ int trunc_i32(float y) { return fabsf(y) < 2147483648.0f ? (int)y : (int)0x80000000u; }

__device__ __forceinline__ int palette_index(float v, int mapping, float density, const cm::Exp2Table& tab, int& fb) {
    float f;
    if (mapping == MBX_MAP_STRIPE) {
        f = cm::mul(v, cm::div(density, 20.0f));
    } else if (mapping == MBX_MAP_DISTANCE) {
        const float t = cm::mul(cm::div(cm::mul(v, density), 3600.0f), 5.0f);
        f = __double2float_rn(tanh((double)t));
    } else if (mapping == MBX_MAP_TRAP) {
        f = v;
    } else {
        if (!(v <= FLT_MAX)) return 0; // +inf / NaN: the reference's conversion yields INT_MIN % 2048 = 0
        const float x = cm::add(v, 2.0f);
        const float L = cm::logf_cr(x, fb);
        const float e = cm::div(cm::mul(cm::mul(L, L), density), 3600.0f);
        f = cm::powf_cr(L, e, tab, fb);
    }
    int i = trunc_i32(cm::mul(f, (float)kPaletteSize)) % kPaletteSize;
    if (i < 0) i += kPaletteSize;
    return i;
}

// render.cpp:47-69 on the supersampled grid.
__device__ float relief_shade(const float* __restrict__ v, int y, int x, int ws, int hs, double strength, double lx, double ly, double lz) {
    const float c = v[(size_t)y * ws + x];
    if (c < 0) return 1.0f;
    auto at = [&](int yy, int xx) -> float {
        if (xx < 0 || xx >= ws || yy < 0 || yy >= hs) return c;
        const float q = v[(size_t)yy * ws + xx];
        return q < 0 ? c : q;
    };
    const float sx = cm::mul(cm::sub(at(y, x + 1), at(y, x - 1)), 0.5f);
    const float sy = cm::mul(cm::sub(at(y + 1, x), at(y - 1, x)), 0.5f);
    const double nx = __dmul_rn((double)(-sx), strength), ny = __dmul_rn((double)(-sy), strength);
    const double inv = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nx, nx), __dmul_rn(ny, ny)), 1.0)));
    double d = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(nx, lx), __dmul_rn(ny, ly)), lz), inv);
    if (d < 0) d = 0;
    return __double2float_rn(__dadd_rn(0.25, __dmul_rn(0.85, d)));
}

// render.cpp:276-287.
__device__ float normal_shade(float ang, double lx, double ly, double lz) {
    const double nx = cos((double)ang), ny = sin((double)ang);
    const double inv = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nx, nx), __dmul_rn(ny, ny)), 1.0)));
    double d = __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(nx, lx), __dmul_rn(ny, ly)), lz), inv);
    if (d < 0) d = 0;
    return __double2float_rn(__dadd_rn(0.3, __dmul_rn(0.8, d)));
}

__device__ __forceinline__ float acc_shaded(float acc, float c, float sh) { // acc += (double)c * sh in double, stored to float
    return __double2float_rn(__dadd_rn((double)acc, __dmul_rn((double)c, (double)sh)));
}

__device__ __forceinline__ int gamma_byte(float l, const float* s_gamma) {
    int lo = 0, hi = kGammaSteps; // number of thresholds <= l
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s_gamma[mid] <= l) lo = mid + 1;
        else hi = mid;
    }
    return lo & 0xff; // (uint8_t)(int32_t)(...) of render.cpp:297-299
}

constexpr int kColorThreads = 256;

__global__ void __launch_bounds__(kColorThreads) k_colorize(ColorLaunch a) {
    __shared__ float s_gamma[kGammaSteps];
    __shared__ cm::Exp2Table s_exp2;
    for (int i = threadIdx.x; i < kGammaSteps; i += blockDim.x) s_gamma[i] = a.tables->gamma[i];
    if (threadIdx.x < 32) {
        s_exp2.hi[threadIdx.x] = a.tables->exp2.hi[threadIdx.x];
        s_exp2.lo[threadIdx.x] = a.tables->exp2.lo[threadIdx.x];
    }
    __syncthreads();
    const float4* __restrict__ lin = a.tables->lin;
    const float* __restrict__ values = a.values;
    const float* __restrict__ aux = a.aux;
    const int ss = a.ss, ws = a.width * ss, hs = a.height * ss;
    const long long npix = (long long)a.width * a.height;
    int fb = 0;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(p / a.width), j = (int)(p - (long long)i * a.width);
        float lr = 0.0f, lg = 0.0f, lb = 0.0f;
        for (int sa = 0; sa < ss; ++sa)
            for (int sb = 0; sb < ss; ++sb) {
                const int yy = i * ss + sa, xx = j * ss + sb;
                const size_t k = (size_t)yy * ws + xx;
                const float v = __ldg(values + k);
                float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f); // interior: black (render.cpp:72-75)
                if (!(v < 0)) c = __ldg(lin + palette_index(v, a.mapping, a.density, s_exp2, fb));
                if (a.shading == MBX_SHADE_DE_OVERLAY) {
                    const double de = (double)__ldg(aux + k);
                    const double bw = __ddiv_rn(de, __dadd_rn(de, a.de_k));
                    const double cw = __dmul_rn(bw, bw), om = __dsub_rn(1.0, cw), g = __dmul_rn(bw, om);
                    lr = __double2float_rn(__dadd_rn((double)lr, __dadd_rn(__dmul_rn((double)c.x, cw), g)));
                    lg = __double2float_rn(__dadd_rn((double)lg, __dadd_rn(__dmul_rn((double)c.y, cw), g)));
                    lb = __double2float_rn(__dadd_rn((double)lb, __dadd_rn(__dmul_rn((double)c.z, cw), g)));
                } else if (a.shading == MBX_SHADE_NONE) {
                    // (float)((double)acc + (double)c * 1.0): the double sum of two
                    // floats rounds to float exactly as the float sum does
                    lr = cm::add(lr, c.x);
                    lg = cm::add(lg, c.y);
                    lb = cm::add(lb, c.z);
                } else {
                    const float sh = a.shading == MBX_SHADE_NORMAL_MAP ? normal_shade(__ldg(aux + k), a.lx, a.ly, a.lz)
                                                                       : relief_shade(values, yy, xx, ws, hs, a.relief, a.lx, a.ly, a.lz);
                    lr = acc_shaded(lr, c.x, sh);
                    lg = acc_shaded(lg, c.y, sh);
                    lb = acc_shaded(lb, c.z, sh);
                }
            }
        const float n = (float)(ss * ss);
        uint8_t* px = a.rgb + (size_t)p * 3;
        px[0] = (uint8_t)gamma_byte(cm::div(lr, n), s_gamma);
        px[1] = (uint8_t)gamma_byte(cm::div(lg, n), s_gamma);
        px[2] = (uint8_t)gamma_byte(cm::div(lb, n), s_gamma);
    }
    if (fb) atomicAdd(a.fallbacks, (unsigned)fb);
}

} // namespace

cudaError_t launch_colorize(const ColorLaunch& a, int nsm, cudaStream_t st) {
    const long long npix = (long long)a.width * a.height;
    long long blocks = (npix + kColorThreads - 1) / kColorThreads;
    const long long cap = (long long)nsm * 8; // eight resident blocks per SM, grid-stride beyond
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    k_colorize<<<(unsigned)blocks, kColorThreads, 0, st>>>(a);
    return cudaGetLastError();
}

int validate_color_params(const mbx_color_params* p, std::string& why) {
    if (!p) why = "null colour parameters";
    else if (p->supersample < 1 || p->supersample > 64) why = "supersample must be in [1, 64]";
    else if (p->mapping < MBX_MAP_LOG_POWER || p->mapping > MBX_MAP_TRAP) why = "unknown colour mapping";
    else if (p->shading < MBX_SHADE_NONE || p->shading > MBX_SHADE_DE_OVERLAY) why = "unknown shading";
    else if (!(p->density > 0.0f) || !(p->density < 1e6f)) why = "density must be in (0, 1e6)";
    else if (!std::isfinite(p->light_az) || !std::isfinite(p->light_el) || !std::isfinite(p->relief_strength) || !std::isfinite(p->de_k)) why = "light, relief and overlay parameters must be finite";
    else return MBX_OK;
    return MBX_E_INVALID;
}

Colorizer::~Colorizer() {
    for (void* q : {(void*)d_tables_, (void*)d_fallbacks_, (void*)d_values_, (void*)d_aux_, (void*)d_rgb_})
        if (q) cudaFree(q);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
}

int Colorizer::ensure(size_t samples, size_t pixels, bool need_aux, std::string& err) {
    if (!d_tables_) {
        ColorTables* h = new (std::nothrow) ColorTables();
        if (!h) return MBX_E_NOMEM;
        build_color_tables(*h);
        cudaError_t e = cudaMalloc(&d_tables_, sizeof(ColorTables));
        if (e == cudaSuccess) e = cudaMemcpy(d_tables_, h, sizeof(ColorTables), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&d_fallbacks_, sizeof(unsigned));
        if (e == cudaSuccess) e = cudaEventCreate(&ev0_);
        if (e == cudaSuccess) e = cudaEventCreate(&ev1_);
        delete h;
        if (e != cudaSuccess) {
            err = std::string("colour tables: ") + cudaGetErrorString(e);
            return MBX_E_CUDA;
        }
    }
    if (samples > cap_samples_ || (need_aux && (!cap_aux_ || samples > cap_samples_))) {
        if (d_values_) cudaFree(d_values_);
        if (d_aux_) cudaFree(d_aux_);
        d_values_ = nullptr;
        d_aux_ = nullptr;
        cap_samples_ = 0;
        cap_aux_ = false;
        if (cudaMalloc(&d_values_, samples * sizeof(float)) != cudaSuccess || (need_aux && cudaMalloc(&d_aux_, samples * sizeof(float)) != cudaSuccess)) {
            err = "colour staging buffers";
            return MBX_E_NOMEM;
        }
        cap_samples_ = samples;
        cap_aux_ = need_aux;
    }
    if (pixels > cap_pixels_) {
        if (d_rgb_) cudaFree(d_rgb_);
        d_rgb_ = nullptr;
        cap_pixels_ = 0;
        if (cudaMalloc(&d_rgb_, pixels * 3) != cudaSuccess) {
            err = "colour output buffer";
            return MBX_E_NOMEM;
        }
        cap_pixels_ = pixels;
    }
    return MBX_OK;
}

int Colorizer::device_buffers(size_t samples, size_t pixels, bool need_aux, float** values, float** aux, uint8_t** rgb, std::string& err) {
    const int rc = ensure(samples, pixels, need_aux, err);
    if (rc != MBX_OK) return rc;
    *values = d_values_;
    *aux = need_aux ? d_aux_ : nullptr;
    *rgb = d_rgb_;
    return MBX_OK;
}

int Colorizer::colorize(const mbx_color_params& p, const float* values, const float* aux, int width, int height, bool on_device, uint8_t* rgb,
                        cudaStream_t st, int nsm, std::string& err, unsigned* fallbacks_out, float* gpu_ms) {
    const bool need_aux = p.shading == MBX_SHADE_NORMAL_MAP || p.shading == MBX_SHADE_DE_OVERLAY;
    if (!values || !rgb || (need_aux && !aux)) {
        err = need_aux && !aux ? "this shading needs the aux buffer" : "missing values or rgb buffer";
        return MBX_E_INVALID;
    }
    if (width < 1 || height < 1 || (long long)width * p.supersample * height * p.supersample > (1ll << 31) - 1) {
        err = "image dimensions out of range";
        return MBX_E_INVALID;
    }
    const size_t samples = (size_t)width * p.supersample * height * p.supersample, pixels = (size_t)width * height;
    int rc = ensure(on_device ? 0 : samples, on_device ? 0 : pixels, !on_device && need_aux, err);
    if (rc != MBX_OK) return rc;
    ColorLaunch a{};
    a.values = on_device ? values : d_values_;
    a.aux = need_aux ? (on_device ? aux : d_aux_) : nullptr;
    a.rgb = on_device ? rgb : d_rgb_;
    a.width = width;
    a.height = height;
    a.ss = p.supersample;
    a.mapping = p.mapping;
    a.shading = p.shading;
    a.density = p.density;
    a.relief = p.relief_strength;
    a.de_k = p.de_k;
    // the light vector of render.cpp:59-61 / 283-285, from the host libm
    a.lx = std::cos(p.light_el) * std::cos(p.light_az);
    a.ly = std::cos(p.light_el) * std::sin(p.light_az);
    a.lz = std::sin(p.light_el);
    a.tables = d_tables_;
    a.fallbacks = d_fallbacks_;
    cudaError_t e = cudaMemsetAsync(d_fallbacks_, 0, sizeof(unsigned), st);
    if (!on_device) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_values_, values, samples * sizeof(float), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && need_aux) e = cudaMemcpyAsync(d_aux_, aux, samples * sizeof(float), cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev0_, st);
    if (e == cudaSuccess) e = launch_colorize(a, nsm, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev1_, st);
    if (e == cudaSuccess && !on_device) e = cudaMemcpyAsync(rgb, d_rgb_, pixels * 3, cudaMemcpyDeviceToHost, st);
    unsigned fb = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&fb, d_fallbacks_, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        err = std::string("colorize: ") + cudaGetErrorString(e);
        return MBX_E_CUDA;
    }
    if (fallbacks_out) *fallbacks_out = fb;
    if (gpu_ms) cudaEventElapsedTime(gpu_ms, ev0_, ev1_);
    return MBX_OK;
}

int write_bmp(const char* path, const uint8_t* rgb, int width, int height) { // render.cpp:101-137
    if (!path || !rgb || width < 1 || height < 1 || width > (1 << 24) || height > (1 << 24)) return MBX_E_INVALID;
    const long long row = ((long long)width * 3 + 3) & ~3ll;
    const long long data = row * height;
    if (54 + data > 0xffffffffll) return MBX_E_TOO_LARGE;
    uint8_t head[54] = {'B', 'M'};
    auto put32 = [&](int at, uint32_t v) { memcpy(head + at, &v, 4); };
    auto put16 = [&](int at, uint16_t v) { memcpy(head + at, &v, 2); };
    put32(2, (uint32_t)(54 + data));
    put32(10, 54);
    put32(14, 40);
    put32(18, (uint32_t)width);
    put32(22, (uint32_t)height);
    put16(26, 1);
    put16(28, 24);
    put32(34, (uint32_t)data);
    FILE* f = fopen(path, "wb");
    if (!f) return MBX_E_INVALID;
    bool ok = fwrite(head, 1, 54, f) == 54;
    std::vector<uint8_t> line((size_t)row, 0);
    for (int y = height - 1; y >= 0 && ok; --y) { // bottom-up, BGR
        const uint8_t* src = rgb + (size_t)y * width * 3;
        for (int x = 0; x < width; ++x) {
            line[(size_t)x * 3 + 0] = src[(size_t)x * 3 + 2];
            line[(size_t)x * 3 + 1] = src[(size_t)x * 3 + 1];
            line[(size_t)x * 3 + 2] = src[(size_t)x * 3 + 0];
        }
        ok = fwrite(line.data(), 1, (size_t)row, f) == (size_t)row;
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? MBX_OK : MBX_E_INVALID;
}

} // namespace mbx

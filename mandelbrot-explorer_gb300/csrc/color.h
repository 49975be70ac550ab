// Image epilogue: the reference's render-tool colouring (src/tools/render.cpp:
// palette, value mapping, linear-light supersample downsample, shading, gamma)
// as one device pass from the value buffer to packed 8-bit RGB, plus the BMP
// writer (render.cpp:101-137).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mbx_gb300.h"
#include "color_math.cuh"

namespace mbx {

constexpr int kPaletteSize = 2048;  // render.cpp:20 colP
constexpr int kGammaSteps = 352;    // thresholds of the gamma-encoded value 1..352 (linear light up to 2)

// Tables the kernel reads; built once on the host from the host's libm, the
// same functions the reference calls for them.
struct ColorTables {
    float4 lin[kPaletteSize];   // powf(palette/255, 2.2) per channel (render.cpp:94-96)
    float gamma[kGammaSteps];   // gamma[k-1] = least l with (int)(255 powf(l, 1/2.2) + 0.5) >= k
    cm::Exp2Table exp2;
};
void build_color_tables(ColorTables& t);
void build_palette(float* map /* [3][2048] */);

struct ColorLaunch {
    const float* values;   // (width*ss) x (height*ss)
    const float* aux;      // normal-map angles or distance-overlay values, same layout
    uint8_t* rgb;          // height x width x 3
    int width, height, ss;
    int mapping, shading;
    float density;
    double relief, de_k, lx, ly, lz;
    const ColorTables* tables;   // device copy
    unsigned* fallbacks;         // device counter of FP64 fallbacks
};
cudaError_t launch_colorize(const ColorLaunch& a, int nsm, cudaStream_t st);

// Owns the device tables and the staging buffers of host-pointer calls.
class Colorizer {
  public:
    ~Colorizer();
    int colorize(const mbx_color_params& p, const float* values, const float* aux, int width, int height, bool on_device, uint8_t* rgb,
                 cudaStream_t st, int nsm, std::string& err, unsigned* fallbacks_out = nullptr, float* gpu_ms = nullptr);

    // Device buffers for a render that is coloured in place (values, aux when
    // need_aux, rgb), grown as needed and owned by this object.
    int device_buffers(size_t samples, size_t pixels, bool need_aux, float** values, float** aux, uint8_t** rgb, std::string& err);

  private:
    int ensure(size_t samples, size_t pixels, bool need_aux, std::string& err);
    ColorTables* d_tables_ = nullptr;
    unsigned* d_fallbacks_ = nullptr;
    float* d_values_ = nullptr;
    float* d_aux_ = nullptr;
    uint8_t* d_rgb_ = nullptr;
    size_t cap_samples_ = 0, cap_pixels_ = 0;
    bool cap_aux_ = false;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
};

int validate_color_params(const mbx_color_params* p, std::string& why);
int write_bmp(const char* path, const uint8_t* rgb, int width, int height);

} // namespace mbx

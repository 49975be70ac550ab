// Allocation-free entry point: a variant of the shallow (direct-iteration)
// pass for callers that cannot allocate device memory — code running where
// cudaMalloc is unavailable or forbidden (inside a host application that owns
// all device memory up front, a real-time loop that must not allocate, or a
// plugin host that only lends it device buffers). The caller passes the frame
// geometry and its own device output buffers; the pass's scratch (the work
// queue counters and the per-sample completion flags) lives in one file-scope
// device array instead of cudaMalloc'd memory.
#include <mutex>

#include "../../include/mbx_gb300.h"
#include "kernels.h"

namespace mbx {
namespace {

constexpr int kNoAllocMaxSamples = 1 << 21; // 2,097,152 samples (1920x1080 fits)

// Scratch: Counters followed by one completion byte per sample. Every GPU that
// loads this library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[256 + kNoAllocMaxSamples];
static_assert(sizeof(Counters) <= 256, "the counters must fit the scratch array's 256-byte header");

std::mutex g_setup_mu;
void* g_scratch_addr[64] = {nullptr};

} // namespace
} // namespace mbx

extern "C" int mbx_render_shallow_noalloc(double c0_re, double c0_im, double dx, double dy, int width, int height, int max_iterations, double bailout, int coloring_method, float* iterations, int32_t* escape_iteration, float* normal, void* stream) {
    using namespace mbx;
    if (width < 2 || height < 2 || max_iterations < 1 || !iterations) return MBX_E_INVALID;
    if ((coloring_method & ~(MBX_EXTERIOR_DIST_EST | MBX_DE_OVERLAY)) != 0) return MBX_E_INVALID;
    // the distance overlay is written to the normal buffer: without one it has nowhere to go
    if ((coloring_method & MBX_DE_OVERLAY) && !normal) return MBX_E_INVALID;
    if ((long long)width * height > kNoAllocMaxSamples) return MBX_E_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MBX_E_NODEVICE;
    void* scratch = nullptr;
    {
        // First call on a device: resolve the device address of the scratch
        // array with that device current (a host-side use of the symbol is not
        // a device address).
        std::lock_guard<std::mutex> lock(g_setup_mu);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return MBX_E_CUDA;
            }
            g_scratch_addr[dev] = p;
        }
        scratch = g_scratch_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    Counters* ctr = reinterpret_cast<Counters*>(scratch);
    uint8_t* done = reinterpret_cast<uint8_t*>(scratch) + 256;
    const size_t n = (size_t)width * height;
    // The scratch keeps the previous call's contents: reset the counters.
    if (cudaMemsetAsync(ctr, 0, sizeof(Counters), st) != cudaSuccess) return MBX_E_CUDA;
    if (launch_fill(iterations, normal, escape_iteration, n, st) != cudaSuccess) return MBX_E_CUDA;
    const float escf = (float)(bailout > 0 ? bailout : 1e8);
    ShallowParams p{}; // value-initialised: fields not set below (normal map off) are zero
    p.g.W = width;
    p.g.H = height;
    p.g.sub = 1;
    p.g.mxit = max_iterations;
    p.g.ESC2 = (double)(escf * escf);
    p.g.dxf = dx;
    p.g.ede = (coloring_method & MBX_EXTERIOR_DIST_EST) ? 1 : 0;
    p.g.deovl = (coloring_method & MBX_DE_OVERLAY) ? 1 : 0;
    p.g.deriv = (p.g.ede || p.g.deovl) ? 1 : 0;
    p.c0r = c0_re;
    p.c0i = c0_im;
    p.dx = dx;
    p.dy = dy;
    p.simd_semantics = p.g.deovl ? 0 : 1;
    DeviceFrame f;
    f.orbit = OrbitView{nullptr, nullptr, nullptr, nullptr};
    f.bla = BlaView();
    f.px.keys = nullptr;
    f.px.n = (int)n;
    f.px.grid_w = width;
    f.px.grid_h = height;
    f.px.grid_step = 1;
    f.px.skip_i = f.px.skip_j = -1;
    f.out.iter = iterations;
    f.out.normal = normal;
    f.out.escN = escape_iteration;
    f.out.glitch = nullptr;
    f.out.done = done;
    f.out.gmp = nullptr;
    f.ctr = ctr;
    f.cancel = nullptr;
    int dev_sms = 0;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = (int)std::min<size_t>((n + 127) / 128, (size_t)(dev_sms > 0 ? dev_sms * 8 : 1216));
    if (launch_shallow(f, p, blocks, 128, st) != cudaSuccess) return MBX_E_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return MBX_E_CUDA;
    return MBX_OK;
}

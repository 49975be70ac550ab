// Host/device interface of the CUDA passes. Plain structs passed by value to
// the kernels; the launchers are implemented in the .cu files and called by the
// host engine (engine.cpp). Reference file:line citations refer to
// cbotx/Mandelbrot-Explorer, src/engine/mandel_perturbation.cpp ("mp.cpp").
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "floatexp.h"

namespace mbx {

constexpr float kEmpty = -10.0f; // mp.h:23 EMPTYPIXEL
constexpr int kSaTerms = 30;     // mp.h:288
constexpr int kMaxLevels = 32;

// Pixel/sample key: lexicographic order of the reference's std::array<int,4>
// {row, col, subrow, subcol} equals unsigned order of this packing.
__host__ __device__ inline uint64_t key_pack(int i, int j, int u, int v) {
    return ((uint64_t)(uint32_t)i << 40) | ((uint64_t)(uint32_t)j << 16) | ((uint64_t)(uint32_t)(u + 128) << 8) | (uint64_t)(uint32_t)(v + 128);
}
__host__ __device__ inline void key_unpack(uint64_t k, int* a) {
    a[0] = (int)(k >> 40);
    a[1] = (int)((k >> 16) & 0xffffff);
    a[2] = (int)((k >> 8) & 0xff) - 128;
    a[3] = (int)(k & 0xff) - 128;
}

struct FE2 {
    FE re, im;
};

// FP32-floatexp copy of one BLA entry for the mixed-precision pass: A and B as
// float2 mantissas with one exponent each, radius^2 as mantissa + exponent.
struct Bla32 {
    float4 ab; // A.re, A.im (scaled by 2^-ea), B.re, B.im (scaled by 2^-eb)
    int ea, eb;
    float r2m; // r2 = r2m * 2^r2e, r2m in [0.5,1); 0 when r2 <= 0
    int r2e;
};

// Reference orbit shadows in device memory (mp.h:295-371).
struct OrbitView {
    const double2* Z;   // Z[k] = (_zfr[k], _zfi[k]); Z[k] is reference value X_{k+1}
    const FE2* Zfe;     // floatexp shadow (floatexp path)
    const double2* D;   // derivative shadow (_dfr, _dfi)
    const double* zm3;  // |Z|^2 / 1e6 (glitch score normaliser)
};

// BLA table (mp.h:193-206) in level-major concatenated arrays.
struct BlaView {
    const double* r2;
    const double4* ab;  // (A.re, A.im, B.re, B.im)
    const double4* ce;  // (C.re, C.im, E.re, E.im) under the derivative
    int nlev;
    int off[kMaxLevels];
    int size[kMaxLevels];
    double rmax2;
    int minlevel;
    int use;
};

// Which pixels a pass iterates: either an explicit sorted key list or the full
// W x H base grid (optionally minus one skipped pixel), or a strided probe grid.
struct PixelSet {
    const uint64_t* keys; // null => grid mode
    int n;
    int grid_w, grid_step, grid_h;
    int skip_i, skip_j;   // grid mode: pixel excluded (reference pixel), -1 none
};

struct Outputs {
    float* iter;     // (W*sub) x (H*sub), reference layout (getIndex mp.cpp:4334-4340)
    float* normal;   // DE overlay, may be null
    int32_t* escN;   // escape iteration N (or -1 interior), may be null
    double* glitch;  // per list entry glitch score (double path), -1 none
    uint8_t* done;   // per list entry: 1 finished, 0 pending
    uint8_t* gmp;    // per list entry: needs the arbitrary-precision recompute
};

struct Counters {
    unsigned long long steps, bla_applies, bla_skipped, rebases, rescales;
    unsigned int next;  // work-queue head
    unsigned int interior;
    unsigned long long glitch_min_bits;  // min glitch score (as non-negative double bits)
    unsigned long long effective_iters;  // sum of N (maxiter for interior)
};

struct FrameGeom {
    int W, H, sub;
    int mxit;
    double ESC2;      // (double)(float R * float R) (mp.h:115-118)
    double dxf;       // mpf_get_ld(_dx)
    int ede, deovl, deriv;
};

// Double-precision delta loop parameters (mp.cpp:2290-2585).
struct Fp64Params {
    FrameGeom g;
    int ref[4];
    int xoff, yoff;          // dcx[xpix + xoff], dcy[ypix + yoff]
    const double* dcx;
    const double* dcy;
    double frac_re, frac_im; // periodic-nucleus sub-pixel offset
    int per;
    C2 A[kSaTerms], B[kSaTerms], sa_delta;
    int sa_order, sa_it;
    int mx_ref_it;
    int use_interior, int_rep, interior_confirm;
    double interior_eps2;
};

// Floatexp rescaled loop parameters (mp.cpp:3287-3618, 3620-3816).
struct FeParams {
    FrameGeom g;
    FE dxfe, dyfe;
    double ref_x, ref_y;
    int per;
    int mx_ref_it;
    int use_interior, int_rep, interior_confirm;
    double interior_eps2;
    int fused;
    int no_bla_kernel;       // mp.cpp:2185-2193 solveRescaledSimd8NoBla semantics
    int ref_period_gt0;
    int cutoff_sensitive;
};

// Shallow direct loop (mp.cpp:330-532).
struct ShallowParams {
    FrameGeom g;
    double c0r, c0i, dx, dy;
    int simd_semantics;      // 1: lane-refill kernel (float result), 0: floatPointCompute
};

struct DeviceFrame {
    OrbitView orbit;
    BlaView bla;
    PixelSet px;
    Outputs out;
    Counters* ctr;
    volatile int* cancel;    // host-mapped flag
};

// Launchers (kernels_exact.cu).
cudaError_t launch_fill(float* iter, float* normal, int32_t* escN, size_t n, cudaStream_t st);
cudaError_t launch_fp64_pass(const DeviceFrame& f, const Fp64Params& p, int blocks, int threads, cudaStream_t st);
cudaError_t launch_fe_pass(const DeviceFrame& f, const FeParams& p, int blocks, int threads, cudaStream_t st);
cudaError_t launch_shallow(const DeviceFrame& f, const ShallowParams& p, int blocks, int threads, cudaStream_t st);
cudaError_t launch_bla_build(const double2* Z, const double2* D, int reflen, double eps, double dcmax, bool ede,
                             double* r2, double4* ab, double4* ce, const int* off, const int* size, int nlev,
                             unsigned long long* rmax2_bits, cudaStream_t st);
cudaError_t launch_ss_flags(const float* iter, int W, int H, int sub, int ede, double thresh, uint8_t* flags, cudaStream_t st);

// Mixed-precision (FP32 floatexp) pass (kernels_mixed.cu).
struct MixedParams {
    FrameGeom g;
    FE dxfe, dyfe;
    double ref_x, ref_y;
    int per;
    int mx_ref_it;
    int use_interior;
    double interior_eps2;
    int interior_confirm;
    const float2* Zf;        // FP32 orbit (Z[k] as float2), valid where representable
    const uint8_t* Zsmall;   // 1 where |Z| is below FP32 normal range (use the floatexp shadow)
    int orbit_in_smem;       // stage the whole (periodic) orbit into shared memory
    int smem_entries;
    float wmax2, wmin2;      // |w|^2 rescale window
};
cudaError_t launch_mixed_pass(const DeviceFrame& f, const MixedParams& p, int blocks, int threads, size_t smem, cudaStream_t st);

} // namespace mbx

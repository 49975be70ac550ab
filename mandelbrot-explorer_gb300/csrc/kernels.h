// Host/device interface of the CUDA passes. Plain structs passed by value to
// the kernels; the launchers are implemented in the .cu files and called by the
// host engine (engine.cpp). Reference file:line citations refer to
// cbotx/Mandelbrot-Explorer, src/engine/mandel_perturbation.cpp ("mp.cpp").
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "dfloat.cuh"
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

// Floatexp copy of one BLA entry for the lane passes (T = float: the mixed
// pass, T = df32: the double-float rerun pass, T = double: the FP64 rerun
// pass): A and B as mantissa pairs with one exponent each, radius^2 as mantissa
// + exponent.
template <class T>
struct __align__(16) BlaEntry {
    T ar, ai, br, bi; // A.re, A.im (scaled by 2^-ea), B.re, B.im (scaled by 2^-eb)
    int ea, eb;
    T r2m;            // r2 = r2m * 2^r2e, r2m in [0.5,1); 0 when r2 <= 0
    int r2e;
};
using Bla32 = BlaEntry<float>;
using BlaDF = BlaEntry<df32>;
using Bla64 = BlaEntry<double>;
// Per BLA position of the FP32 lane (orbit index s with s - 1 a multiple of
// 2^minlevel): the largest radius^2 over the levels the lane tries there, as
// mantissa + exponent of the FP32 table; m = 0 when no level has a radius. A
// |dz|^2 at or above it fails every level's radius test.
struct BlaMaxR2 {
    float m;
    int e;
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
    const unsigned int* n_dev = nullptr; // list mode: entry count read on the device (bounded by n)
};

// Sample coordinates {row, col, subrow, subcol} of pass entry i.
__host__ __device__ inline void entry_coords(const PixelSet& px, int i, int* a) {
    if (px.keys) {
        key_unpack(px.keys[i], a);
        return;
    }
    // Grid mode: row-major over a strided grid, optionally skipping one pixel
    // (the reference pixel, erased from the pending set at mp.cpp:1726).
    int cols = (px.grid_w + px.grid_step - 1) / px.grid_step;
    int q = i;
    if (px.skip_i >= 0) {
        int sq = (px.skip_i / px.grid_step) * cols + px.skip_j / px.grid_step;
        if (q >= sq) ++q;
    }
    a[0] = (q / cols) * px.grid_step;
    a[1] = (q % cols) * px.grid_step;
    a[2] = 0;
    a[3] = 0;
}

struct Outputs {
    float* iter;     // (W*sub) x (H*sub), reference layout (getIndex mp.cpp:4334-4340)
    float* normal;   // DE overlay, may be null
    int32_t* escN;   // escape iteration N (or -1 interior), may be null
    double* glitch;  // per list entry glitch score (double path), -1 none
    uint8_t* done;   // per list entry: 1 finished, 0 pending
    uint8_t* gmp;    // per list entry: needs the arbitrary-precision recompute
    uint32_t* cost = nullptr; // lane passes: per sample (getIndex layout, sub 1) lane steps + 4 per BLA skip
    uint32_t* bla = nullptr;  // with cost: BLA skips of the sample's FP32 lane (learned ordering's probe features)
};

struct Counters {
    unsigned long long steps, bla_applies, bla_skipped, rebases;
    unsigned int next;  // work-queue head
    unsigned int interior;
    unsigned long long glitch_min_bits;  // min glitch score (as non-negative double bits)
    unsigned long long effective_iters;  // sum of N (maxiter for interior)
    unsigned int rerun_n;                // mixed pass: entries queued for the FP64 floatexp pass
    unsigned int finished;               // mixed pass: entries finished or queued
    unsigned int gmp_flags;              // floatexp pass: entries flagged for the arbitrary-precision recompute
    unsigned int interior_flagged;       // lane passes: interior decisions queued for the next tier
    unsigned int escape_flagged;         // lane passes: escapes queued for the next tier (|z|^2 too near the bailout for the estimate)
    unsigned int probe_hit;              // interior gate probe: set by the first interior decision (the probe then stops)
    unsigned long long exact_steps;      // lane passes: steps taken in floatexp (orbit or delta below the lane's range)
    unsigned long long fe_rebases;       // lane passes: rebases decided in floatexp
    // lane passes: blocks whose TMA orbit staging missed its wait limit (low 16
    // bits; such a block reads the orbit from global memory) and, times 2^16,
    // those whose copy was still in flight after a second bounded wait at exit
    unsigned int stage_timeouts;
};

struct FrameGeom {
    int W, H, sub;
    int mxit;
    double ESC2;      // (double)(float R * float R) (mp.h:115-118)
    double dxf;       // mpf_get_ld(_dx)
    int ede, deovl, deriv;
    int normal;       // normal map: arg(z) - arg(dz/dc) into the normal buffer (EDE takes precedence)
    int oc = 0;       // orbit colourings (orbit_color.h): kOcStripe | kOcTrap (exact form only)
    double ER = 0.0;  // escape radius as the reference keeps it: (double)(float R)
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
    int lanes_per_warp = 0;  // exact-form leftovers: lanes of each warp that take samples (0: all 32)
};

// Shallow direct loop (mp.cpp:330-532).
struct ShallowParams {
    FrameGeom g;
    double c0r, c0i, dx, dy;
    int simd_semantics;      // 1: lane-refill kernel (float result), 0: floatPointCompute
};

// Julia frames (Mandel::ComputeJulia, mp.cpp:992-1044): z0 = c0 + (dx j, dy i).
struct JuliaParams {
    FrameGeom g;
    double z0r, z0i, dx, dy; // lower-left sample and spacings (mpf_get_ld)
    double cr, ci;           // the fixed c
};

struct DeviceFrame {
    OrbitView orbit;
    BlaView bla;
    PixelSet px;
    Outputs out;
    Counters* ctr;
    volatile int* cancel;    // host-mapped flag
    uint64_t* rerun_keys = nullptr; // mixed pass: queue of sample keys for the FP64 floatexp pass
    uint8_t* rerun_flag = nullptr;  // mixed FP32 pass: per entry, set when left to the next tier (then compacted in entry order)
};

// Launchers (kernels_exact.cu).
cudaError_t launch_fill(float* iter, float* normal, int32_t* escN, size_t n, cudaStream_t st);
cudaError_t launch_fp64_pass(const DeviceFrame& f, const Fp64Params& p, int blocks, int threads, cudaStream_t st);
cudaError_t launch_fe_pass(const DeviceFrame& f, const FeParams& p, int blocks, int threads, cudaStream_t st);
cudaError_t launch_shallow(const DeviceFrame& f, const ShallowParams& p, int blocks, int threads, cudaStream_t st);
cudaError_t launch_julia(const DeviceFrame& f, const JuliaParams& p, int blocks, int threads, cudaStream_t st);
cudaError_t launch_bla_build(const double2* Z, const double2* D, int reflen, double eps, double dcmax, bool ede,
                             double* r2, double4* ab, double4* ce, const int* off, const int* size, int nlev,
                             unsigned long long* rmax2_bits, cudaStream_t st);
// adaptive-SS selection modes (k_ss_flags)
constexpr int kSsIterations = 0, kSsEde = 1, kSsStripe = 2, kSsTrap = 3;
cudaError_t launch_ss_flags(const float* iter, int W, int H, int sub, int mode, double thresh, double gain, double steps, uint8_t* flags, cudaStream_t st);

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
    // FP32 orbit for the common-step loop: {2 X.x, 2 X.y, q, 0} per entry, with
    // q = |X|^2 (fmaf(X.x, X.x, X.y * X.y)) when X is in the lane's range
    // (not both |components| below kTinyX and |X|^2 above kTinyX^2), else 0
    const float4* Zq = nullptr;
    float esc2f = 0.0f;      // (float)ESC2, and its screen bound (float)ESC2 * kEscLo, host-rounded
    float esc2lo = 0.0f;
    const uint8_t* Zsmall;   // 1 where |Z| is below FP32 normal range (use the floatexp shadow)
    int orbit_in_smem;       // stage the whole (periodic) orbit into shared memory
    int lane_budget = 256;   // iterations (orbit entries) a lane walks per call between its warp's refill points
    int smem_entries;
    float wmax2, wmin2;      // |w|^2 rescale window
    // Per supersampled column / row: the sample's offset from the reference in
    // pixels, arr[1] + arr[3] / sub - ref_x (and the same for rows), computed
    // on the host with the lane's own double expression, plus its float
    // rounding: the per-sample setup then needs no FP64 arithmetic. Null:
    // computed in the lane.
    const double* dpx_tab = nullptr;
    const double* dpy_tab = nullptr;
    const float* dpx_tabf = nullptr;
    const float* dpy_tabf = nullptr;
    const BlaMaxR2* blamax = nullptr; // FP32 lane: index (s - 1) >> minlevel
    int probe_stop = 0;               // interior gate probe: stop at the first interior decision
    unsigned wide_from = 0;  // rerun passes launched in two widths: the 32-lane
                             // variant runs when the queue holds >= wide_from
                             // entries, the narrow one below (0: no selection)
};
// The lane passes are launched by Engine::run_mixed_pass / run_df_pass
// (kernels_mixed.cu), which own their per-reference tables.

// One view of a batch: what a lane needs to iterate that view's samples. The
// batch passes read it from device memory per lane, so lanes of one warp may
// work on different views.
struct ViewDesc {
    DeviceFrame f;           // outputs, orbit shadows, BLA view, the view's pixel set
    MixedParams p;
    const Bla32* bla32;
    const float2* orb32;
    const BlaDF* bladf;
    const df2* orbdf;
    unsigned base;           // first batch-wide sample index of this view
    unsigned count;          // samples of this view in the pass
    int interior_gate;       // main pass: interior detection follows the probe's interior count
    float4* pgrid;           // learned ordering, per 8x8 cell of the probe: log2(1 + cost) / 24, interior,
                             // fraction of iterations BLA skipped, log2(1 + mean skip length) / 24
    int pgw, pgh;
    unsigned tile_base;      // first batch-wide 16x16 tile of this view
    int tw, th;              // its tiles across and down
};

// Batch-wide pass arguments. Queue entries are sample keys with the view index
// in bits 56..63 (rows below 2^16).
struct BatchArgs {
    const ViewDesc* views;
    int nviews;
    unsigned total;          // sample count (FP32 pass)
    const uint64_t* queue;   // rerun passes: queue of keys; null for the FP32 pass
    const unsigned* queue_n; // its length (on the device)
    const uint64_t* order;   // FP32 pass: the batch-wide sample indices in the order to take them (null: natural)
    uint8_t* rerun_flag;     // FP32 pass: per batch-wide sample, set when it is left to the next tier (null: queue it)
    unsigned capacity;       // queue capacity
    Counters* ctr;           // work counter and totals of this pass
    uint64_t* next_queue;    // where samples this pass cannot vouch for go (null: none)
    unsigned* view_interior; // probe pass: interior count per view (null otherwise)
    volatile int* cancel;
    unsigned wide_from = 0;  // as MixedParams::wide_from
    int deriv = 0;           // some view has a DE colouring: the lanes that carry the derivative
};
// Rerun queues at least this many entries per SM take 32 lanes per warp
// (fewer warp instructions for the same samples); shorter ones 8 (less
// divergence on each sample's latency chain). Measured on the 1e-300 frame's
// double-float queue: 19,932 entries 4.23 -> 2.89 ms wide, 4,965 entries 1.88
// (narrow) vs 2.76 ms (wide).
constexpr unsigned kWideLanesPerSm = 96;
constexpr int kBatchViewShift = 56;
constexpr int kBatchMaxViews = 256;
cudaError_t launch_batch_pass(int tier, const BatchArgs& a, int nsm, cudaStream_t st); // tier 0 FP32, 1 double-float, 2 FP64
cudaError_t launch_batch_gate(ViewDesc* views, int n, const unsigned* view_interior, cudaStream_t st);
// the rerun queue of the flagged samples, in the batch's natural order (view
// by view, rows of samples): sums holds flag_blocks(total) words
unsigned flag_blocks(unsigned total);
cudaError_t launch_flag_compact(const ViewDesc* views, int nv, unsigned total, const uint8_t* flag, unsigned* sums, uint64_t* out, cudaStream_t st);
// the same over one pass's entries (keys in entry order)
cudaError_t launch_flag_compact(const PixelSet& px, unsigned total, const uint8_t* flag, unsigned* sums, uint64_t* out, cudaStream_t st);

} // namespace mbx

/* mbx_gb300.h — C ABI of the GB300 deep-zoom Mandelbrot perturbation renderer.
 *
 * Drop-in boundary for the reference's compute-backend plugin API
 * (cbotx/Mandelbrot-Explorer src/engine/compute_backend.h). Plain C types only:
 * pointers, sizes and a status code. One context owns one CUDA device, one
 * stream and its device buffers; renders on one context are serialised.
 * Reference citations below are file:line in that project.
 */
#ifndef MBX_GB300_H
#define MBX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MBX_ABI_VERSION 4

/* Coloring flags: same bit values as the reference's ColoringMethod enum
 * (src/engine/mandel_perturbation.h:30-49). Other bits are rejected. */
#define MBX_SUPER_SAMPLING 1
#define MBX_EXTERIOR_DIST_EST 2
#define MBX_STRIPE_AVERAGE 8 /* value = stripe average over the last 256 iterations (src/engine/orbit_coloring.h:21-95); exact form; with MBX_SUPER_SAMPLING the set boundary is resampled (mp.cpp:1810-1826) */
#define MBX_NORMAL_MAP 16 /* value = smooth iteration; normal buffer = arg(z) - arg(dz/dc) (mp.cpp:375-378, 2489-2492, 3512-3515) */
#define MBX_ORBIT_TRAP 32 /* value = 0.17 (-log10 trap distance) + 0.025 mu (orbit_coloring.h:97-132); interior samples carry it too; exact form; with MBX_SUPER_SAMPLING pixels whose trap colour changes by more than 3 palette entries are resampled (mp.cpp:1827-1838) */
#define MBX_DE_OVERLAY 64

/* What a request renders (ComputeMode, src/engine/compute_backend.h:18). */
#define MBX_MODE_MANDELBROT 0
#define MBX_MODE_JULIA 1 /* z0 = the sample, fixed c (Mandel::ComputeJulia, mp.cpp:992-1044) */

/* Arithmetic of the per-sample delta loop. */
#define MBX_PRECISION_EXACT 0 /* FP64 / FP64-floatexp in the reference's exact operation order */
#define MBX_PRECISION_MIXED 1 /* FP32-mantissa floatexp bulk iteration with rebasing, for every perturbation frame (scale > 1e6), DE colourings included; shallow frames and the orbit colourings (SAC, traps) take the exact form */

/* Status codes (the reference returns bool + ComputeBackendInfo strings). */
#define MBX_OK 0
#define MBX_E_INVALID (-1)     /* request failed validation (compute_backend.cpp:263-272) */
#define MBX_E_CUDA (-2)        /* a CUDA call failed; see mbx_last_error */
#define MBX_E_CANCELLED (-3)   /* mbx_cancel was called; outputs are partial (EMPTYPIXEL = -10) */
#define MBX_E_NODEVICE (-4)    /* no usable CUDA device (there is no CPU fallback) */
#define MBX_E_BUSY (-5)        /* another compute is active on this context */
#define MBX_E_NOMEM (-6)       /* device or host allocation failed */
#define MBX_E_TOO_LARGE (-7)   /* frame exceeds a fixed capacity (mbx_render_shallow_noalloc) */

typedef struct mbx_context mbx_context;

/* One frame request. Mirrors ComputeRequest (src/engine/compute_backend.h:17-51)
 * for ComputeMode::Mandelbrot with the view given as decimal strings instead of
 * mpf_ptr, and the engine owned by the context instead of a Mandel*. */
typedef struct {
    const char* center_re;     /* view centre, decimal */
    const char* center_im;
    const char* scale;         /* reference scale: half-width = 2/scale (mp.cpp:1403-1416), decimal */
    int precision_bits;        /* mpf precision; 0 => digits(scale)*log2(10)+64 (src/tools/render.cpp:170-174) */
    int width, height;         /* base grid of this (strip) frame */
    int full_height, row_base; /* strip rendering; 0 => whole frame (mp.cpp:1399-1424) */
    int sub;                   /* odd sub-sample factor >= 1; buffers hold (width*sub) x (height*sub) */
    int max_iterations;
    int coloring_method;       /* MBX_* coloring flags */
    double bailout;            /* escape radius; 0 => 1e8 (mp.h:283) */
    int precision_mode;        /* MBX_PRECISION_* */
    int outputs_on_device;     /* 1: the three output pointers are CUDA device pointers */
    float* iterations;         /* required: smooth value / EDE distance / -2 interior / -10 empty */
    float* normal;             /* optional: DE-overlay distance (MBX_DE_OVERLAY) or normal-map angle (MBX_NORMAL_MAP), else NULL */
    int32_t* escape_iteration; /* optional: escape iteration N per sample, -1 interior, -10 empty */
    volatile float* progress;  /* optional: 0..1 progress, written between passes */
    int reuse_reference;       /* 1: reuse the previous frame's reference orbit and BLA table when the view,
                                  size, iteration and coloring parameters are unchanged (zoom-sequence reuse) */
    int compute_mode;          /* MBX_MODE_*; Julia takes sub 1, coloring 0 or MBX_EXTERIOR_DIST_EST and the
                                  fixed c below (compute_backend.cpp:268); precision_mode does not apply */
    const char* fixed_c_re;    /* Julia: fixed c, decimal (ComputeRequest::fixedCRe / fixedCIm) */
    const char* fixed_c_im;
    /* Optional periodic reference (no reference counterpart; the reference finds a
     * nucleus per frame, mp.cpp:1227-1386): with reference_period > 0 the frame's
     * reference is the given nucleus of that period, used whatever its size in
     * the frame, and its one-period orbit is kept on the context, so that every
     * frame of a zoom sequence toward it (the same nucleus, period and
     * precision_bits) reuses the orbit; only the per-frame parts (its position
     * in the frame, the BLA table for the frame's radius) are redone. Perturbation
     * frames (scale > 1e6) only. */
    const char* reference_re;
    const char* reference_im;
    int reference_period;
} mbx_request;

typedef struct {
    double total_ms, orbit_ms, bla_ms, kernel_ms, copy_ms;
    long long steps;                /* executed delta-loop iterations */
    long long bla_applies;          /* BLA skips taken */
    long long bla_skipped;          /* iterations skipped by BLA */
    long long effective_iterations; /* sum over samples of N (max_iterations for interior) */
    long long gmp_pixels;           /* samples recomputed in arbitrary precision (mp.cpp:2173-2183) */
    long long samples;              /* samples computed */
    int passes, references, method, used_floatexp, period, reference_length, kernel_launches, interior;
    double pass_gpu_ms;             /* CUDA-event time of the delta-pass kernels on the context's stream */
    int reused_reference;           /* 1 when the cached reference was reused */
    long long rebases;              /* rebases taken (mixed form) */
    long long fp64_reruns;          /* mixed form: samples rerun in double-float (FP32 error estimate too large) */
    double rerun_gpu_ms;            /* device time of the reruns (included in pass_gpu_ms); batch: the main
                                       pass's double-float tier with its queue's compaction (and training, mode 1) */
    long long fp64_reruns_fp64;     /* of those, samples rerun again in FP64: the exact form (double-float estimate too large) */
    double rerun_fp64_gpu_ms;       /* device time of the exact-form reruns (included in rerun_gpu_ms); batch:
                                       host wall time of the views' concurrent exact-form leftovers (after pass_gpu_ms) */
    long long exact_steps;          /* mixed form: steps taken in floatexp (orbit or delta below the lane type's range) */
    long long fe_rebases;           /* mixed form: rebases decided in floatexp (inside the margin, end of reference) */
    long long exact_reruns;         /* mixed form: samples finished by the exact form (no tier could vouch for them; equals fp64_reruns_fp64) */
    long long h2d_bytes, d2h_bytes; /* bytes copied host->device / device->host by the call (counted at each copy) */
    double fp32_pass_gpu_ms;        /* mixed form: CUDA-event time of the FP32 lane passes alone (probe and main;
                                       batch: the main pass) */
    long long fp32_pass_steps;      /* mixed form: delta steps executed by those passes */
    long long fp32_pass_bla_applies;/* mixed form: BLA skips taken by those passes */
    long long fp32_unvouched_interior; /* mixed form: of fp64_reruns, interior decisions the FP32 estimate could not vouch for */
    long long fp32_unvouched_escape;   /* mixed form: of fp64_reruns, escapes with |z|^2 within the estimated error of the bailout */
} mbx_stats;

/* createComputeBackend("cuda") (src/engine/compute_backend.cpp:277-290). Returns
 * NULL with a message in err when no CUDA device is usable; never falls back. */
mbx_context* mbx_create(int device, char* err, int err_len);
void mbx_destroy(mbx_context* ctx);

/* IComputeBackend::compute (src/engine/compute_backend.h:106-117, CPU version
 * compute_backend.cpp:44-117). Synchronous; returns MBX_OK or a negative code. */
int mbx_compute(mbx_context* ctx, const mbx_request* req, mbx_stats* stats);

/* IComputeBackend::cancel / resetCancellation (compute_backend.cpp:119-128). Thread-safe. */
void mbx_cancel(mbx_context* ctx);
void mbx_reset_cancellation(mbx_context* ctx);

/* ComputeBackendInfo (compute_backend.h:53-58): name/detail strings. */
const char* mbx_info_name(const mbx_context* ctx);
const char* mbx_info_detail(const mbx_context* ctx);
const char* mbx_last_error(const mbx_context* ctx);
int mbx_abi_version(void);

/* Launch shape and numerics knobs of the mixed-precision pass. */
typedef struct {
    int threads;            /* block size: 128 or 256 */
    int blocks_per_sm;      /* resident blocks per SM the kernel is compiled for: 2, 3 or 4 */
    int smem_orbit_limit;   /* stage the FP32 orbit into shared memory when it fits in this many bytes (0: never) */
    double rescale_window;  /* |w|^2 is kept in [1/window, window]; 1e4 to 1e16 */
    double pass_ms;         /* autotune: GPU time of the calibration pass with this shape */
    int lane_budget;        /* iterations a lane walks per call between its warp's refill points: 16 to 4096 */
} mbx_tuning;

/* Sets the mixed-pass tuning of a context (values out of range are ignored). */
int mbx_set_tuning(mbx_context* ctx, int threads, int blocks_per_sm, int smem_orbit_limit, double rescale_window);

/* Sets the iterations a mixed-pass lane walks per call between its warp's
 * refill points (16 to 4096; the span of the orbit a warp covers between
 * refills; results do not depend on it). */
int mbx_set_lane_budget(mbx_context* ctx, int iterations);

/* Autotuner: renders `calibration` (a floatexp frame) in mixed precision once
 * per candidate (block size x resident blocks x orbit staging x rescale
 * window x lane span between refills), keeps the fastest shape on the context
 * and returns it in *best. */
int mbx_autotune(mbx_context* ctx, const mbx_request* calibration, mbx_tuning* best);

/* Diagnostic: measured issue rate of dependent-free FMA chains on the context's
 * device, in TFLOP/s (an FMA counts as 2); fp64 = 1 for double, 0 for float.
 * The roofline denominators of the delta loops (FP64 / FP32 pipes). */
int mbx_measure_fma_peak(mbx_context* ctx, int fp64, double* tflops);

/* Host-only nucleus search (no context, no GPU): findNucleus for the disk
 * (centre, radius) — ball-arithmetic period up to max_period, then Newton
 * refinement (src/engine/mandel_perturbation.cpp:116-223, 1072-1107) — with
 * the minibrot size estimate of nucleusSizeMag (mp.cpp:1195-1219) returned as
 * log10. Writes the nucleus as decimal strings (buf_len bytes each). Returns
 * the period, 0 when the disk holds no nucleus, or a negative MBX_E_* code. */
int mbx_find_nucleus(const char* center_re, const char* center_im, const char* radius, int max_period, int precision_bits,
                     char* nucleus_re, char* nucleus_im, int buf_len, double* size_log10);

/* Batched rendering of n (1..256) frames (no reference counterpart: the
 * reference renders one frame per compute() call). Each frame is prepared as
 * by mbx_compute (reference orbit, BLA tables, outputs); the probe and main
 * passes of every perturbation frame in the mixed form (any colouring) then
 * run in shared persistent launches — one batch-wide work counter over all
 * frames' samples, then the double-float tier — captured once as a CUDA graph
 * and replayed while the batch keeps its shape; what no lane tier vouches for
 * is finished per frame in the exact form, and the adaptive-supersampling
 * passes of supersampled frames run per frame after the graph, on the frames'
 * own streams from concurrent host threads. Frames of 2^20 pixels or more
 * (mbx_set_batch_direct; unless the learned ordering is on) and other frames (shallow, exact form,
 * orbit colourings, and supersampled frames while the learned ordering is on)
 * are rendered on their own, each on its engine's stream from the host thread
 * that prepared it, so a large frame's passes overlap the other frames' host
 * work. Results are identical to mbx_compute of each frame. view_stats
 * (n entries) and batch_stats may be NULL; the shared passes' counters go to
 * batch_stats. Frames need fewer than 65536 sample rows. */
int mbx_compute_batch(mbx_context* ctx, const mbx_request* reqs, int n, mbx_stats* view_stats, mbx_stats* batch_stats);

/* Learned ordering of the batched main pass (no reference counterpart). A
 * BF16 MLP (24 -> 64 -> 64 -> 1) predicts each 16x16 tile's mean FP32-lane
 * cost from the probe pass (its four probe cells' costs, BLA-skip fractions
 * and mean skip lengths, interior flags, the neighbouring tiles' costs, view
 * features). With mode 1 the main FP32 pass takes the views in decreasing
 * predicted cost and each view's samples in decreasing predicted tile cost;
 * after the passes the model trains on the batch's tiles and their measured
 * costs (tcgen05 kernels, Adam, 32 steps), so the next batch uses it. Mode 2
 * orders with the model as it stands (no training). A fresh context's model
 * predicts a tile's mean probe cost. Outputs are identical in every mode.
 * 0 (default): natural order. */
int mbx_set_batch_scheduling(mbx_context* ctx, int mode);

/* Frames of mbx_compute_batch with at least `pixels` pixels (default 2^20)
 * render on their own as soon as their host work is done instead of joining
 * the shared graph; pixels <= 0 keeps every eligible frame in the graph.
 * Results are identical either way. */
int mbx_set_batch_direct(mbx_context* ctx, long long pixels);

/* Diagnostics of the ordering model: parameters (5825 floats: W1 [64][24], b1
 * [64], W2 [64][64], b2 [64], w3 [64], b3) set and/or read, and the gradients
 * of one training step over n >= 128 samples (mean squared error / 2;
 * features n x 24, targets n) without an update. */
int mbx_schedule_params(mbx_context* ctx, const float* set, float* get);
int mbx_schedule_gradient(mbx_context* ctx, const float* features, const float* targets, int n, float* grad);

/* Allocation-free render of a shallow frame (no reference counterpart: the
 * reference has no device and allocates its buffers itself). For callers that
 * cannot allocate device memory: the caller passes the frame geometry — the
 * lower-left corner c0 and the pixel spacings dx, dy as doubles, i.e. the
 * double values the reference derives at mp.cpp:1445-1448 — and device
 * pointers to its own output buffers (iterations required; escape_iteration
 * and normal optional; width*height entries). The direct-iteration pass
 * (floatPointCompute semantics, mp.cpp:330-532) runs on `stream` (a
 * cudaStream_t, NULL for the default stream) and the call returns after it
 * completes. Its scratch (work counters, completion flags) is one fixed device
 * array of 256 B + 2,097,152 B that every GPU loading this library holds until
 * the process exits; frames above 2,097,152 samples are rejected with
 * MBX_E_TOO_LARGE. The first call on each device resolves the array's device
 * address with that device current, so make that first call before any stream
 * capture. Every call waits for `stream` to finish before it returns. All
 * calls share the one array: calls that overlap on the GPU race.
 * Coloring bits: MBX_EXTERIOR_DIST_EST and MBX_DE_OVERLAY only (no
 * supersampling); MBX_DE_OVERLAY needs the normal buffer, which receives the
 * overlay distance (MBX_E_INVALID without it). Calls no allocating CUDA or
 * library routine. */
int mbx_render_shallow_noalloc(double c0_re, double c0_im, double dx, double dy, int width, int height, int max_iterations,
                               double bailout, int coloring_method, float* iterations, int32_t* escape_iteration,
                               float* normal, void* stream);

/* ---- Image epilogue: the reference's render tool (src/tools/render.cpp) ----
 * Value -> palette coordinate (getColor, render.cpp:71-92): */
#define MBX_MAP_LOG_POWER 0 /* powf(logf(v+2), logf(v+2)^2 * density/3600) (color_func, render.cpp:31-33) */
#define MBX_MAP_DISTANCE 1  /* tanhf(v * density/3600 * 5): exterior distance values (MANDEL_EDE) */
#define MBX_MAP_STRIPE 2    /* v * (density/20): stripe-average values (MANDEL_SAC) */
#define MBX_MAP_TRAP 3      /* v: orbit-trap values are palette coordinates (MANDEL_TRAP) */
/* Per-sample shade (render.cpp:255-292): */
#define MBX_SHADE_NONE 0
#define MBX_SHADE_RELIEF 1     /* screen-space slope of the values, Lambert (reliefShadeAt, render.cpp:47-69) */
#define MBX_SHADE_NORMAL_MAP 2 /* Lambert from a normal-angle buffer (MANDEL_NORMAL, render.cpp:276-287) */
#define MBX_SHADE_DE_OVERLAY 3 /* black-and-white filament layer from a distance buffer (render.cpp:263-274) */

typedef struct {
    int supersample;          /* ss: each output pixel averages ss x ss values in linear light */
    int mapping;              /* MBX_MAP_* */
    int shading;              /* MBX_SHADE_* */
    float density;            /* colour density (color_density, render.cpp:21; MANDEL_DENS) */
    double light_az, light_el; /* light direction in radians (render.cpp:45; MANDEL_LIGHT_AZ/EL) */
    double relief_strength;   /* slope strength (MANDEL_RELIEF_STR) */
    double de_k;              /* overlay falloff (MANDEL_DE_K) */
} mbx_color_params;

/* The render tool's defaults: ss 1, log-power mapping, no shading, density 60,
 * light (2.3, 0.55), relief strength 1, overlay falloff 1.5. */
void mbx_color_defaults(mbx_color_params* p);

/* Colours (width*ss) x (height*ss) values (the iterations output of a render)
 * into rgb[height][width][3] (render.cpp:248-300). aux is the normal-angle or
 * distance buffer of the same layout for those shadings, else NULL. With
 * on_device = 1 values, aux and rgb are CUDA device pointers and nothing is
 * copied; otherwise they are host pointers. Runs on the context's stream and
 * returns when the image is complete. */
int mbx_colorize(mbx_context* ctx, const mbx_color_params* p, const float* values, const float* aux, int width, int height,
                 int on_device, uint8_t* rgb);

/* Render and colour in one call, the render tool's pipeline without its host
 * colouring loop: the frame (req: sub 1, width and height multiples of
 * p->supersample; its output pointers are ignored) is computed into
 * context-owned device buffers, coloured there, and only the
 * (width/ss) x (height/ss) RGB image is copied to rgb (host). The distance
 * overlay takes its buffer from MBX_DE_OVERLAY in req->coloring_method. */
int mbx_render_image(mbx_context* ctx, const mbx_request* req, const mbx_color_params* p, uint8_t* rgb, mbx_stats* stats);

/* Device time of the last colour pass (CUDA events on the context's stream)
 * and how many palette coordinates took the FP64 path (see mbx_colorize). */
int mbx_last_color_stats(const mbx_context* ctx, double* gpu_ms, long long* fp64_fallbacks);

/* writeBMP (render.cpp:101-137): 24-bit BMP, bottom-up BGR rows padded to 4
 * bytes. Host only. */
int mbx_write_bmp(const char* path, const uint8_t* rgb, int width, int height);

/* The epilogue's host-built tables, for inspection: the palette as three
 * 2048-entry channels (render.cpp:23-29), and the 352 gamma thresholds
 * (least linear value giving each encoded value 1..352). Host only. */
void mbx_color_tables(float* palette, float* gamma_thresholds);

#ifdef __cplusplus
}
#endif
#endif

// extern "C" boundary (include/mbx_gb300.h). Validation mirrors the
// reference's CpuComputeBackend::valid (src/engine/compute_backend.cpp:263-272)
// plus the engine's own constraints (odd sub, mp.cpp:230).
#include <cstring>
#include <algorithm>
#include <mutex>
#include <new>
#include <string>

#include "batch.h"
#include "color.h"
#include "engine.h"

struct mbx_context {
    mbx::Engine* engine = nullptr;
    mbx::BatchRunner* batch = nullptr;
    mbx::Colorizer* color = nullptr;
    double color_gpu_ms = 0.0;
    long long color_fallbacks = 0;
    std::string name = "cuda";
    std::string detail;
    std::string last_error;
    std::mutex mu;
};

namespace {
// GMP keeps its default mpf precision in process-global state, which every
// render sets; renders are therefore serialised process-wide.
std::mutex g_gmp_mutex;

int validate(const mbx_request* r, std::string& why) {
    if (!r) {
        why = "null request";
        return MBX_E_INVALID;
    }
    const int full_h = r->full_height > 0 ? r->full_height : r->height;
    if (!r->center_re || !r->center_im || !r->scale || !r->iterations) why = "missing centre, scale or iterations buffer";
    else if (r->width < 2 || r->height < 1 || full_h < 2) why = "width must be >= 2 and the (full) height >= 2";
    else if (r->row_base < 0 || r->row_base > full_h - r->height) why = "row_base outside the full frame";
    else if (r->sub < 1 || (r->sub % 2) == 0 || r->sub > 255) why = "sub must be odd and in [1, 255]";
    else if (r->max_iterations < 1) why = "max_iterations must be >= 1";
    else if (r->compute_mode != MBX_MODE_MANDELBROT && r->compute_mode != MBX_MODE_JULIA) why = "unknown compute_mode";
    else if (r->compute_mode == MBX_MODE_JULIA && (r->sub != 1 || !r->fixed_c_re || !r->fixed_c_im || (r->coloring_method & ~MBX_EXTERIOR_DIST_EST) != 0))
        why = "Julia takes sub 1, the fixed c and coloring 0 or MBX_EXTERIOR_DIST_EST";
    else if ((r->coloring_method & ~(MBX_SUPER_SAMPLING | MBX_EXTERIOR_DIST_EST | MBX_STRIPE_AVERAGE | MBX_NORMAL_MAP | MBX_ORBIT_TRAP | MBX_DE_OVERLAY)) != 0)
        why = "unsupported coloring_method bits";
    else if (r->precision_mode != MBX_PRECISION_EXACT && r->precision_mode != MBX_PRECISION_MIXED) why = "unknown precision_mode";
    else if (!(r->bailout >= 0.0) || r->bailout > 1e18) why = "bailout must be in [0, 1e18]";
    else if ((long long)r->width * r->sub * r->height * r->sub > (1ll << 31) - 1) why = "frame too large";
    else if (r->height >= (1 << 24) || r->width >= (1 << 24)) why = "dimensions too large";
    else if (r->reference_period < 0 || (r->reference_period > 0 && (!r->reference_re || !r->reference_im || r->compute_mode != MBX_MODE_MANDELBROT)))
        why = "a periodic reference needs its nucleus (reference_re, reference_im), a period >= 1 and a Mandelbrot frame";
    else return MBX_OK;
    return MBX_E_INVALID;
}
mbx::BatchRunner* batch_of(mbx_context* c) {
    if (!c->batch) c->batch = new (std::nothrow) mbx::BatchRunner(c->engine->device());
    return c->batch;
}
mbx::Colorizer* color_of(mbx_context* c) {
    if (!c->color) c->color = new (std::nothrow) mbx::Colorizer();
    return c->color;
}
} // namespace

extern "C" {

int mbx_abi_version(void) { return MBX_ABI_VERSION; }

mbx_context* mbx_create(int device, char* err, int err_len) {
    auto fail = [&](const std::string& m) -> mbx_context* {
        if (err && err_len > 0) {
            strncpy(err, m.c_str(), (size_t)err_len - 1);
            err[err_len - 1] = 0;
        }
        return nullptr;
    };
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count <= device || device < 0) return fail(std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "index out of range"));
    mbx_context* c = new (std::nothrow) mbx_context();
    if (!c) return fail("out of memory");
    c->engine = new (std::nothrow) mbx::Engine(device);
    std::string why;
    if (!c->engine || c->engine->init(why) != 0) {
        delete c->engine;
        delete c;
        return fail("CUDA initialisation failed: " + why);
    }
    c->detail = std::string("GB300 perturbation renderer on ") + c->engine->device_name();
    return c;
}

void mbx_destroy(mbx_context* c) {
    if (!c) return;
    delete c->batch;
    delete c->color;
    delete c->engine;
    delete c;
}

int mbx_compute_batch(mbx_context* c, const mbx_request* reqs, int n, mbx_stats* view_stats, mbx_stats* batch_stats) {
    if (!c || !reqs || n < 1 || n > mbx::kBatchMaxViews) return MBX_E_INVALID;
    std::string why;
    for (int i = 0; i < n; ++i) {
        int v = validate(reqs + i, why);
        if (v == MBX_OK && reqs[i].compute_mode != MBX_MODE_MANDELBROT) {
            why = "batches hold Mandelbrot frames only";
            v = MBX_E_INVALID;
        }
        if (v != MBX_OK) {
            std::lock_guard<std::mutex> l(c->mu);
            c->last_error = "request " + std::to_string(i) + ": " + why;
            return v;
        }
    }
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    std::lock_guard<std::mutex> g(g_gmp_mutex);
    if (!batch_of(c)) return MBX_E_NOMEM;
    std::string err;
    int rc = c->batch->run(reqs, n, view_stats, batch_stats, c->engine->device_cancel_flag(), err);
    c->last_error = rc == MBX_OK ? std::string() : (err.empty() ? std::string("batch failed") : err);
    return rc;
}

int mbx_compute(mbx_context* c, const mbx_request* r, mbx_stats* stats) {
    if (!c) return MBX_E_INVALID;
    std::string why;
    int v = validate(r, why);
    if (v != MBX_OK) {
        std::lock_guard<std::mutex> l(c->mu);
        c->last_error = why;
        return v;
    }
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    std::lock_guard<std::mutex> g(g_gmp_mutex);
    int rc = c->engine->compute(*r, stats);
    c->last_error = rc == MBX_OK ? std::string() : (c->engine->error().empty() ? std::string("compute failed") : c->engine->error());
    if (rc == MBX_E_CANCELLED) c->last_error = "cancelled";
    return rc;
}

int mbx_set_batch_scheduling(mbx_context* c, int mode) {
    if (!c) return MBX_E_INVALID;
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    mbx::BatchRunner* b = batch_of(c);
    if (!b) return MBX_E_NOMEM;
    std::string err;
    int rc = b->set_schedule(mode, err);
    c->last_error = err;
    return rc;
}

int mbx_set_batch_direct(mbx_context* c, long long pixels) {
    if (!c) return MBX_E_INVALID;
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    mbx::BatchRunner* b = batch_of(c);
    if (!b) return MBX_E_NOMEM;
    b->set_direct(pixels);
    return MBX_OK;
}

int mbx_schedule_params(mbx_context* c, const float* set, float* get) {
    if (!c || (!set && !get)) return MBX_E_INVALID;
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    mbx::BatchRunner* b = batch_of(c);
    if (!b) return MBX_E_NOMEM;
    std::string err;
    int rc = b->schedule_params(set, get, err);
    c->last_error = err;
    return rc;
}

int mbx_schedule_gradient(mbx_context* c, const float* features, const float* targets, int n, float* grad) {
    if (!c) return MBX_E_INVALID;
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    mbx::BatchRunner* b = batch_of(c);
    if (!b) return MBX_E_NOMEM;
    std::string err;
    int rc = b->schedule_gradient(features, targets, n, grad, err);
    c->last_error = err;
    return rc;
}

void mbx_cancel(mbx_context* c) {
    if (c && c->engine) c->engine->cancel();
    if (c && c->batch) c->batch->cancel();
}
void mbx_reset_cancellation(mbx_context* c) {
    if (c && c->engine) c->engine->reset_cancel();
    if (c && c->batch) c->batch->reset_cancel();
}
const char* mbx_info_name(const mbx_context* c) { return c ? c->name.c_str() : ""; }
const char* mbx_info_detail(const mbx_context* c) { return c ? c->detail.c_str() : ""; }
const char* mbx_last_error(const mbx_context* c) { return c ? c->last_error.c_str() : ""; }

int mbx_set_tuning(mbx_context* c, int threads, int blocks_per_sm, int smem_orbit_limit, double rescale_window) {
    if (!c) return MBX_E_INVALID;
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    c->engine->set_tuning(threads, blocks_per_sm, smem_orbit_limit, (float)rescale_window);
    return MBX_OK;
}

int mbx_set_lane_budget(mbx_context* c, int iterations) {
    if (!c) return MBX_E_INVALID;
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    c->engine->set_lane_budget(iterations);
    return MBX_OK;
}

int mbx_autotune(mbx_context* c, const mbx_request* calib, mbx_tuning* best) {
    if (!c || !calib) return MBX_E_INVALID;
    std::string why;
    if (validate(calib, why) != MBX_OK) {
        c->last_error = why;
        return MBX_E_INVALID;
    }
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    std::lock_guard<std::mutex> g(g_gmp_mutex);
    mbx_request r = *calib;
    r.precision_mode = MBX_PRECISION_MIXED;
    r.reuse_reference = 1;
    mbx_stats st;
    int rc = c->engine->compute(r, &st); // builds (and caches) the calibration reference
    if (rc != MBX_OK) {
        c->last_error = c->engine->error();
        return rc;
    }
    if (!st.used_floatexp) {
        c->last_error = "calibration frame does not use the floatexp path";
        return MBX_E_INVALID;
    }
    const int threads_opts[] = {128, 256};
    const int blocks_opts[] = {2, 3, 4};
    const int smem_opts[] = {200 * 1024, 0};
    const double window_opts[] = {1e8, 1e12, 1e16};
    const int budget_opts[] = {64, 256, 1024};
    double best_ms = 1e300;
    mbx_tuning b = {};
    for (int t : threads_opts)
        for (int bl : blocks_opts)
            for (int sm : smem_opts)
                for (double w : window_opts)
                    for (int lb : budget_opts) {
                    c->engine->set_tuning(t, bl, sm, (float)w);
                    c->engine->set_lane_budget(lb);
                    double ms = 1e300;
                    for (int rep = 0; rep < 2; ++rep) {
                        rc = c->engine->compute(r, &st);
                        if (rc != MBX_OK) {
                            c->last_error = c->engine->error();
                            return rc;
                        }
                        ms = std::min(ms, st.pass_gpu_ms);
                    }
                    if (ms < best_ms) {
                        best_ms = ms;
                        b.threads = t;
                        b.blocks_per_sm = bl;
                        b.smem_orbit_limit = sm;
                        b.rescale_window = w;
                        b.pass_ms = ms;
                        b.lane_budget = lb;
                    }
                    }
    c->engine->set_tuning(b.threads, b.blocks_per_sm, b.smem_orbit_limit, (float)b.rescale_window);
    c->engine->set_lane_budget(b.lane_budget);
    if (best) *best = b;
    return MBX_OK;
}

int mbx_measure_fma_peak(mbx_context* c, int fp64, double* tflops) {
    if (!c || !tflops) return MBX_E_INVALID;
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    return c->engine->measure_fma_peak(fp64, tflops);
}

int mbx_find_nucleus(const char* center_re, const char* center_im, const char* radius, int max_period, int precision_bits, char* nucleus_re, char* nucleus_im, int buf_len, double* size_log10) {
    if (!center_re || !center_im || !radius || !nucleus_re || !nucleus_im || buf_len < 8 || max_period < 1 || precision_bits < 64) return MBX_E_INVALID;
    std::lock_guard<std::mutex> g(g_gmp_mutex);
    std::string a, b;
    int p = mbx::find_nucleus_disk(center_re, center_im, radius, max_period, precision_bits, a, b, size_log10);
    if (p < 0) return MBX_E_INVALID;
    if (p > 0 && ((int)a.size() >= buf_len || (int)b.size() >= buf_len)) return MBX_E_NOMEM;
    if (p > 0) {
        memcpy(nucleus_re, a.c_str(), a.size() + 1);
        memcpy(nucleus_im, b.c_str(), b.size() + 1);
    }
    return p;
}

void mbx_color_defaults(mbx_color_params* p) { // render.cpp:21, 44-46
    if (!p) return;
    p->supersample = 1;
    p->mapping = MBX_MAP_LOG_POWER;
    p->shading = MBX_SHADE_NONE;
    p->density = 60.0f;
    p->light_az = 2.3;
    p->light_el = 0.55;
    p->relief_strength = 1.0;
    p->de_k = 1.5;
}

int mbx_colorize(mbx_context* c, const mbx_color_params* p, const float* values, const float* aux, int width, int height, int on_device, uint8_t* rgb) {
    if (!c) return MBX_E_INVALID;
    std::string why;
    if (mbx::validate_color_params(p, why) != MBX_OK) {
        std::lock_guard<std::mutex> l(c->mu);
        c->last_error = why;
        return MBX_E_INVALID;
    }
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    mbx::Colorizer* col = color_of(c);
    if (!col) return MBX_E_NOMEM;
    unsigned fb = 0;
    float ms = 0.0f;
    std::string err;
    const int rc = col->colorize(*p, values, aux, width, height, on_device != 0, rgb, c->engine->stream(), c->engine->sm_count(), err, &fb, &ms);
    c->last_error = err;
    if (rc == MBX_OK) {
        c->color_gpu_ms = ms;
        c->color_fallbacks = fb;
    }
    return rc;
}

int mbx_render_image(mbx_context* c, const mbx_request* r, const mbx_color_params* p, uint8_t* rgb, mbx_stats* stats) {
    if (!c || !r || !rgb) return MBX_E_INVALID;
    std::string why;
    mbx_request q = *r;
    float dummy = 0.0f;
    if (!q.iterations) q.iterations = &dummy; // replaced below; validate() wants a buffer
    int v = validate(&q, why);
    if (v == MBX_OK) v = mbx::validate_color_params(p, why);
    if (v == MBX_OK) {
        if (r->sub != 1) why = "render_image takes sub 1 (supersampling is the colour pass's ss)";
        else if (r->width % p->supersample || r->height % p->supersample) why = "width and height must be multiples of supersample";
        else if (p->shading == MBX_SHADE_NORMAL_MAP && !(r->coloring_method & MBX_NORMAL_MAP)) why = "normal-map shading needs MBX_NORMAL_MAP in coloring_method";
        else if (p->shading == MBX_SHADE_DE_OVERLAY && !(r->coloring_method & MBX_DE_OVERLAY)) why = "distance-overlay shading needs MBX_DE_OVERLAY in coloring_method";
        v = why.empty() ? MBX_OK : MBX_E_INVALID;
    }
    if (v != MBX_OK) {
        std::lock_guard<std::mutex> l(c->mu);
        c->last_error = why;
        return v;
    }
    std::unique_lock<std::mutex> busy(c->mu, std::try_to_lock);
    if (!busy.owns_lock()) return MBX_E_BUSY;
    mbx::Colorizer* col = color_of(c);
    if (!col) return MBX_E_NOMEM;
    const int ow = r->width / p->supersample, oh = r->height / p->supersample;
    const size_t samples = (size_t)r->width * r->height, pixels = (size_t)ow * oh;
    const bool need_aux = p->shading == MBX_SHADE_DE_OVERLAY || p->shading == MBX_SHADE_NORMAL_MAP;
    float *dv = nullptr, *da = nullptr;
    uint8_t* drgb = nullptr;
    std::string err;
    int rc = col->device_buffers(samples, pixels, need_aux, &dv, &da, &drgb, err);
    if (rc != MBX_OK) {
        c->last_error = err;
        return rc;
    }
    q.outputs_on_device = 1;
    q.iterations = dv;
    const bool wants_aux = (r->coloring_method & (MBX_DE_OVERLAY | MBX_NORMAL_MAP)) != 0;
    q.normal = wants_aux ? da : nullptr;
    if (wants_aux && !da) {
        // the second buffer is computed even when the chosen shading ignores it
        rc = col->device_buffers(samples, pixels, true, &dv, &da, &drgb, err);
        if (rc != MBX_OK) {
            c->last_error = err;
            return rc;
        }
        q.iterations = dv;
        q.normal = da;
    }
    q.escape_iteration = nullptr;
    {
        std::lock_guard<std::mutex> g(g_gmp_mutex);
        rc = c->engine->compute(q, stats);
    }
    if (rc != MBX_OK) {
        c->last_error = c->engine->error().empty() ? std::string("compute failed") : c->engine->error();
        if (rc == MBX_E_CANCELLED) c->last_error = "cancelled";
        return rc;
    }
    unsigned fb = 0;
    float ms = 0.0f;
    rc = col->colorize(*p, dv, da, ow, oh, true, drgb, c->engine->stream(), c->engine->sm_count(), err, &fb, &ms);
    if (rc == MBX_OK) {
        const cudaError_t e = cudaMemcpyAsync(rgb, drgb, pixels * 3, cudaMemcpyDeviceToHost, c->engine->stream());
        const cudaError_t e2 = e == cudaSuccess ? cudaStreamSynchronize(c->engine->stream()) : e;
        if (e2 != cudaSuccess) {
            err = std::string("image copy: ") + cudaGetErrorString(e2);
            rc = MBX_E_CUDA;
        }
    }
    c->last_error = err;
    if (rc == MBX_OK) {
        c->color_gpu_ms = ms;
        c->color_fallbacks = fb;
    }
    return rc;
}

int mbx_last_color_stats(const mbx_context* c, double* gpu_ms, long long* fp64_fallbacks) {
    if (!c) return MBX_E_INVALID;
    if (gpu_ms) *gpu_ms = c->color_gpu_ms;
    if (fp64_fallbacks) *fp64_fallbacks = c->color_fallbacks;
    return MBX_OK;
}

int mbx_write_bmp(const char* path, const uint8_t* rgb, int width, int height) { return mbx::write_bmp(path, rgb, width, height); }

void mbx_color_tables(float* palette, float* gamma_thresholds) {
    if (palette) mbx::build_palette(palette);
    if (gamma_thresholds) {
        mbx::ColorTables* t = new (std::nothrow) mbx::ColorTables();
        if (!t) return;
        mbx::build_color_tables(*t);
        memcpy(gamma_thresholds, t->gamma, sizeof(t->gamma));
        delete t;
    }
}

} // extern "C"

// Host engine of the GB300 renderer (see engine.cpp).
#pragma once
#include <atomic>
#include <functional>
#include <string>
#include <vector>

#include "../../include/mbx_gb300.h"
#include "gmp_abi.h"
#include "kernels.h"

namespace mbx {

// The additive-feedback generator behind glibc's rand() (random_r TYPE_3,
// degree 31, separation 3), seeded like srand(1). The reference picks a
// fallback reference pixel with rand() (mp.cpp:4039-4052); a private replica
// replays that sequence for every frame without touching the host's libc state.
struct LibcRand {
    int32_t st[31];
    int f = 3, r = 0;
    void seed(uint32_t s) {
        if (s == 0) s = 1;
        st[0] = (int32_t)s;
        for (int i = 1; i < 31; ++i) {
            int32_t hi = st[i - 1] / 127773, lo = st[i - 1] % 127773;
            int32_t word = 16807 * lo - 2836 * hi;
            if (word < 0) word += 2147483647;
            st[i] = word;
        }
        f = 3;
        r = 0;
        for (int i = 0; i < 310; ++i) (void)next();
    }
    int next() {
        uint32_t val = (uint32_t)st[f] + (uint32_t)st[r];
        st[f] = (int32_t)val;
        int out = (int)(val >> 1);
        if (++f >= 31) {
            f = 0;
            ++r;
        } else if (++r >= 31) {
            r = 0;
        }
        return out;
    }
};

// Fixed-point big real for the floatexp-path reference orbit (bigfixed.h).
struct FixedReal {
    int L = 0;
    int sign = 0;
    std::vector<uint64_t> limb;
    void set_len(int l);
    void from_mpf(mpf_srcptr x, int l);
    void to_mpf(mpf_ptr out) const;
    FE to_fe() const;
    double to_double() const;
    static void addsub(FixedReal& r, const FixedReal& a, int sa, const FixedReal& b, int sb);
    static void mul(FixedReal& r, const FixedReal& a, const FixedReal& b, uint64_t* tmp);
};

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
};

int ball_period(mpf_srcptr cr, mpf_srcptr ci, mpf_srcptr r, int maxp, mp_bitcnt_t prec, const std::atomic<bool>* cancel);
bool newton_nucleus(mpf_ptr cr, mpf_ptr ci, int period, mp_bitcnt_t prec, int maxit);
int find_nucleus_disk(const char* cre, const char* cim, const char* radius, int maxp, int prec, std::string& nre, std::string& nim, double* size_log10);

// A frame handed to a batch: the engine prepares everything up to the passes
// (reference, BLA, outputs) and describes its probe and main pass; the batch
// runs those passes for all its frames in shared launches.
struct BatchSlot {
    bool deferred = false;
    bool want_cost = false; // learned ordering: per-sample costs and the probe grid
    ViewDesc probe, main;
};

class Engine {
  public:
    explicit Engine(int device);
    ~Engine();
    int init(std::string& err);
    int compute(const mbx_request& r, mbx_stats* st);
    void cancel();
    void reset_cancel();
    const std::string& error() const { return err_; }
    const char* device_name() const { return devname_; }
    // Batch support: compute up to the passes (slot->deferred), or the whole
    // frame when it is not eligible (mixed form, floatexp, no DE, sub 1);
    // finish copies host outputs and completes the stats of a deferred frame.
    int compute_deferred(const mbx_request& r, BatchSlot* slot, mbx_stats* st);
    int batch_supersample(bool interior_seen);
    int batch_finish(const mbx_request& r, mbx_stats* st);
    // the exact form over a deferred frame's samples the batched tiers could
    // not vouch for (keys as key_pack; emptied on success); interior_seen: the
    // batch's interior gate found interior samples in this frame's probe
    int batch_exact_rerun(std::vector<uint64_t>& keys, bool interior_seen);
    cudaStream_t stream() const { return st_; }
    volatile int* device_cancel_flag() const { return dcancel_; }
    int sm_count() const { return nsm_; }
    int device() const { return device_; }

  private:
    int compute_frame(const mbx_request& r);
    int render(mpf_ptr c_re, mpf_ptr c_im, mpf_ptr scale, int full_h, int row_base, volatile float* progress);
    int render_shallow(volatile float* progress);
    int render_julia(mpf_ptr z_re, mpf_ptr z_im, mpf_ptr scale, const char* fcr, const char* fci, int full_h, int row_base);
    int shallow_samples(const std::vector<uint64_t>& samples);
    int glitch_loop(std::vector<uint64_t>& pending, int& ref_it, bool have, int* nr, volatile float* progress);
    int supersample(int ref_it);
    int run_pass(std::vector<uint64_t>* keys, const PixelSet& grid, int mx_ref_it, bool* have_new_ref, int* new_ref);
    int run_pass_mixed(std::vector<uint64_t>* keys, const PixelSet& grid, int mx_ref_it);
    FeParams fe_params(int mx_ref_it) const;
    cudaError_t run_mixed_pass(const DeviceFrame& f);
    cudaError_t run_df_pass(const DeviceFrame& f);
    MixedParams mixed_params() const;
    int prepare_mixed();
    int recompute_gmp(const std::vector<int>& list, const std::function<void(int, int*)>& key_of);
    int write_sample(const int* a, float v, int32_t n);
    int flush_ref_value();

    void set_precision(int p);
    bool orbit_step(int i, int pr_it, bool past);
    void sa_update(int i);
    void reset_series();
    float gmp_point(mpf_srcptr c_re, mpf_srcptr c_im, int mxit, int* nout) const;
    float gmp_sample(const int* a, int mxit, int* nout) const;
    bool ref_tail_escapes(int last, int extra);
    int build_reference(const int* pick, bool view_center);
    int find_nucleus(int maxp);
    int build_periodic_reference(int period);
    void periodic_reference_geometry();
    int zoom_reference(int* ref_it);
    FE nucleus_size() const;
    int reference_for_frame();
    int upload_reference(int ref_it);
    int build_bla(int reflen);
    int build_dc_tables();

    DeviceFrame frame_view();
    FrameGeom geom() const;
    int cuda_ok(const char* what);
    int fail_cuda(const char* what, cudaError_t e);
    // cudaMemcpyAsync on the context's stream; host<->device bytes are counted
    // into the frame's statistics (h2d_bytes / d2h_bytes)
    cudaError_t copy_async(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind);
    void release_device();
    template <typename T>
    bool ensure(DevBuf<T>& b, size_t n);

    // device / context
    int device_;
    int nsm_ = 0;
    char devname_[160] = {0};
    cudaStream_t st_ = nullptr;
    Counters* dctr_ = nullptr;
    Counters* hctr_ = nullptr;
    volatile int* hcancel_ = nullptr;
    int* dcancel_ = nullptr;
    std::atomic<bool> cancel_{false};
    std::atomic<bool> active_{false};
    std::string err_;
    LibcRand rng_;
    mbx_stats stats_{};

    // frame configuration
    int W_ = 0, H_ = 0, SUB_ = 1, MXIT_ = 0, cm_ = 0, mode_ = 0, method_ = 0;
    bool deriv_ = false;
    float escf_ = 1e8f;
    double ESC2_ = 0.0;

    // arbitrary-precision state
    bool mpf_ready_ = false;
    mpf_t c0_re_, c0_im_, dx_, dy_, scale_, ref_re_, ref_im_, t1_, t2_;
    mpf_t zre_[2], zim_[2];
    bool use_fixed_ = false;
    int fixL_ = 0;
    std::vector<uint64_t> ftmp_, ftmp2_;
    FixedReal fc_re_, fc_im_, fz_re_[2], fz_im_[2], ft1_, ft2_, fab_, fre_, fim_;
    FE dfe_r_{1.0, 0}, dfe_i_{0.0, 0};

    // reference orbit shadows (host staging)
    std::vector<double2> hZ_, hD_;
    std::vector<double> hzm3_;
    std::vector<FE2> hZfe_;
    int orbit_len_ = 0;

    // series approximation
    C2 sa_A_[kSaTerms], sa_B_[kSaTerms], sa_delta_{0, 0};
    bool sa_valid_ = false;
    int sa_it_ = 0, sa_order_ = 0;

    // reference bookkeeping
    int ref_[4] = {0, 0, 0, 0};
    double ref_x_ = 0, ref_y_ = 0, ref_frac_re_ = 0, ref_frac_im_ = 0;
    bool ref_virtual_ = false, ref_subpixel_ = false, ref_escaped_ = false;
    int ref_period_ = 0, ref_escape_it_ = 0;
    float ref_value_ = 0.0f, ref_value_store_ = 0.0f;
    int32_t ref_n_ = -1, ref_n_store_ = -1;
    bool ref_value_pending_ = false;

    // engine switches (reference defaults, mp.cpp:1530-1588)
    bool use_floatexp_ = false, fe_cutoff_sensitive_ = false, use_bla_ = true, use_interior_ = true;
    int bla_minlevel_ = 3, interior_confirm_ = 4;
    double interior_eps2_ = 9e-18;
    FE dxfe_{0, 0}, dyfe_{0, 0};
    BlaView bla_{};

    // double-path spacing tables
    std::vector<double> hdcx_, hdcy_;
    int dc_xoff_ = 0, dc_yoff_ = 0;

    // device buffers
    DevBuf<double2> dZ_, dD_;
    DevBuf<FE2> dZfe_;
    DevBuf<double> dzm3_, dr2_, ddcx_, ddcy_, dglitch_;
    DevBuf<double4> dab_, dce_;
    DevBuf<float> diter_own_, dnormal_own_;
    DevBuf<int32_t> descN_own_;
    DevBuf<uint64_t> dkeys_;
    DevBuf<uint8_t> ddone_, dgmp_, dflags_, dZsmall_;
    DevBuf<float2> dZf_;
    DevBuf<float4> dZq_;  // FP32 lane's common-step orbit table (MixedParams::Zq)
    DevBuf<Bla32> dbla32_;
    DevBuf<BlaMaxR2> dblamax_;
    bool blamax_ok_ = false; // dblamax_ holds the current reference's table
    DevBuf<BlaDF> dbladf_;
    DevBuf<df2> dZdf_;
    DevBuf<uint32_t> dcost_;  // batch learned ordering: per-sample FP32-lane cost
    DevBuf<uint32_t> dblac_;  // its BLA skips
    DevBuf<float4> dpgrid_;   // and the probe pass's record per 8x8 cell
    DevBuf<double> ddpxy_;    // mixed passes: sample offsets per column then per row
    DevBuf<float> ddpxyf_;    // (their float roundings)
    std::vector<double> hdpxy_;
    std::vector<float> hdpxyf_;
    int dpxy_w_ = 0;
    bool probe_gate_only_ = false; // mixed form: the gate's probe pass runs its FP32 tier only
    DevBuf<uint64_t> drerun_keys_;            // mixed pass: queue for the double-float pass
    DevBuf<uint8_t> drerun_flag_;             // mixed main pass: per entry, left to the double-float pass
    DevBuf<unsigned> dflag_sums_;             // block sums of their compaction
    DevBuf<uint64_t> drerun2_keys_;           // double-float pass: samples it cannot vouch for (the exact form finishes them)
    DevBuf<uint8_t> drerun_done_, drerun_gmp_; // flags of that pass, by queue position
    bool exact_rerun_ = false; // mixed form: the FP64 floatexp rerun of flagged samples is running
    BatchSlot* batch_slot_ = nullptr;
    void fill_batch_slot();
    int batch_ref_it_ = 0; // reference length of the deferred frame's passes
    // The FP32 pass carries no derivative: DE colourings take the exact form.
    // the mixed form renders every perturbation frame except orbit colourings (SAC, traps: exact form)
    bool mixed_active() const { return mode_ == MBX_PRECISION_MIXED && !(cm_ & (8 | 32)); }

    // mixed-pass launch shape (set by the autotuner / defaults: orbit read
    // through L1, the choice of the autotuner on both 1080p deep frames).
    // The rescale window |w|^2 in [1/wmax2, wmax2] stays at or below 1e16:
    // with a wider one, |w| down to 1e-15 times an orbit value near the
    // lanes' 1e-30 floor leaves FP32's normal range (and the double-float
    // low parts leave it 2^24 sooner), a rounding loss the error estimate
    // does not model (class errors on a 1e-875 minibrot frame at 1e30).
    int mixed_threads_ = 256;
    int mixed_blocks_per_sm_ = 3;
    int smem_orbit_limit_ = 0;
    int lane_budget_ = 256;
    float mixed_wmax2_ = 1e16f;

  public:
    void set_tuning(int threads, int blocks_per_sm, int smem_limit, float wmax2) {
        if (threads == 128 || threads == 256) mixed_threads_ = threads;
        if (blocks_per_sm >= 1 && blocks_per_sm <= 4) mixed_blocks_per_sm_ = blocks_per_sm;
        if (smem_limit >= 0 && smem_limit <= 220 * 1024) smem_orbit_limit_ = smem_limit;
        if (wmax2 >= 1e4f && wmax2 <= 1e16f) mixed_wmax2_ = wmax2;
    }
    void set_lane_budget(int n) {
        if (n >= 16 && n <= 4096) lane_budget_ = n;
    }
    int lane_budget() const { return lane_budget_; }
    void get_tuning(int* threads, int* blocks_per_sm, int* smem_limit, float* wmax2) const {
        *threads = mixed_threads_;
        *blocks_per_sm = mixed_blocks_per_sm_;
        *smem_limit = smem_orbit_limit_;
        *wmax2 = mixed_wmax2_;
    }

  private:
    float* out_iter_ = nullptr;
    float* out_norm_ = nullptr;
    int32_t* out_n_ = nullptr;

    // reference cache (mbx_request.reuse_reference)
    struct RefCache {
        bool valid = false;
        std::string key;
        bool use_floatexp, use_bla, ref_subpixel, ref_virtual, fe_cutoff_sensitive, ref_value_pending;
        int ref_period, ref[4], orbit_len, sa_order, sa_it, ref_it, dc_xoff, dc_yoff, reference_length;
        double ref_x, ref_y, ref_frac_re, ref_frac_im;
        C2 A[kSaTerms], B[kSaTerms], delta;
        BlaView bla;
        FE dxfe, dyfe;
        float ref_value;
        int32_t ref_n;
    } cache_;
    std::string frame_key_;
    bool reuse_ = false;
    // the request's periodic reference (zoom sequences): nucleus, period, and
    // whether the orbit shadows hold its orbit (zoom_key_)
    std::string zoom_re_, zoom_im_, zoom_key_;
    int zoom_period_ = 0;
    bool zoom_valid_ = false;
    int refs_built_in_frame_ = 0;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr, evm_ = nullptr;
    void save_cache(int ref_it);
    bool restore_cache(int* ref_it);

  public:
    int measure_fma_peak(int fp64, double* tflops);

  private:
    // pass readback
    std::vector<uint8_t> hdone_, hgmp_;
    std::vector<double> hglitch_;
    std::vector<uint64_t> grid_pending_;
};

template <typename T>
bool Engine::ensure(DevBuf<T>& b, size_t n) {
    if (n <= b.cap) return true;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    size_t want = n > 0 ? n : 1;
    if (cudaMalloc(&b.p, want * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    b.cap = want;
    return true;
}

} // namespace mbx

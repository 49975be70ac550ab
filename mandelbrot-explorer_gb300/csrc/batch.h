// Batched rendering of several views: one engine per view prepares its frame
// (reference orbit, BLA tables, outputs), then one launch sequence runs the
// probe and main passes of all views together — a batch-wide work counter
// shared by the persistent lane passes, followed by the two rerun tiers — as a
// CUDA graph that is replayed while the batch's shape stays the same.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "engine.h"
#include "order_model.h"

namespace mbx {

// default: frames of at least this many pixels render on their own, not in the shared graph
constexpr long long kBatchDirectSamples = 1ll << 20;

class BatchRunner {
  public:
    explicit BatchRunner(int device) : device_(device) {}
    ~BatchRunner();
    // Renders reqs[0..n) (each validated by the caller). view_stats may be
    // null; batch_stats (may be null) receives the shared passes' counters.
    int run(const mbx_request* reqs, int n, mbx_stats* view_stats, mbx_stats* batch_stats, volatile int* cancel_flag, std::string& err);
    void cancel();
    void reset_cancel();
    // 1: order each batch's main pass by the learned cost model and train it on
    // the batch's costs; 2: order with the model as it stands; 0: natural order
    int set_schedule(int mode, std::string& err);
    void set_direct(long long pixels) { direct_pixels_ = pixels; }
    int schedule_params(const float* set, float* get, std::string& err);
    int schedule_gradient(const float* features, const float* targets, int n, float* grad, std::string& err);

  private:
    int ensure_engines(int n, std::string& err);
    int ensure_buffers(int nviews, unsigned capacity, unsigned tiles, std::string& err);
    int build_graph(int nviews, unsigned probe_total, unsigned main_total, unsigned tile_total, volatile int* cancel_flag, int deriv, std::string& err);

    int device_;
    std::vector<std::unique_ptr<Engine>> eng_;
    cudaStream_t st_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    cudaEvent_t evm_[2] = {nullptr, nullptr}; // in the graph: main FP32 pass start and end
    ViewDesc* d_probe_ = nullptr;
    ViewDesc* d_main_ = nullptr;
    ViewDesc* h_desc_ = nullptr;   // pinned staging: probe descriptors then main descriptors
    Counters* d_ctr_ = nullptr;    // 4 blocks: probe FP32 / double-float, main likewise
    Counters* h_ctr_ = nullptr;
    unsigned* d_view_interior_ = nullptr;
    uint64_t* d_qa_ = nullptr;     // FP32 -> double-float queue
    uint64_t* d_qb_ = nullptr;     // double-float -> the views' exact form
    int cap_views_ = 0;
    unsigned cap_samples_ = 0;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    int g_views_ = -1;
    unsigned g_probe_ = 0, g_main_ = 0, g_tiles_ = 0;
    unsigned cap_tiles_ = 0;
    volatile int* g_cancel_ = nullptr;
    int g_schedule_ = -1;
    int g_deriv_ = -1;     // the captured graph's lanes carry the derivative (DE colourings)
    // learned ordering
    int schedule_ = 0;
    long long direct_pixels_ = kBatchDirectSamples; // <= 0: every frame joins the shared graph
    SchedState sched_{};
    bool sched_ready_ = false;
    uint64_t* d_qo_ = nullptr;       // the main FP32 pass's order (sample indices), then the double-float queue
    uint8_t* d_flag_ = nullptr;      // main FP32 pass: per sample, left to the double-float tier
    unsigned* d_fsum_ = nullptr;     // block sums of the flags' compaction
    unsigned* d_main_total_ = nullptr;
    unsigned h_main_total_ = 0;
    int ensure_sched(std::string& err);
};

} // namespace mbx

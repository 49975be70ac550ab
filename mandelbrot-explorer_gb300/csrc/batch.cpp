// Batched rendering (batch.h). The engines prepare their frames on their own
// streams; the runner waits for them, uploads the view descriptors and replays
// (or captures, when the shape changed) one CUDA graph holding every pass of
// every view:
//   memset counters -> probe: FP32, double-float, FP64 lane passes -> interior
//   gate -> main: FP32, double-float, FP64 lane passes -> counters to the host.
#include "batch.h"

#include <chrono>
#include <thread>

#include <algorithm>
#include <cstring>

namespace mbx {

namespace {
int cuda_fail(std::string& err, const char* what, cudaError_t e) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return MBX_E_CUDA;
}
} // namespace

BatchRunner::~BatchRunner() {
    if (st_) cudaStreamSynchronize(st_);
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    for (void* p : {(void*)d_probe_, (void*)d_main_, (void*)d_ctr_, (void*)d_view_interior_, (void*)d_qa_, (void*)d_qb_, (void*)d_qo_, (void*)d_main_total_, (void*)d_flag_, (void*)d_fsum_,
                    (void*)sched_.params, (void*)sched_.adam_m, (void*)sched_.adam_v, (void*)sched_.ready, (void*)sched_.steps, (void*)sched_.loss,
                    (void*)sched_.hist, (void*)sched_.bucket, (void*)sched_.tile_bucket, (void*)sched_.X, (void*)sched_.T, (void*)sched_.grad,
                    (void*)sched_.err})
        if (p) cudaFree(p);
    if (h_desc_) cudaFreeHost(h_desc_);
    if (h_ctr_) cudaFreeHost(h_ctr_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    for (cudaEvent_t ev : evm_)
        if (ev) cudaEventDestroy(ev);
    if (st_) cudaStreamDestroy(st_);
}

void BatchRunner::cancel() {
    for (auto& e : eng_) e->cancel();
}
void BatchRunner::reset_cancel() {
    for (auto& e : eng_) e->reset_cancel();
}

int BatchRunner::ensure_engines(int n, std::string& err) {
    if (!st_) {
        if (cudaSetDevice(device_) != cudaSuccess || cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&ev0_) != cudaSuccess || cudaEventCreate(&ev1_) != cudaSuccess || cudaEventCreate(&evm_[0]) != cudaSuccess ||
            cudaEventCreate(&evm_[1]) != cudaSuccess) {
            err = "batch stream creation failed";
            return MBX_E_CUDA;
        }
    }
    while ((int)eng_.size() < n) {
        std::unique_ptr<Engine> e(new Engine(device_));
        std::string why;
        if (e->init(why) != 0) {
            err = "batch engine initialisation failed: " + why;
            return MBX_E_CUDA;
        }
        eng_.push_back(std::move(e));
    }
    return MBX_OK;
}

int BatchRunner::ensure_buffers(int nviews, unsigned capacity, unsigned tiles, std::string& err) {
    if (tiles > cap_tiles_) {
        if (sched_.tile_bucket) cudaFree(sched_.tile_bucket);
        sched_.tile_bucket = nullptr;
        if (cudaMalloc(&sched_.tile_bucket, tiles) != cudaSuccess) {
            err = "batch tile buffer allocation failed";
            cap_tiles_ = 0;
            return MBX_E_NOMEM;
        }
        cap_tiles_ = tiles;
        g_views_ = -1;
    }
    if (nviews > cap_views_) {
        if (d_probe_) cudaFree(d_probe_);
        if (d_main_) cudaFree(d_main_);
        if (d_view_interior_) cudaFree(d_view_interior_);
        if (h_desc_) cudaFreeHost(h_desc_);
        d_probe_ = d_main_ = nullptr;
        d_view_interior_ = nullptr;
        h_desc_ = nullptr;
        if (cudaMalloc(&d_probe_, sizeof(ViewDesc) * nviews) != cudaSuccess || cudaMalloc(&d_main_, sizeof(ViewDesc) * nviews) != cudaSuccess ||
            cudaMalloc(&d_view_interior_, sizeof(unsigned) * nviews) != cudaSuccess ||
            cudaHostAlloc((void**)&h_desc_, sizeof(ViewDesc) * 2 * nviews, cudaHostAllocDefault) != cudaSuccess) {
            err = "batch descriptor allocation failed";
            cap_views_ = 0;
            return MBX_E_NOMEM;
        }
        cap_views_ = nviews;
        g_views_ = -1; // the graph holds the old pointers
    }
    if (!d_ctr_) {
        if (cudaMalloc(&d_ctr_, 4 * sizeof(Counters)) != cudaSuccess || cudaHostAlloc((void**)&h_ctr_, 4 * sizeof(Counters), cudaHostAllocDefault) != cudaSuccess) {
            err = "batch counter allocation failed";
            return MBX_E_NOMEM;
        }
    }
    if (capacity > cap_samples_) {
        for (uint64_t** q : {&d_qa_, &d_qb_, &d_qo_}) {
            if (*q) cudaFree(*q);
            *q = nullptr;
        }
        if (sched_.bucket) cudaFree(sched_.bucket);
        if (d_flag_) cudaFree(d_flag_);
        if (d_fsum_) cudaFree(d_fsum_);
        sched_.bucket = nullptr;
        d_flag_ = nullptr;
        d_fsum_ = nullptr;
        if (cudaMalloc(&d_qa_, sizeof(uint64_t) * capacity) != cudaSuccess || cudaMalloc(&d_qb_, sizeof(uint64_t) * capacity) != cudaSuccess ||
            cudaMalloc(&d_qo_, sizeof(uint64_t) * capacity) != cudaSuccess || cudaMalloc(&sched_.bucket, sizeof(uint16_t) * capacity) != cudaSuccess ||
            cudaMalloc(&d_flag_, capacity) != cudaSuccess || cudaMalloc(&d_fsum_, sizeof(unsigned) * (flag_blocks(capacity) + 1)) != cudaSuccess) {
            err = "batch queue allocation failed";
            cap_samples_ = 0;
            return MBX_E_NOMEM;
        }
        cap_samples_ = capacity;
        g_views_ = -1;
    }
    if (!d_main_total_ && cudaMalloc(&d_main_total_, sizeof(unsigned)) != cudaSuccess) {
        err = "batch counter allocation failed";
        return MBX_E_NOMEM;
    }
    return MBX_OK;
}

int BatchRunner::ensure_sched(std::string& err) {
    if (sched_ready_) return MBX_OK;
    if (!st_) {
        int rc = ensure_engines(1, err);
        if (rc != MBX_OK) return rc;
    }
    const int N = SchedLayout::N;
    if (cudaMalloc(&sched_.params, sizeof(float) * N) != cudaSuccess || cudaMalloc(&sched_.adam_m, sizeof(float) * N) != cudaSuccess ||
        cudaMalloc(&sched_.adam_v, sizeof(float) * N) != cudaSuccess || cudaMalloc(&sched_.ready, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&sched_.steps, sizeof(int)) != cudaSuccess || cudaMalloc(&sched_.loss, sizeof(float)) != cudaSuccess ||
        cudaMalloc(&sched_.grad, sizeof(float) * N) != cudaSuccess || cudaMalloc(&sched_.err, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&sched_.hist, sizeof(unsigned) * sched_scratch_words()) != cudaSuccess ||
        cudaMalloc(&sched_.X, sizeof(__nv_bfloat16) * kSchedTiles * kSchedFeatures) != cudaSuccess ||
        cudaMalloc(&sched_.T, sizeof(float) * kSchedTiles) != cudaSuccess) {
        err = "scheduler allocation failed";
        return MBX_E_NOMEM;
    }
    cudaError_t e = sched_init(sched_, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return cuda_fail(err, "scheduler initialisation", e);
    sched_ready_ = true;
    return MBX_OK;
}

int BatchRunner::set_schedule(int mode, std::string& err) {
    if (mode < 0 || mode > 2) {
        err = "scheduling mode must be 0, 1 or 2";
        return MBX_E_INVALID;
    }
    if (mode != 0) {
        int rc = ensure_sched(err);
        if (rc != MBX_OK) return rc;
    }
    schedule_ = mode;
    return MBX_OK;
}

int BatchRunner::schedule_params(const float* set, float* get, std::string& err) {
    int rc = ensure_sched(err);
    if (rc != MBX_OK) return rc;
    const size_t bytes = sizeof(float) * SchedLayout::N;
    if (set) {
        cudaMemcpyAsync(sched_.params, set, bytes, cudaMemcpyHostToDevice, st_);
        cudaMemsetAsync(sched_.adam_m, 0, bytes, st_);
        cudaMemsetAsync(sched_.adam_v, 0, bytes, st_);
    }
    if (get) cudaMemcpyAsync(get, sched_.params, bytes, cudaMemcpyDeviceToHost, st_);
    cudaError_t e = cudaStreamSynchronize(st_);
    return e == cudaSuccess ? MBX_OK : cuda_fail(err, "scheduler parameters", e);
}

namespace {
uint16_t bf16_rne(float f) { // round to nearest even, as __float2bfloat16_rn for finite values
    uint32_t u;
    memcpy(&u, &f, 4);
    const uint32_t r = u + 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(r >> 16);
}
} // namespace

int BatchRunner::schedule_gradient(const float* features, const float* targets, int n, float* grad, std::string& err) {
    if (!features || !targets || !grad || n < 128) {
        err = "gradient check needs at least 128 samples";
        return MBX_E_INVALID;
    }
    int rc = ensure_sched(err);
    if (rc != MBX_OK) return rc;
    std::vector<uint16_t> xh((size_t)n * kSchedFeatures, 0);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 24; ++k) xh[(size_t)i * kSchedFeatures + k] = bf16_rne(features[(size_t)i * 24 + k]);
    void *dx = nullptr, *dt = nullptr, *dg = nullptr;
    if (cudaMalloc(&dx, xh.size() * 2) != cudaSuccess || cudaMalloc(&dt, sizeof(float) * n) != cudaSuccess ||
        cudaMalloc(&dg, sizeof(float) * SchedLayout::N) != cudaSuccess) {
        if (dx) cudaFree(dx);
        if (dt) cudaFree(dt);
        err = "gradient check allocation failed";
        return MBX_E_NOMEM;
    }
    cudaMemcpyAsync(dx, xh.data(), xh.size() * 2, cudaMemcpyHostToDevice, st_);
    cudaMemcpyAsync(dt, targets, sizeof(float) * n, cudaMemcpyHostToDevice, st_);
    cudaError_t e = sched_gradient(sched_, (const __nv_bfloat16*)dx, (const float*)dt, n, (float*)dg, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(grad, dg, sizeof(float) * SchedLayout::N, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    cudaFree(dx);
    cudaFree(dt);
    cudaFree(dg);
    return e == cudaSuccess ? MBX_OK : cuda_fail(err, "gradient check", e);
}

int BatchRunner::build_graph(int nviews, unsigned probe_total, unsigned main_total, unsigned tile_total, volatile int* cancel_flag, int deriv, std::string& err) {
    if (exec_ && g_views_ == nviews && g_probe_ == probe_total && g_main_ == main_total && g_tiles_ == tile_total && g_cancel_ == cancel_flag &&
        g_schedule_ == schedule_ && g_deriv_ == deriv)
        return MBX_OK;
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
    int nsm = eng_[0]->sm_count();
    cudaError_t e = cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(err, "graph capture", e);
    cudaMemsetAsync(d_ctr_, 0, 4 * sizeof(Counters), st_);
    cudaMemsetAsync(d_view_interior_, 0, sizeof(unsigned) * nviews, st_);
    // probe_only: the probe's samples are rendered again by the main pass, so
    // the probe needs only its FP32 tier (its gate counts unvouched interior
    // decisions as interior)
    auto tiers = [&](const ViewDesc* views, unsigned total, int c0, unsigned* vint, const uint64_t* order, bool probe_only) {
        BatchArgs a{};
        a.views = views;
        a.nviews = nviews;
        a.capacity = cap_samples_;
        a.view_interior = vint;
        a.cancel = cancel_flag;
        a.deriv = deriv;
        // FP32 over all samples (in the learned order when given); the main
        // pass flags its leftovers per sample
        a.total = total;
        a.order = order;
        a.ctr = d_ctr_ + c0;
        a.next_queue = d_qa_;
        if (!probe_only) {
            a.rerun_flag = d_flag_;
            cudaMemsetAsync(d_flag_, 0, total, st_);
            // event-record nodes of the graph (plain records in a capture add none)
            cudaEventRecordWithFlags(evm_[0], st_, cudaEventRecordExternal);
        }
        launch_batch_pass(0, a, nsm, st_);
        if (probe_only) return;
        cudaEventRecordWithFlags(evm_[1], st_, cudaEventRecordExternal);
        // double-float over the leftovers in the natural order (the FP32 pass
        // is done with d_qo_); what it cannot vouch for is queued for the
        // views' exact form (host side, after the graph)
        launch_flag_compact(views, nviews, total, d_flag_, d_fsum_, d_qo_, st_);
        a.order = nullptr;
        a.rerun_flag = nullptr;
        a.queue = d_qo_;
        a.queue_n = &d_ctr_[c0].rerun_n;
        a.ctr = d_ctr_ + c0 + 1;
        a.next_queue = d_qb_;
        launch_batch_pass(1, a, nsm, st_);
    };
    tiers(d_probe_, probe_total, 0, d_view_interior_, nullptr, true);
    launch_batch_gate(d_main_, nviews, d_view_interior_, st_);
    if (schedule_) {
        sched_probe_grid(d_probe_, d_main_, nviews, probe_total, st_);
        sched_order(sched_, d_main_, nviews, main_total, tile_total, nsm, d_qo_, st_);
        tiers(d_main_, main_total, 2, nullptr, d_qo_, false);
        if (schedule_ == 1) sched_train(sched_, d_main_, nviews, tile_total, kSchedTrainSteps, 2e-3f, st_);
    } else {
        tiers(d_main_, main_total, 2, nullptr, nullptr, false);
    }
    cudaMemcpyAsync(h_ctr_, d_ctr_, 4 * sizeof(Counters), cudaMemcpyDeviceToHost, st_);
    e = cudaStreamEndCapture(st_, &graph_);
    if (e != cudaSuccess) return cuda_fail(err, "graph capture", e);
    e = cudaGraphInstantiate(&exec_, graph_, 0);
    if (e != cudaSuccess) return cuda_fail(err, "graph instantiation", e);
    g_views_ = nviews;
    g_probe_ = probe_total;
    g_main_ = main_total;
    g_tiles_ = tile_total;
    g_cancel_ = cancel_flag;
    g_schedule_ = schedule_;
    g_deriv_ = deriv;
    return MBX_OK;
}

int BatchRunner::run(const mbx_request* reqs, int n, mbx_stats* view_stats, mbx_stats* batch_stats, volatile int* cancel_flag, std::string& err) {
    if (n < 1 || n > kBatchMaxViews) {
        err = "batch size must be in [1, 256]";
        return MBX_E_INVALID;
    }
    int rc = ensure_engines(n, err);
    if (rc != MBX_OK) return rc;
    std::vector<BatchSlot> slots(n);
    std::vector<mbx_stats> vst(n);
    for (int i = 0; i < n; ++i) slots[i].want_cost = schedule_ != 0;
    {
        // The frames' host work (GMP reference orbits, nucleus searches) is
        // independent per engine: up to `lanes` engines build concurrently,
        // each thread with its own product helpers (up to seven threads each
        // while a loop runs), so the lane count follows the host's cores.
        // A frame of at least direct_pixels_ pixels fills the GPU by itself:
        // unless the learned ordering wants every frame in the shared graph,
        // it renders on its own engine's stream as soon as its host work is
        // done, overlapping the other frames' host work (its thread then
        // mostly waits on the stream, hence up to one more lane).
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        int direct = 0;
        std::vector<char> is_direct((size_t)n, 0);
        for (int i = 0; i < n; ++i) {
            const long long px = (long long)reqs[i].width * reqs[i].height;
            if (schedule_ == 0 && direct_pixels_ > 0 && px >= direct_pixels_) {
                is_direct[(size_t)i] = 1;
                ++direct;
            }
        }
        const int lanes = std::max(1, std::min({n, 4, (int)(hw / 7) + (direct ? 1 : 0)}));
        std::vector<int> rcs((size_t)n, MBX_OK);
        auto work = [&](int t) {
            for (int i = t; i < n; i += lanes)
                rcs[(size_t)i] = is_direct[(size_t)i] ? eng_[i]->compute(reqs[i], &vst[i]) : eng_[i]->compute_deferred(reqs[i], &slots[i], &vst[i]);
        };
        std::vector<std::thread> th;
        for (int t = 1; t < lanes; ++t) th.emplace_back(work, t);
        work(0);
        for (auto& x : th) x.join();
        for (int i = 0; i < n; ++i)
            if (rcs[(size_t)i] != MBX_OK) {
                err = eng_[i]->error();
                return rcs[(size_t)i];
            }
    }
    std::vector<int> deferred;
    for (int i = 0; i < n; ++i)
        if (slots[i].deferred) deferred.push_back(i);
    mbx_stats bs = mbx_stats();
    if (!deferred.empty()) {
        const int nv = (int)deferred.size();
        unsigned probe_total = 0, main_total = 0, tile_total = 0;
        for (int k = 0; k < nv; ++k) {
            const int i = deferred[k];
            if (reqs[i].height * reqs[i].sub >= (1 << 16)) {
                err = "batched frames must have fewer than 65536 sample rows";
                return MBX_E_INVALID;
            }
            slots[i].probe.base = probe_total;
            slots[i].main.base = main_total;
            slots[i].probe.tile_base = slots[i].main.tile_base = tile_total;
            probe_total += slots[i].probe.count;
            main_total += slots[i].main.count;
            tile_total += (unsigned)(slots[i].main.tw * slots[i].main.th);
        }
        rc = ensure_buffers(nv, std::max(probe_total, main_total), tile_total, err);
        if (rc != MBX_OK) return rc;
        for (int k = 0; k < nv; ++k) {
            h_desc_[k] = slots[deferred[k]].probe;
            h_desc_[nv + k] = slots[deferred[k]].main;
        }
        // the engines prepared their frames on their own streams
        for (int k = 0; k < nv; ++k) {
            cudaError_t e = cudaStreamSynchronize(eng_[deferred[k]]->stream());
            if (e != cudaSuccess) return cuda_fail(err, "batch preparation", e);
        }
        if (schedule_)
            for (int k = 0; k < nv; ++k)
                if (!h_desc_[k].f.out.cost || !h_desc_[nv + k].pgrid) {
                    err = "scheduling buffers could not be allocated";
                    return MBX_E_NOMEM;
                }
        h_main_total_ = main_total;
        cudaMemcpyAsync(d_main_total_, &h_main_total_, sizeof(unsigned), cudaMemcpyHostToDevice, st_);
        cudaMemcpyAsync(d_probe_, h_desc_, sizeof(ViewDesc) * nv, cudaMemcpyHostToDevice, st_);
        cudaMemcpyAsync(d_main_, h_desc_ + nv, sizeof(ViewDesc) * nv, cudaMemcpyHostToDevice, st_);
        bs.h2d_bytes += (long long)(sizeof(unsigned) + 2 * sizeof(ViewDesc) * nv);
        int deriv = 0;
        for (int k = 0; k < nv; ++k) deriv |= h_desc_[nv + k].p.g.deriv ? 1 : 0;
        rc = build_graph(nv, probe_total, main_total, tile_total, cancel_flag, deriv, err);
        if (rc != MBX_OK) return rc;
        cudaEventRecord(ev0_, st_);
        cudaError_t e = cudaGraphLaunch(exec_, st_);
        if (e != cudaSuccess) return cuda_fail(err, "graph launch", e);
        cudaEventRecord(ev1_, st_);
        e = cudaStreamSynchronize(st_);
        if (e != cudaSuccess) return cuda_fail(err, "batched passes", e);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev0_, ev1_);
        if (cancel_flag && *cancel_flag) {
            err = "cancelled";
            return MBX_E_CANCELLED;
        }
        if (schedule_) {
            int terr = 0;
            e = cudaMemcpy(&terr, sched_.err, sizeof(int), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return cuda_fail(err, "scheduler status", e);
            if (terr) {
                err = "ordering model: a tensor-core completion wait ran out of its limit";
                return MBX_E_CUDA;
            }
        }
        bs.pass_gpu_ms = ms;
        // the main FP32 pass alone; the rest of the graph's main part is the
        // regrouping and the double-float tier
        float f32 = 0.0f, rest = 0.0f;
        if (cudaEventElapsedTime(&f32, evm_[0], evm_[1]) == cudaSuccess && cudaEventElapsedTime(&rest, evm_[1], ev1_) == cudaSuccess) {
            bs.fp32_pass_gpu_ms = f32;
            bs.rerun_gpu_ms = rest;
        } else {
            (void)cudaGetLastError(); // no split: leave no error behind for later calls
        }
        bs.d2h_bytes += (long long)(4 * sizeof(Counters)); // the graph's counter readback
        // probe FP32; gate; main FP32; regrouping (3); double-float (two widths); ordering and training
        bs.kernel_launches = 8 + (schedule_ ? 6 + (schedule_ == 1 ? sched_train_launches(kSchedTrainSteps) : 0) : 0);
        bs.passes = 2;
        for (int c = 0; c < 4; ++c) {
            const Counters& k = h_ctr_[c];
            bs.steps += (long long)k.steps;
            bs.bla_applies += (long long)k.bla_applies;
            bs.bla_skipped += (long long)k.bla_skipped;
            bs.effective_iterations += (long long)k.effective_iters;
            bs.interior += (int)k.interior;
            bs.rebases += (long long)k.rebases;
            bs.exact_steps += (long long)k.exact_steps;
            bs.fe_rebases += (long long)k.fe_rebases;
        }
        bs.fp64_reruns = (long long)h_ctr_[2].rerun_n; // the main pass's queues (the probe's are not rerun)
        bs.fp64_reruns_fp64 = (long long)h_ctr_[3].rerun_n;
        bs.samples = (int)(probe_total + main_total);
        const unsigned want[2] = {probe_total, main_total};
        for (int ph = 0; ph < 2; ++ph) {
            const Counters* c = h_ctr_ + 2 * ph;
            // every sample finishes in the FP32 pass or one of the queues it
            // feeds (the probe has no rerun tiers)
            if (c[0].finished != want[ph] || (ph == 1 && c[1].finished != std::min(c[0].rerun_n, cap_samples_))) {
                err = "batched pass left samples unfinished";
                return MBX_E_CUDA;
            }
        }
        // samples the double-float tier could not vouch for: each view's exact
        // form finishes its own (keys carry the view's position among the deferred)
        const unsigned n_exact = std::min(h_ctr_[3].rerun_n, cap_samples_);
        bs.exact_reruns = (long long)n_exact;
        if (n_exact > 0) {
            std::vector<uint64_t> q(n_exact);
            cudaMemcpyAsync(q.data(), d_qb_, sizeof(uint64_t) * n_exact, cudaMemcpyDeviceToHost, st_);
            e = cudaStreamSynchronize(st_);
            if (e != cudaSuccess) return cuda_fail(err, "double-float rerun readback", e);
            std::vector<unsigned> vint((size_t)nv);
            cudaMemcpyAsync(vint.data(), d_view_interior_, sizeof(unsigned) * nv, cudaMemcpyDeviceToHost, st_);
            bs.d2h_bytes += (long long)(sizeof(uint64_t) * n_exact + sizeof(unsigned) * nv);
            e = cudaStreamSynchronize(st_);
            if (e != cudaSuccess) return cuda_fail(err, "interior gate readback", e);
            std::vector<std::vector<uint64_t>> per((size_t)nv);
            for (uint64_t k : q) {
                const int v = (int)(k >> kBatchViewShift);
                if (v < 0 || v >= nv) {
                    err = "batched rerun queue holds a bad view index";
                    return MBX_E_CUDA;
                }
                per[(size_t)v].push_back(k & ((1ull << kBatchViewShift) - 1ull));
            }
            // each view's leftovers are a few long FP64 dependency chains: the
            // engines run them on their own streams from concurrent host
            // threads, so the views' chains overlap on the device
            std::vector<int> ex;
            for (int k = 0; k < nv; ++k)
                if (!per[(size_t)k].empty()) ex.push_back(k);
            const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
            const int lanes = std::max(1, std::min({(int)ex.size(), 16, (int)hw}));
            std::vector<int> rcs(ex.size(), MBX_OK);
            auto work = [&](int t) {
                for (size_t q = (size_t)t; q < ex.size(); q += (size_t)lanes) {
                    const int k = ex[q];
                    rcs[q] = eng_[deferred[k]]->batch_exact_rerun(per[(size_t)k], vint[(size_t)k] > 0);
                }
            };
            const auto t0 = std::chrono::steady_clock::now();
            std::vector<std::thread> th;
            for (int t = 1; t < lanes; ++t) th.emplace_back(work, t);
            work(0);
            for (auto& x : th) x.join();
            bs.rerun_fp64_gpu_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            for (size_t q = 0; q < ex.size(); ++q)
                if (rcs[q] != MBX_OK) {
                    err = eng_[deferred[ex[q]]]->error();
                    return rcs[q];
                }
        }
        {
            // supersampled frames: each engine's adaptive-supersampling passes on
            // its own stream, driven from concurrent host threads so that the
            // frames' passes overlap on the device
            std::vector<unsigned> vint((size_t)nv, 0u);
            cudaMemcpyAsync(vint.data(), d_view_interior_, sizeof(unsigned) * nv, cudaMemcpyDeviceToHost, st_);
            bs.d2h_bytes += (long long)(sizeof(unsigned) * nv);
            e = cudaStreamSynchronize(st_);
            if (e != cudaSuccess) return cuda_fail(err, "interior gate readback", e);
            std::vector<int> ss;
            for (int k = 0; k < nv; ++k)
                if (reqs[deferred[k]].sub > 1) ss.push_back(k);
            if (!ss.empty()) {
                const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
                const int lanes = std::max(1, std::min({(int)ss.size(), 8, (int)hw}));
                std::vector<int> rcs(ss.size(), MBX_OK);
                auto work = [&](int t) {
                    for (size_t q = (size_t)t; q < ss.size(); q += (size_t)lanes) rcs[q] = eng_[deferred[ss[q]]]->batch_supersample(vint[(size_t)ss[q]] > 0);
                };
                std::vector<std::thread> th;
                for (int t = 1; t < lanes; ++t) th.emplace_back(work, t);
                work(0);
                for (auto& x : th) x.join();
                for (size_t q = 0; q < ss.size(); ++q)
                    if (rcs[q] != MBX_OK) {
                        err = eng_[deferred[ss[q]]]->error();
                        return rcs[q];
                    }
            }
        }
        for (int k = 0; k < nv; ++k) {
            const int i = deferred[k];
            rc = eng_[i]->batch_finish(reqs[i], &vst[i]);
            if (rc != MBX_OK) {
                err = eng_[i]->error();
                return rc;
            }
        }
    }
    if (view_stats)
        for (int i = 0; i < n; ++i) view_stats[i] = vst[i];
    if (batch_stats) *batch_stats = bs;
    return MBX_OK;
}

} // namespace mbx

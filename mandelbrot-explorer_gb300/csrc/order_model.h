// Learned work ordering of the batched passes (order_model.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kernels.h"

namespace mbx {

// Offsets of the model parameters (FP32 masters) in one flat array:
// W1 [64][24], b1 [64], W2 [64][64], b2 [64], w3 [64], b3.
struct SchedLayout {
    static constexpr int W1 = 0;
    static constexpr int B1 = W1 + 64 * 24;
    static constexpr int W2 = B1 + 64;
    static constexpr int B2 = W2 + 64 * 64;
    static constexpr int W3 = B2 + 64;
    static constexpr int B3 = W3 + 64;
    static constexpr int N = B3 + 1;
};
constexpr int kSchedSamples = 8192;  // training samples taken from each batch
constexpr int kSchedTrainSteps = 32; // Adam steps (128-sample minibatches) per batch
constexpr int kSchedFeatures = 32;  // features per sample as stored (24 used)

// Device state of the model and the ordering.
struct SchedState {
    float* params = nullptr;   // SchedLayout::N
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    int* ready = nullptr;      // 1 once trained
    int* steps = nullptr;      // Adam steps taken
    float* loss = nullptr;     // mean loss of the last training launch
    unsigned* hist = nullptr;   // per-warp bucket counts, then offsets (32 per 1024 samples)
    unsigned* cursor = nullptr; // unused
    uint8_t* bucket = nullptr;  // per main-pass sample
    __nv_bfloat16* X = nullptr; // training features [kSchedSamples][32]
    float* T = nullptr;         // training targets
};

size_t sched_train_smem();
cudaError_t sched_init(SchedState& s, cudaStream_t st);
// probe costs -> each view's probe grid (main[v].pgrid)
cudaError_t sched_probe_grid(const ViewDesc* probe, const ViewDesc* main, int nv, unsigned probe_total, cudaStream_t st);
// ordered queue of the main-pass keys (view index in the top byte)
cudaError_t sched_order(SchedState& s, const ViewDesc* main, int nv, unsigned total, int nsm, uint64_t* out, cudaStream_t st);
// collect a training set from the main pass's measured costs and train
cudaError_t sched_train(SchedState& s, const ViewDesc* main, int nv, unsigned total, int steps, float lr, cudaStream_t st);
// one step's gradients for given samples (no update)
cudaError_t sched_gradient(SchedState& s, const __nv_bfloat16* X, const float* T, int n, float* grad_out, cudaStream_t st);

} // namespace mbx

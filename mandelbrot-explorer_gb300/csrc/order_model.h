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
constexpr int kSchedTiles = 32768;   // training tiles taken from each batch (at most)
constexpr int kSchedTrainSteps = 32; // Adam steps per batch (minibatches of 16 x 128 tiles)
constexpr int kSchedFeatures = 32;  // features per tile as stored (24 used)

// Device state of the model and the ordering.
struct SchedState {
    float* params = nullptr;   // SchedLayout::N
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    int* ready = nullptr;      // 1 once trained
    int* steps = nullptr;      // Adam steps taken
    float* loss = nullptr;     // mean loss of the last training launch
    unsigned* hist = nullptr;   // ordering scratch (sched_scratch_words): bin counts / cursors, view costs and ranks
    uint16_t* bucket = nullptr; // per main-pass sample: its bin (view rank, tile bucket)
    uint8_t* tile_bucket = nullptr; // per 16x16 tile of the batch
    __nv_bfloat16* X = nullptr; // training features [kSchedTiles][32]
    float* T = nullptr;         // training targets
    float* grad = nullptr;      // summed gradients of one training step
    int* err = nullptr;         // a tensor-core wait ran out of its iteration limit
};

size_t sched_train_smem();
size_t sched_scratch_words();
cudaError_t sched_init(SchedState& s, cudaStream_t st);
// probe costs -> each view's probe grid (main[v].pgrid)
cudaError_t sched_probe_grid(const ViewDesc* probe, const ViewDesc* main, int nv, unsigned probe_total, cudaStream_t st);
// the main FP32 pass's order (batch-wide sample indices): the model's
// prediction per tile, views and their samples sorted by predicted cost
cudaError_t sched_order(SchedState& s, const ViewDesc* main, int nv, unsigned total, unsigned ntiles, int nsm, uint64_t* out, cudaStream_t st);
// collect a training set (tiles, their measured mean costs) and train `steps` Adam steps
cudaError_t sched_train(SchedState& s, const ViewDesc* main, int nv, unsigned ntiles, int steps, float lr, cudaStream_t st);
int sched_train_rows(unsigned ntiles);
int sched_train_launches(int steps); // kernel launches of sched_train
// the summed gradients over n given rows (features bf16 [n][32]), no update
cudaError_t sched_gradient(SchedState& s, const __nv_bfloat16* X, const float* T, int n, float* grad_out, cudaStream_t st);

} // namespace mbx

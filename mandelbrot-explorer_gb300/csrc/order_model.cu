// Learned work ordering for the batched passes.
//
// A BF16 multilayer perceptron (24 -> 64 -> 64 -> 1, ReLU) predicts each
// sample's cost (log2 of 1 + the lane steps it takes) from the probe pass's
// costs around it and a few view features. Before the main FP32 pass the
// samples of all views are bucket-sorted by decreasing predicted cost, so long
// samples start first and do not trail the launch; after it, the model trains
// on a fixed subset of the samples' measured costs (Adam, a few hundred
// minibatch steps), ready for the next batch. The order changes nothing in
// the outputs: every sample's iteration depends only on its own coordinates.
//
// Tensor cores: all products (inference, and the training step's forward,
// input-gradient and weight-gradient products) are mma.sync m16n8k16 with BF16
// operands and FP32 accumulation, operands staged in shared memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "order_model.h"

namespace mbx {
namespace {

constexpr int kIn = 24, kInPad = 32, kHid = 64;
constexpr int kBuckets = 32;       // half-octaves of predicted cost (one per lane)
constexpr unsigned kWarpSpan = 1024; // samples per warp in the bucket sort

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<unsigned*>(&v);
}

// D += A(16x16, row-major) B(16x8, column-major); fragments per the PTX ISA
// (mma.m16n8k16: a0..a3, b0..b1, c0..c3).
__device__ __forceinline__ void mma_bf16(float* d, const unsigned* a, const unsigned* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment of a 16-row tile from a row-major bf16 matrix in shared memory
// (row stride `ld` elements), k-step ks (16 columns).
__device__ __forceinline__ void load_a(unsigned* a, const __nv_bfloat16* m, int ld, int ks, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* r0 = m + g * ld + ks * 16 + 2 * t;
    const __nv_bfloat16* r1 = m + (g + 8) * ld + ks * 16 + 2 * t;
    a[0] = *reinterpret_cast<const unsigned*>(r0);
    a[1] = *reinterpret_cast<const unsigned*>(r1);
    a[2] = *reinterpret_cast<const unsigned*>(r0 + 8);
    a[3] = *reinterpret_cast<const unsigned*>(r1 + 8);
}
// B fragment (16 x 8, k-step ks, n-tile nt) from an [N][K] bf16 matrix in
// shared memory (K contiguous, row stride `ld`).
__device__ __forceinline__ void load_b(unsigned* b, const __nv_bfloat16* m, int ld, int ks, int nt, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* r = m + (nt * 8 + g) * ld + ks * 16 + 2 * t;
    b[0] = *reinterpret_cast<const unsigned*>(r);
    b[1] = *reinterpret_cast<const unsigned*>(r + 8);
}

// Feature vector of sample (i, j) of a view (24 values, zero padded to 32).
__device__ void features(const ViewDesc& vd, int i, int j, float* f) {
    const int gw = vd.pgw, gh = vd.pgh;
    const int a = i >> 3, b = j >> 3;
    auto P = [&](int aa, int bb) -> float2 {
        aa = max(0, min(gh - 1, aa));
        bb = max(0, min(gw - 1, bb));
        return vd.pgrid[aa * gw + bb];
    };
    const float2 p00 = P(a, b), p10 = P(a + 1, b), p01 = P(a, b + 1), p11 = P(a + 1, b + 1);
    const float u = (i - 8 * a) * 0.125f, v = (j - 8 * b) * 0.125f;
    f[0] = p00.x;
    f[1] = p10.x;
    f[2] = p01.x;
    f[3] = p11.x;
    f[4] = p00.y;
    f[5] = p10.y;
    f[6] = p01.y;
    f[7] = p11.y;
    f[8] = u;
    f[9] = v;
    f[10] = (1 - u) * (1 - v) * p00.x + u * (1 - v) * p10.x + (1 - u) * v * p01.x + u * v * p11.x;
    const float mn = fminf(fminf(p00.x, p10.x), fminf(p01.x, p11.x)), mx = fmaxf(fmaxf(p00.x, p10.x), fmaxf(p01.x, p11.x));
    f[11] = mn;
    f[12] = mx;
    f[13] = mx - mn;
    f[14] = 0.25f * (p00.y + p10.y + p01.y + p11.y);
    f[15] = P(a - 1, b).x;
    f[16] = P(a + 2, b).x;
    f[17] = P(a, b - 1).x;
    f[18] = P(a, b + 2).x;
    f[19] = (float)i / (float)vd.p.g.H - 0.5f;
    f[20] = (float)j / (float)vd.p.g.W - 0.5f;
    f[21] = log2f((float)vd.p.g.mxit) * (1.0f / 24.0f);
    f[22] = vd.p.per > 0 ? 1.0f : 0.0f;
    f[23] = 1.0f;
    for (int k = kIn; k < kInPad; ++k) f[k] = 0.0f;
}

__device__ __forceinline__ int find_view(const ViewDesc* views, int nv, unsigned g) {
    int lo = 0, hi = nv - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (views[mid].base <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Shared-memory copy of the model for the products: weights in bf16, [out][in].
struct SmemModel {
    __nv_bfloat16 w1[kHid * kInPad];
    __nv_bfloat16 w2[kHid * kHid];
    float b1[kHid], b2[kHid], w3[kHid];
    float b3;
};

__device__ void stage_model(SmemModel& s, const float* P) {
    const float* w1 = P + SchedLayout::W1;
    const float* w2 = P + SchedLayout::W2;
    for (int k = threadIdx.x; k < kHid * kInPad; k += blockDim.x) {
        const int o = k / kInPad, in = k % kInPad;
        s.w1[k] = __float2bfloat16_rn(in < kIn ? w1[o * kIn + in] : 0.0f);
    }
    for (int k = threadIdx.x; k < kHid * kHid; k += blockDim.x) s.w2[k] = __float2bfloat16_rn(w2[k]);
    for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
        s.b1[k] = P[SchedLayout::B1 + k];
        s.b2[k] = P[SchedLayout::B2 + k];
        s.w3[k] = P[SchedLayout::W3 + k];
    }
    if (threadIdx.x == 0) s.b3 = P[SchedLayout::B3];
}

// Forward pass of one 16-sample tile held by a warp: x (16 x 32 bf16, row
// stride 32) in shared memory. Returns the prediction of rows g and g + 8 in
// y[0], y[1] (valid in every lane of the group). h1 / h2 (16 x 64 bf16) and the
// pre-activation signs are written when the pointers are non-null (training).
__device__ void forward_tile(const SmemModel& m, const __nv_bfloat16* x, __nv_bfloat16* h1, __nv_bfloat16* h2, int lane, float* y) {
    const int g = lane >> 2, t = lane & 3;
    float acc[8][4];
    // layer 1
    for (int nt = 0; nt < 8; ++nt)
        for (int q = 0; q < 4; ++q) acc[nt][q] = 0.0f;
    for (int ks = 0; ks < kInPad / 16; ++ks) {
        unsigned a[4];
        load_a(a, x, kInPad, ks, lane);
        for (int nt = 0; nt < 8; ++nt) {
            unsigned b[2];
            load_b(b, m.w1, kInPad, ks, nt, lane);
            mma_bf16(acc[nt], a, b);
        }
    }
    // bias + ReLU; C fragments become layer 2's A fragments in registers
    unsigned a2[4][4];
    for (int nt = 0; nt < 8; ++nt) {
        const int c0 = nt * 8 + 2 * t;
        const float v0 = fmaxf(acc[nt][0] + m.b1[c0], 0.0f), v1 = fmaxf(acc[nt][1] + m.b1[c0 + 1], 0.0f);
        const float v2 = fmaxf(acc[nt][2] + m.b1[c0], 0.0f), v3 = fmaxf(acc[nt][3] + m.b1[c0 + 1], 0.0f);
        const unsigned lo = pack_bf16(v0, v1), hi = pack_bf16(v2, v3);
        a2[nt >> 1][(nt & 1) ? 2 : 0] = lo;
        a2[nt >> 1][(nt & 1) ? 3 : 1] = hi;
        if (h1) {
            *reinterpret_cast<unsigned*>(h1 + g * kHid + c0) = lo;
            *reinterpret_cast<unsigned*>(h1 + (g + 8) * kHid + c0) = hi;
        }
    }
    // layer 2
    for (int nt = 0; nt < 8; ++nt)
        for (int q = 0; q < 4; ++q) acc[nt][q] = 0.0f;
    for (int ks = 0; ks < kHid / 16; ++ks)
        for (int nt = 0; nt < 8; ++nt) {
            unsigned b[2];
            load_b(b, m.w2, kHid, ks, nt, lane);
            mma_bf16(acc[nt], a2[ks], b);
        }
    // bias + ReLU, then the output row sums (layer 3 on the CUDA cores)
    float s0 = 0.0f, s1 = 0.0f;
    for (int nt = 0; nt < 8; ++nt) {
        const int c0 = nt * 8 + 2 * t;
        const float v0 = fmaxf(acc[nt][0] + m.b2[c0], 0.0f), v1 = fmaxf(acc[nt][1] + m.b2[c0 + 1], 0.0f);
        const float v2 = fmaxf(acc[nt][2] + m.b2[c0], 0.0f), v3 = fmaxf(acc[nt][3] + m.b2[c0 + 1], 0.0f);
        // layer 3 consumes the same bf16-rounded activations the backward pass sees
        const unsigned lo = pack_bf16(v0, v1), hi = pack_bf16(v2, v3);
        const __nv_bfloat162 l = *reinterpret_cast<const __nv_bfloat162*>(&lo), h = *reinterpret_cast<const __nv_bfloat162*>(&hi);
        s0 += __low2float(l) * m.w3[c0] + __high2float(l) * m.w3[c0 + 1];
        s1 += __low2float(h) * m.w3[c0] + __high2float(h) * m.w3[c0 + 1];
        if (h2) {
            *reinterpret_cast<unsigned*>(h2 + g * kHid + c0) = lo;
            *reinterpret_cast<unsigned*>(h2 + (g + 8) * kHid + c0) = hi;
        }
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
    s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
    y[0] = s0 + m.b3;
    y[1] = s1 + m.b3;
}

// ---- probe grid -------------------------------------------------------------
__global__ void k_probe_grid(const ViewDesc* probe, const ViewDesc* main, int nv, unsigned total) {
    const unsigned g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int v = find_view(probe, nv, g);
    const ViewDesc& pd = probe[v];
    int arr[4];
    entry_coords(pd.f.px, (int)(g - pd.base), arr);
    const int oidx = arr[0] * pd.p.g.W + arr[1];
    const float c = pd.f.out.cost ? (float)pd.f.out.cost[oidx] : 0.0f;
    const float interior = pd.f.out.iter[oidx] == -2.0f ? 1.0f : 0.0f;
    main[v].pgrid[(arr[0] >> 3) * main[v].pgw + (arr[1] >> 3)] = make_float2(log2f(1.0f + c) * (1.0f / 24.0f), interior);
}

// ---- prediction + stable bucket sort ----------------------------------------
// One warp per 16-sample tile: features, MLP, bucket of the predicted cost in
// half-octaves, descending (bucket 0 holds the most expensive samples).
__global__ void __launch_bounds__(128) k_predict(const ViewDesc* views, int nv, unsigned total, const float* P, const int* ready, uint8_t* bucket) {
    __shared__ SmemModel m;
    __shared__ __align__(16) __nv_bfloat16 xs[4][16 * kInPad];
    stage_model(m, P);
    __syncthreads();
    if (*ready == 0) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned tiles = (total + 15) / 16;
    for (unsigned tile = blockIdx.x * 4 + warp; tile < tiles; tile += gridDim.x * 4) {
        // lanes 0..15 build one row each
        if (lane < 16) {
            const unsigned g = tile * 16 + lane;
            float f[kInPad];
            if (g < total) {
                const int v = find_view(views, nv, g);
                int arr[4];
                entry_coords(views[v].f.px, (int)(g - views[v].base), arr);
                features(views[v], arr[0], arr[1], f);
            } else {
                for (int k = 0; k < kInPad; ++k) f[k] = 0.0f;
            }
            for (int k = 0; k < kInPad; k += 2) *reinterpret_cast<unsigned*>(&xs[warp][lane * kInPad + k]) = pack_bf16(f[k], f[k + 1]);
        }
        __syncwarp();
        float y[2];
        forward_tile(m, xs[warp], nullptr, nullptr, lane, y);
        __syncwarp();
        if ((lane & 3) == 0) {
            for (int h = 0; h < 2; ++h) {
                const unsigned g = tile * 16 + (lane >> 2) + 8 * h;
                if (g >= total) continue;
                // prediction in log2(1 + steps) / 24 -> half-octave buckets
                const int b = max(0, min(kBuckets - 1, (int)(y[h] * 24.0f * 2.0f)));
                bucket[g] = (uint8_t)(kBuckets - 1 - b);
            }
        }
    }
}

// Stable counting sort: every warp owns kWarpSpan consecutive samples.
// 1) per-warp bucket counts;
__global__ void __launch_bounds__(256) k_bucket_count(unsigned total, const uint8_t* bucket, unsigned* cnt) {
    const unsigned w = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    unsigned c = 0; // lane b counts bucket b
    const unsigned g0 = w * kWarpSpan;
    for (unsigned k = 0; k < kWarpSpan; k += 32) {
        const unsigned g = g0 + k + lane;
        const int d = g < total ? bucket[g] : -1;
        for (int b = 0; b < kBuckets; ++b) {
            const unsigned m = __ballot_sync(0xffffffffu, d == b);
            if ((int)lane == b) c += __popc(m);
        }
    }
    cnt[w * kBuckets + lane] = c;
}
// 2) offsets in bucket-major, warp-minor order (one block, lane b = bucket b of
//    warp group; the warps are walked in order);
__global__ void k_bucket_offsets(unsigned nw, unsigned* cnt) {
    __shared__ unsigned tot[kBuckets];
    const int b = threadIdx.x;
    if (b < kBuckets) {
        unsigned run = 0;
        for (unsigned w = 0; w < nw; ++w) {
            const unsigned c = cnt[w * kBuckets + b];
            cnt[w * kBuckets + b] = run;
            run += c;
        }
        tot[b] = run;
    }
    __syncthreads();
    if (b < kBuckets) {
        unsigned base = 0;
        for (int q = 0; q < b; ++q) base += tot[q];
        for (unsigned w = 0; w < nw; ++w) cnt[w * kBuckets + b] += base;
    }
}
// 3) placement: each warp walks its samples in order, ranking equal buckets
//    within each 32-sample piece, so the natural order survives within a bucket.
__global__ void __launch_bounds__(256) k_bucket_place(const ViewDesc* views, int nv, unsigned total, const int* ready, const uint8_t* bucket, const unsigned* off,
                                                      uint64_t* out) {
    const unsigned w = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    unsigned run = *ready ? off[w * kBuckets + lane] : 0; // lane b: next position of bucket b
    const unsigned g0 = w * kWarpSpan;
    for (unsigned k = 0; k < kWarpSpan; k += 32) {
        const unsigned g = g0 + k + lane;
        const bool in = g < total;
        if (__ballot_sync(0xffffffffu, in) == 0) break;
        uint64_t key = 0;
        if (in) {
            const int v = find_view(views, nv, g);
            int arr[4];
            entry_coords(views[v].f.px, (int)(g - views[v].base), arr);
            key = key_pack(arr[0], arr[1], arr[2], arr[3]) | ((uint64_t)v << kBatchViewShift);
        }
        if (!*ready) {
            if (in) out[g] = key;
            continue;
        }
        const int d = in ? bucket[g] : kBuckets; // out-of-range lanes form their own group
        const unsigned same = __match_any_sync(0xffffffffu, d);
        const unsigned rank = __popc(same & ((1u << lane) - 1u));
        const unsigned base = __shfl_sync(0xffffffffu, run, d < kBuckets ? d : 0);
        if (in) out[base + rank] = key;
        // advance each bucket's position by its count in this piece
        for (int b = 0; b < kBuckets; ++b) {
            const unsigned m = __ballot_sync(0xffffffffu, in && d == b);
            if ((int)lane == b) run += __popc(m);
        }
    }
}

// ---- training ---------------------------------------------------------------
// Training set: kSchedSamples main-pass samples at a fixed stride; features
// in bf16, target log2(1 + measured cost) / 24.
__global__ void k_collect(const ViewDesc* views, int nv, unsigned total, __nv_bfloat16* X, float* T, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned g = (unsigned)(((unsigned long long)k * 2654435761ull) % total);
    const int v = find_view(views, nv, g);
    int arr[4];
    entry_coords(views[v].f.px, (int)(g - views[v].base), arr);
    float f[kInPad];
    features(views[v], arr[0], arr[1], f);
    for (int q = 0; q < kInPad; ++q) X[k * kInPad + q] = __float2bfloat16_rn(f[q]);
    const uint32_t c = views[v].f.out.cost[arr[0] * views[v].p.g.W + arr[1]];
    T[k] = log2f(1.0f + (float)c) * (1.0f / 24.0f);
}

// One block of 256 threads (8 warps, a 128-sample minibatch: one 16-row tile
// per warp). steps minibatch steps over the n-sample set with Adam; with
// grad_out non-null, one step with no update that writes the gradients.
constexpr int kBatch = 128;
struct TrainSmem {
    SmemModel m;
    __nv_bfloat16 x[kBatch * kInPad];
    __nv_bfloat16 xt[kInPad * kBatch];  // x transposed: [in][batch]
    __nv_bfloat16 h1[kBatch * kHid];
    __nv_bfloat16 h1t[kHid * kBatch];
    __nv_bfloat16 h2[kBatch * kHid];
    __nv_bfloat16 dz2[kBatch * kHid];   // [batch][out], layer 2 pre-activation gradient
    __nv_bfloat16 dz2t[kHid * kBatch];  // [out][batch]
    __nv_bfloat16 dz1t[kHid * kBatch];
    __nv_bfloat16 w2t[kHid * kHid];     // [in][out]
    float dy[kBatch];
    float grad[SchedLayout::N];
};

__global__ void __launch_bounds__(256) k_train(float* P, float* Madam, float* Vadam, int* ready, int* step_count, const __nv_bfloat16* X, const float* T, int n, int steps,
                                             float lr, float* grad_out, float* loss_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float loss_acc = 0.0f;
    for (int st = 0; st < steps; ++st) {
        stage_model(s.m, P);
        for (int k = threadIdx.x; k < kHid * kHid; k += blockDim.x) {
            const int o = k / kHid, in = k % kHid;
            s.w2t[in * kHid + o] = s.m.w2[k];
        }
        for (int k = threadIdx.x; k < SchedLayout::N; k += blockDim.x) s.grad[k] = 0.0f;
        const int base = (int)(((long long)st * kBatch) % (n > kBatch ? n - kBatch + 1 : 1));
        for (int k = threadIdx.x; k < kBatch * kInPad; k += blockDim.x) {
            const int r = k / kInPad, c = k % kInPad;
            const __nv_bfloat16 v = X[(size_t)(base + r) * kInPad + c];
            s.x[k] = v;
            s.xt[c * kBatch + r] = v;
        }
        __syncthreads();
        // forward: warp w owns rows 16w .. 16w + 15
        float y[2];
        forward_tile(s.m, s.x + warp * 16 * kInPad, s.h1 + warp * 16 * kHid, s.h2 + warp * 16 * kHid, lane, y);
        if (t == 0) {
            for (int h = 0; h < 2; ++h) {
                const int r = warp * 16 + g + 8 * h;
                const float e = y[h] - T[base + r];
                s.dy[r] = e * (1.0f / kBatch); // d(mean 1/2 e^2)
                loss_acc += 0.5f * e * e * (1.0f / kBatch);
            }
        }
        __syncthreads();
        // layer 3 gradients and dz2 = dy w3 (x) [h2 > 0]
        for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
            float a = 0.0f;
            for (int r = 0; r < kBatch; ++r) a += s.dy[r] * __bfloat162float(s.h2[r * kHid + k]);
            s.grad[SchedLayout::W3 + k] = a;
        }
        if (threadIdx.x == 0) {
            float a = 0.0f;
            for (int r = 0; r < kBatch; ++r) a += s.dy[r];
            s.grad[SchedLayout::B3] = a;
        }
        for (int k = threadIdx.x; k < kBatch * kHid; k += blockDim.x) {
            const int r = k / kHid, o = k % kHid;
            const float d = __bfloat162float(s.h2[k]) > 0.0f ? s.dy[r] * s.m.w3[o] : 0.0f;
            const __nv_bfloat16 db = __float2bfloat16_rn(d);
            s.dz2[k] = db;
            s.dz2t[o * kBatch + r] = db;
            s.h1t[o * kBatch + r] = s.h1[k]; // h1 [batch][64] -> [64][batch]
        }
        __syncthreads();
        // b2 gradient
        for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
            float a = 0.0f;
            for (int r = 0; r < kBatch; ++r) a += __bfloat162float(s.dz2t[k * kBatch + r]);
            s.grad[SchedLayout::B2 + k] = a;
        }
        // dW2[out][in] = sum_b dz2[b][out] h1[b][in]: M = out (64), N = in (64), K = batch;
        // warp w: out rows 16 (w & 3) .. +15, in columns 32 (w >> 2) .. +31
        {
            const int mt = warp & 3, nh = warp >> 2;
            float acc[4][4] = {};
            for (int ks = 0; ks < kBatch / 16; ++ks) {
                unsigned a[4];
                load_a(a, s.dz2t + mt * 16 * kBatch, kBatch, ks, lane);
                for (int q = 0; q < 4; ++q) {
                    unsigned b[2];
                    load_b(b, s.h1t, kBatch, ks, nh * 4 + q, lane);
                    mma_bf16(acc[q], a, b);
                }
            }
            for (int q = 0; q < 4; ++q) {
                const int o0 = mt * 16 + g, in0 = (nh * 4 + q) * 8 + 2 * t;
                s.grad[SchedLayout::W2 + o0 * kHid + in0] = acc[q][0];
                s.grad[SchedLayout::W2 + o0 * kHid + in0 + 1] = acc[q][1];
                s.grad[SchedLayout::W2 + (o0 + 8) * kHid + in0] = acc[q][2];
                s.grad[SchedLayout::W2 + (o0 + 8) * kHid + in0 + 1] = acc[q][3];
            }
        }
        // dh1 = dz2 W2 (per warp tile: rows 16w.., K = out 64, N = in 64), dz1 = dh1 [h1 > 0]
        {
            float acc[8][4] = {};
            for (int ks = 0; ks < kHid / 16; ++ks) {
                unsigned a[4];
                load_a(a, s.dz2 + warp * 16 * kHid, kHid, ks, lane);
                for (int nt = 0; nt < 8; ++nt) {
                    unsigned b[2];
                    load_b(b, s.w2t, kHid, ks, nt, lane);
                    mma_bf16(acc[nt], a, b);
                }
            }
            for (int nt = 0; nt < 8; ++nt) {
                const int c0 = nt * 8 + 2 * t;
                for (int h = 0; h < 2; ++h) {
                    const int r = warp * 16 + g + 8 * h;
                    for (int e = 0; e < 2; ++e) {
                        const float hv = __bfloat162float(s.h1[r * kHid + c0 + e]);
                        const float d = hv > 0.0f ? acc[nt][2 * h + e] : 0.0f;
                        s.dz1t[(c0 + e) * kBatch + r] = __float2bfloat16_rn(d);
                    }
                }
            }
        }
        __syncthreads();
        for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
            float a = 0.0f;
            for (int r = 0; r < kBatch; ++r) a += __bfloat162float(s.dz1t[k * kBatch + r]);
            s.grad[SchedLayout::B1 + k] = a;
        }
        // dW1[out][in] = sum_b dz1[b][out] x[b][in]: M = out 64, N = in 32 (24 used), K = batch;
        // warp w: out rows 16 (w & 3), in columns 16 (w >> 2) .. +15
        {
            const int mt = warp & 3, nh = warp >> 2;
            float acc[2][4] = {};
            for (int ks = 0; ks < kBatch / 16; ++ks) {
                unsigned a[4];
                load_a(a, s.dz1t + mt * 16 * kBatch, kBatch, ks, lane);
                for (int q = 0; q < 2; ++q) {
                    unsigned b[2];
                    load_b(b, s.xt, kBatch, ks, nh * 2 + q, lane);
                    mma_bf16(acc[q], a, b);
                }
            }
            for (int q = 0; q < 2; ++q) {
                const int o0 = mt * 16 + g, in0 = (nh * 2 + q) * 8 + 2 * t;
                for (int h = 0; h < 2; ++h)
                    for (int e = 0; e < 2; ++e) {
                        const int in = in0 + e;
                        if (in < kIn) s.grad[SchedLayout::W1 + (o0 + 8 * h) * kIn + in] = acc[q][2 * h + e];
                    }
            }
        }
        __syncthreads();
        if (grad_out) {
            for (int k = threadIdx.x; k < SchedLayout::N; k += blockDim.x) grad_out[k] = s.grad[k];
            break;
        }
        // Adam (beta1 0.9, beta2 0.999, eps 1e-8)
        const int it = *step_count + st + 1;
        const float c1 = 1.0f - powf(0.9f, (float)it), c2 = 1.0f - powf(0.999f, (float)it);
        for (int k = threadIdx.x; k < SchedLayout::N; k += blockDim.x) {
            const float gk = s.grad[k];
            const float mk = 0.9f * Madam[k] + 0.1f * gk, vk = 0.999f * Vadam[k] + 0.001f * gk * gk;
            Madam[k] = mk;
            Vadam[k] = vk;
            P[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + 1e-8f);
        }
        __syncthreads();
    }
    // loss of the steps (sum over threads of group leaders)
    for (int o = 16; o > 0; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    __shared__ float lsum[8];
    if (lane == 0) lsum[warp] = loss_acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float l = 0.0f;
        for (int w = 0; w < 8; ++w) l += lsum[w];
        if (loss_out) *loss_out = l / (steps > 0 ? (grad_out ? 1 : steps) : 1);
        if (!grad_out) {
            *step_count += steps;
            *ready = 1;
        }
    }
}

// Initial weights: hidden unit 0 of both layers carries feature 10 (the
// bilinear interpolation of the probe costs) to the output, so the untrained
// model already orders by the probe pass; the other weights are small values
// from a fixed integer hash (He-scaled, times 0.1 into the output), for the
// training to shape.
__global__ void k_init(float* P, float* Madam, float* Vadam, int* ready, int* step_count) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < SchedLayout::N; k += gridDim.x * blockDim.x) {
        unsigned h = (unsigned)k * 2654435761u ^ 0x9e3779b9u;
        h ^= h >> 15;
        h *= 2246822519u;
        h ^= h >> 13;
        const float u = (float)(h & 0xffffff) / 16777216.0f - 0.5f; // [-0.5, 0.5)
        float w = 0.0f;
        if (k < SchedLayout::B1) {
            const int o = k / kIn, in = k % kIn;
            w = o == 0 ? (in == 10 ? 1.0f : 0.0f) : u * 2.0f * sqrtf(6.0f / kIn);
        } else if (k >= SchedLayout::W2 && k < SchedLayout::B2) {
            const int o = (k - SchedLayout::W2) / kHid, in = (k - SchedLayout::W2) % kHid;
            w = o == 0 ? (in == 0 ? 1.0f : 0.0f) : u * 2.0f * sqrtf(6.0f / kHid);
        } else if (k >= SchedLayout::W3 && k < SchedLayout::B3) {
            w = k == SchedLayout::W3 ? 1.0f : 0.1f * u * 2.0f * sqrtf(3.0f / kHid);
        }
        P[k] = w;
        Madam[k] = 0.0f;
        Vadam[k] = 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *ready = 1;
        *step_count = 0;
    }
}

} // namespace

size_t sched_train_smem() { return sizeof(TrainSmem); }

cudaError_t sched_init(SchedState& s, cudaStream_t st) {
    // the training kernel's shared memory exceeds the default 48 KB
    cudaError_t e = cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
    if (e != cudaSuccess) return e;
    k_init<<<8, 256, 0, st>>>(s.params, s.adam_m, s.adam_v, s.ready, s.steps);
    return cudaGetLastError();
}

cudaError_t sched_probe_grid(const ViewDesc* probe, const ViewDesc* main, int nv, unsigned probe_total, cudaStream_t st) {
    if (probe_total == 0) return cudaSuccess;
    k_probe_grid<<<(probe_total + 255) / 256, 256, 0, st>>>(probe, main, nv, probe_total);
    return cudaGetLastError();
}

cudaError_t sched_order(SchedState& s, const ViewDesc* main, int nv, unsigned total, int nsm, uint64_t* out, cudaStream_t st) {
    const unsigned nw = (total + kWarpSpan - 1) / kWarpSpan, nb = (nw + 7) / 8;
    k_predict<<<nsm * 4, 128, 0, st>>>(main, nv, total, s.params, s.ready, s.bucket);
    k_bucket_count<<<nb, 256, 0, st>>>(total, s.bucket, s.hist);
    k_bucket_offsets<<<1, 32, 0, st>>>(nb * 8, s.hist);
    k_bucket_place<<<nb, 256, 0, st>>>(main, nv, total, s.ready, s.bucket, s.hist, out);
    return cudaGetLastError();
}

cudaError_t sched_train(SchedState& s, const ViewDesc* main, int nv, unsigned total, int steps, float lr, cudaStream_t st) {
    if (total == 0) return cudaSuccess;
    k_collect<<<(kSchedSamples + 255) / 256, 256, 0, st>>>(main, nv, total, s.X, s.T, kSchedSamples);
    const size_t smem = sizeof(TrainSmem);
    k_train<<<1, 256, smem, st>>>(s.params, s.adam_m, s.adam_v, s.ready, s.steps, s.X, s.T, kSchedSamples, steps, lr, nullptr, s.loss);
    return cudaGetLastError();
}

cudaError_t sched_gradient(SchedState& s, const __nv_bfloat16* X, const float* T, int n, float* grad_out, cudaStream_t st) {
    const size_t smem = sizeof(TrainSmem);
    k_train<<<1, 256, smem, st>>>(s.params, s.adam_m, s.adam_v, s.ready, s.steps, X, T, n, 1, 0.0f, grad_out, s.loss);
    return cudaGetLastError();
}

} // namespace mbx

// Learned work ordering for the batched passes.
//
// A BF16 multilayer perceptron (24 -> 64 -> 64 -> 1, ReLU) predicts the mean
// FP32-lane cost of each 16x16 tile of a batch's main-pass samples (log2 of 1 +
// lane steps + 4 per BLA skip, / 24) from the probe pass, which renders one
// sample per 8x8 cell (four per tile): the cells' costs, their BLA-skip
// statistics (fraction of the iterations that BLA skipped, mean skip length),
// interior flags, the neighbouring tiles' costs and a few view features.
// Before the main FP32 pass the samples are reordered: views by decreasing
// predicted cost, each view's samples by their tile's predicted cost,
// decreasing (half-octave buckets; within a bucket, pieces of rows): expensive
// tiles start first instead of trailing the launch, tiles of similar cost fill
// the same warps, and the lanes work on one or two views' tables at a time. After the pass (mode 1) the
// model trains on the batch's tiles with their measured mean costs as targets
// (Adam; each step's minibatch spread over several blocks). The order changes
// no output: every sample's result depends only on its own coordinates.
//
// Tensor cores: every product (inference, and the training step's forward,
// input-gradient and weight-gradient products) is a tcgen05.mma of kind f16:
// BF16 operands in shared memory (no-swizzle K-major layout, described by
// shared-memory matrix descriptors), FP32 accumulators in tensor memory, the
// instructions issued by one thread, completion signalled through
// tcgen05.commit on an mbarrier (bounded waits), results read back with
// tcgen05.ld for the epilogues on the CUDA cores.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "order_model.h"

namespace mbx {
namespace {

constexpr int kIn = 24, kInPad = 32, kHid = 64, kRows = 128;
constexpr int kBuckets = 32;         // half-octaves of predicted cost (one per lane)
constexpr int kTile = 16;            // samples per tile side
constexpr int kTrainBlocks = 16;     // blocks per training step (minibatch 16 x 128 tiles)

// ---- tcgen05 / mbarrier helpers ----------------------------------------------
__device__ __forceinline__ uint32_t saddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Element offset of (row r, column k) in a K-major operand tile of K columns:
// 8x8 core matrices (8 rows of 16 bytes, 128 contiguous bytes), K-adjacent core
// matrices 128 bytes apart (leading byte offset), 8-row groups K * 16 bytes
// apart (stride byte offset).
__host__ __device__ constexpr int kidx(int r, int k, int K) { return (r >> 3) * (K * 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7); }

// Shared-memory matrix descriptor, no swizzle: start address >> 4 (bits 0-13),
// leading byte offset >> 4 (16-29), stride byte offset >> 4 (32-45), the
// descriptor version 1 (bits 46-47), base offset 0, layout 0 (no swizzle).
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}
// Instruction descriptor of kind f16: FP32 accumulator (bits 4-5 = 1), BF16 A
// and B (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 (bits
// 17-22), M >> 4 (bits 24-28).
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[128][N] (+)= A[128][K] B[N][K]^T: K / 16 instructions (one thread).
__device__ __forceinline__ void mma_rows128(uint32_t d_tmem, const __nv_bfloat16* A, const __nv_bfloat16* B, int K, int N, bool accumulate) {
    const uint32_t id = idesc_bf16(kRows, N), a0 = saddr(A), b0 = saddr(B), sbo = (uint32_t)K * 16u;
    for (int kk = 0; kk < K / 16; ++kk) {
        const uint64_t a = sdesc(a0 + kk * 256u, sbo), b = sdesc(b0 + kk * 256u, sbo);
        const uint32_t acc = (accumulate || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
            "l"(a), "l"(b), "r"(id), "r"(acc)
            : "memory");
    }
}
__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(mbar)) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor cores' reads
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* m) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(m)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Wait for the completion of the phase with parity ph; false when the
// iteration limit ran out (the caller records an error).
__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t ph) {
    const uint32_t a = saddr(m);
    for (unsigned it = 0; it < (1u << 22); ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(ph)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Tensor memory: allocated by one warp (columns a power of two >= 32); this
// block allocates once, so it gives up its permit right away.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// 32 consecutive FP32 columns of this thread's tensor-memory lane (the warp's
// 32-lane quarter); the wait is in the same statement, so the registers are
// complete when it returns.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),
          "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
          "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr)
        : "memory");
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
// this warp's lane quarter of tensor memory, column c
__device__ __forceinline__ uint32_t tlane(uint32_t base, int c) { return base + ((uint32_t)((threadIdx.x >> 5) & 3) * 32u << 16) + (uint32_t)c; }

__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ---- features -----------------------------------------------------------------
__device__ __forceinline__ int find_view(const ViewDesc* views, int nv, unsigned g) {
    int lo = 0, hi = nv - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (views[mid].base <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ int find_view_tile(const ViewDesc* views, int nv, unsigned t) {
    int lo = 0, hi = nv - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (views[mid].tile_base <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Feature vector of batch tile t (24 values, zero padded to 32). The probe
// cell record (ProbeCell): x log2(1 + cost) / 24, y interior, z fraction of the
// iterations BLA skipped, w log2(1 + mean skip length) / 24.
__device__ void tile_features(const ViewDesc* views, int nv, unsigned t, float* f) {
    const int v = find_view_tile(views, nv, t);
    const ViewDesc& vd = views[v];
    const int local = (int)(t - vd.tile_base), ty = local / vd.tw, tx = local % vd.tw;
    const int gw = vd.pgw, gh = vd.pgh;
    auto C = [&](int a, int b) -> float4 {
        a = max(0, min(gh - 1, a));
        b = max(0, min(gw - 1, b));
        return vd.pgrid[a * gw + b];
    };
    const int a = 2 * ty, b = 2 * tx;
    const float4 c00 = C(a, b), c01 = C(a, b + 1), c10 = C(a + 1, b), c11 = C(a + 1, b + 1);
    f[0] = c00.x;
    f[1] = c01.x;
    f[2] = c10.x;
    f[3] = c11.x;
    f[4] = c00.z;
    f[5] = c01.z;
    f[6] = c10.z;
    f[7] = c11.z;
    f[8] = c00.w;
    f[9] = c01.w;
    f[10] = c10.w;
    f[11] = c11.w;
    f[12] = 0.25f * (c00.y + c01.y + c10.y + c11.y);
    f[13] = fminf(fminf(c00.x, c01.x), fminf(c10.x, c11.x));
    f[14] = fmaxf(fmaxf(c00.x, c01.x), fmaxf(c10.x, c11.x));
    f[15] = 0.25f * (c00.x + c01.x + c10.x + c11.x);
    // neighbouring tiles' mean cell costs: above, below, left, right
    f[16] = 0.5f * (C(a - 1, b).x + C(a - 1, b + 1).x);
    f[17] = 0.5f * (C(a + 2, b).x + C(a + 2, b + 1).x);
    f[18] = 0.5f * (C(a, b - 1).x + C(a + 1, b - 1).x);
    f[19] = 0.5f * (C(a, b + 2).x + C(a + 1, b + 2).x);
    f[20] = log2f((float)vd.p.g.mxit) * (1.0f / 24.0f);
    const int hh = min(kTile, vd.p.g.H - ty * kTile), ww = min(kTile, vd.p.g.W - tx * kTile);
    f[21] = (float)(hh * ww) * (1.0f / (kTile * kTile));
    f[22] = vd.p.per > 0 ? 1.0f : 0.0f;
    f[23] = 1.0f;
    for (int k = kIn; k < kInPad; ++k) f[k] = 0.0f;
}

// ---- probe cells ----------------------------------------------------------------
__global__ void k_probe_grid(const ViewDesc* probe, const ViewDesc* main, int nv, unsigned total) {
    const unsigned g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= total) return;
    const int v = find_view(probe, nv, g);
    const ViewDesc& pd = probe[v];
    int arr[4];
    entry_coords(pd.f.px, (int)(g - pd.base), arr);
    const int oidx = arr[0] * pd.p.g.W + arr[1];
    const float c = pd.f.out.cost ? (float)pd.f.out.cost[oidx] : 0.0f;
    const float nb = pd.f.out.bla ? (float)pd.f.out.bla[oidx] : 0.0f;
    const float it = pd.f.out.iter[oidx];
    const bool interior = it == -2.0f;
    // iterations the sample ran (maxiter when interior) and how many BLA skipped
    const float n_it = interior ? (float)pd.p.g.mxit : fmaxf(it, 1.0f);
    const float steps = fmaxf(c - 4.0f * nb, 0.0f);
    const float skipped = fmaxf(n_it - steps, 0.0f);
    const float frac = fminf(skipped / n_it, 1.0f);
    const float mean_skip = nb > 0.0f ? skipped / nb : 0.0f;
    main[v].pgrid[(arr[0] >> 3) * main[v].pgw + (arr[1] >> 3)] =
        make_float4(log2f(1.0f + c) * (1.0f / 24.0f), interior ? 1.0f : 0.0f, frac, log2f(1.0f + mean_skip) * (1.0f / 24.0f));
}

// ---- prediction -------------------------------------------------------------------
// Shared memory of a 128-thread block: the weights as the B operands, one
// 128-tile block of features as layer 1's A operand, layer 1's activations as
// layer 2's A operand. Operand arrays first (sizes multiples of 128 bytes).
struct __align__(1024) PredSmem {
    __nv_bfloat16 w1[kHid * kInPad]; // [64][32]
    __nv_bfloat16 w2[kHid * kHid];   // [64][64]
    __nv_bfloat16 x[kRows * kInPad]; // [128][32]
    __nv_bfloat16 h1[kRows * kHid];  // [128][64]
    float b1[kHid], b2[kHid], w3[kHid];
    float b3;
    uint64_t mbar;
    uint32_t tmem;
};

__device__ void stage_weights(__nv_bfloat16* w1, __nv_bfloat16* w2, __nv_bfloat16* w2t, float* b1, float* b2, float* w3, float* b3, const float* P) {
    for (int k = threadIdx.x; k < kHid * kInPad; k += blockDim.x) {
        const int o = k / kInPad, in = k % kInPad;
        w1[kidx(o, in, kInPad)] = __float2bfloat16_rn(in < kIn ? P[SchedLayout::W1 + o * kIn + in] : 0.0f);
    }
    for (int k = threadIdx.x; k < kHid * kHid; k += blockDim.x) {
        const int o = k / kHid, in = k % kHid;
        const __nv_bfloat16 w = __float2bfloat16_rn(P[SchedLayout::W2 + k]);
        w2[kidx(o, in, kHid)] = w;         // B of layer 2: [n = out][k = in]
        if (w2t) w2t[kidx(in, o, kHid)] = w; // B of the input gradient: [n = in][k = out]
    }
    for (int k = threadIdx.x; k < kHid; k += blockDim.x) {
        b1[k] = P[SchedLayout::B1 + k];
        b2[k] = P[SchedLayout::B2 + k];
        w3[k] = P[SchedLayout::W3 + k];
    }
    if (threadIdx.x == 0) *b3 = P[SchedLayout::B3];
}

// One 128-thread block per 128 tiles at a time (thread t: tile row t). Writes
// the tile's bucket of its predicted cost in half-octaves, descending (bucket
// 0 the most expensive).
__global__ void __launch_bounds__(128) k_predict(const ViewDesc* views, int nv, unsigned ntiles, const float* P, const int* ready, uint8_t* tile_bucket,
                                                 float* view_cost, int* err) {
    __shared__ PredSmem s;
    const int t = threadIdx.x, warp = t >> 5;
    if (*ready == 0) return; // natural order: the placement ignores the buckets
    stage_weights(s.w1, s.w2, nullptr, s.b1, s.b2, s.w3, &s.b3, P);
    if (warp == 0) tmem_alloc(&s.tmem, 128);
    if (t == 0) mbar_init(&s.mbar);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = s.tmem;
    uint32_t phase = 0, last = 0; // parity of the next and of the last committed phase
    bool ok = true;
    for (unsigned r0 = blockIdx.x * kRows; r0 < ntiles && ok; r0 += gridDim.x * kRows) {
        const unsigned r = r0 + t;
        float f[kInPad];
        if (r < ntiles) tile_features(views, nv, r, f);
        else
            for (int k = 0; k < kInPad; ++k) f[k] = 0.0f;
        for (int k = 0; k < kInPad; ++k) s.x[kidx(t, k, kInPad)] = __float2bfloat16_rn(f[k]);
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            mma_rows128(tm, s.x, s.w1, kInPad, kHid, false);
            mma_commit(&s.mbar);
        }
        ok = __syncthreads_and(mbar_wait(&s.mbar, phase) ? 1 : 0) != 0; // one verdict for the block
        last = phase;
        phase ^= 1u;
        tc_fence_after();
        for (int half = 0; half < 2 && ok; ++half) {
            float a[32];
            tmem_ld32(tlane(tm, 32 * half), a);
            for (int j = 0; j < 32; ++j) s.h1[kidx(t, 32 * half + j, kHid)] = __float2bfloat16_rn(fmaxf(a[j] + s.b1[32 * half + j], 0.0f));
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0 && ok) {
            tc_fence_after();
            mma_rows128(tm + kHid, s.h1, s.w2, kHid, kHid, false);
            mma_commit(&s.mbar);
        }
        if (ok) {
            ok = __syncthreads_and(mbar_wait(&s.mbar, phase) ? 1 : 0) != 0;
            last = phase;
            phase ^= 1u;
        }
        tc_fence_after();
        float y = s.b3;
        for (int half = 0; half < 2 && ok; ++half) {
            float a[32];
            tmem_ld32(tlane(tm, kHid + 32 * half), a);
            for (int j = 0; j < 32; ++j) y += bf(fmaxf(a[j] + s.b2[32 * half + j], 0.0f)) * s.w3[32 * half + j];
        }
        if (ok && r < ntiles) {
            // prediction in log2(1 + cost) / 24 -> half-octave buckets
            const int b = max(0, min(kBuckets - 1, (int)(y * 24.0f * 2.0f)));
            tile_bucket[r] = (uint8_t)(kBuckets - 1 - b);
            // the view's predicted cost: mean cost x the tile's samples
            atomicAdd(&view_cost[find_view_tile(views, nv, r)], exp2f(fminf(24.0f * y, 60.0f)) * f[21] * (float)(kTile * kTile));
        }
        tc_fence_before();
        __syncthreads();
    }
    if (!ok) {
        if (t == 0) atomicExch(err, 1);
        (void)mbar_wait(&s.mbar, last); // the instructions that timed out: one more bounded wait
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tm, 128);
    }
}

// ---- placement ------------------------------------------------------------------
// The order: views by decreasing predicted cost (the sum over their tiles),
// each view's samples by their tile's bucket (decreasing cost), and within a
// (view, bucket) bin 32-sample pieces of rows. Views stay contiguous, so the
// lanes read one or two views' orbit and BLA tables at a time (a batch's
// tables together can exceed L2), and the pieces keep warps on neighbouring
// samples.
constexpr int kMaxBins = kBatchMaxViews * kBuckets;

// the views' ranks by predicted cost (ties by index); one block
__global__ void k_view_rank(int nv, const int* ready, const float* view_cost, int* vrank) {
    const int v = threadIdx.x;
    if (*ready == 0 || v >= nv) return;
    const float c = view_cost[v];
    int r = 0;
    for (int u = 0; u < nv; ++u) {
        const float d = view_cost[u];
        r += (d > c || (d == c && u < v)) ? 1 : 0;
    }
    vrank[v] = r;
}

// every main-pass sample's bin (its view's rank, its tile's bucket) and the
// bins' counts (one atomic per bin and warp)
__global__ void k_bins(const ViewDesc* views, int nv, unsigned total, const int* ready, const uint8_t* tile_bucket, const int* vrank, uint16_t* bin,
                       unsigned* count) {
    if (*ready == 0) return;
    const unsigned g = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31;
    int b = -1;
    if (g < total) {
        const int v = find_view(views, nv, g);
        int arr[4];
        entry_coords(views[v].f.px, (int)(g - views[v].base), arr);
        b = vrank[v] * kBuckets + tile_bucket[views[v].tile_base + (arr[0] / kTile) * views[v].tw + arr[1] / kTile];
        bin[g] = (uint16_t)b;
    }
    const unsigned same = __match_any_sync(0xffffffffu, b);
    if (b >= 0 && (int)lane == __ffs(same) - 1) atomicAdd(&count[b], (unsigned)__popc(same));
}

// exclusive scan of the bin counts into cursors (one block of 1024, 8 bins each)
__global__ void __launch_bounds__(1024) k_bin_scan(const int* ready, unsigned* count) {
    if (*ready == 0) return;
    __shared__ unsigned part[1024];
    const int t = threadIdx.x;
    unsigned c[kMaxBins / 1024], run = 0;
    for (int k = 0; k < kMaxBins / 1024; ++k) {
        c[k] = count[t * (kMaxBins / 1024) + k];
        run += c[k];
    }
    part[t] = run;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) { // inclusive scan of the threads' sums
        const unsigned add = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    unsigned base = part[t] - run;
    for (int k = 0; k < kMaxBins / 1024; ++k) {
        count[t * (kMaxBins / 1024) + k] = base;
        base += c[k];
    }
}

// the order: batch-wide sample indices (the natural order while the model is
// not ready)
__global__ void k_place(unsigned total, const int* ready, const uint16_t* bin, unsigned* cursor, uint64_t* out) {
    const unsigned g = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31;
    const uint64_t key = g;
    if (*ready == 0) {
        if (g < total) out[g] = key;
        return;
    }
    const int b = g < total ? (int)bin[g] : -1;
    const unsigned same = __match_any_sync(0xffffffffu, b);
    const int leader = __ffs(same) - 1;
    unsigned base = 0;
    if (b >= 0 && (int)lane == leader) base = atomicAdd(&cursor[b], (unsigned)__popc(same));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (b >= 0) out[base + __popc(same & ((1u << lane) - 1u))] = key;
}

// ---- training -----------------------------------------------------------------------
// Training set: n tiles of the batch at a uniform stride; features in bf16,
// target log2(1 + the tile's mean FP32-lane cost) / 24.
__global__ void k_collect(const ViewDesc* views, int nv, unsigned ntiles, __nv_bfloat16* X, float* T, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned t = (unsigned)(((unsigned long long)k * ntiles) / (unsigned)n);
    float f[kInPad];
    tile_features(views, nv, t, f);
    for (int q = 0; q < kInPad; ++q) X[(size_t)k * kInPad + q] = __float2bfloat16_rn(f[q]);
    const int v = find_view_tile(views, nv, t);
    const ViewDesc& vd = views[v];
    const int local = (int)(t - vd.tile_base), ty = local / vd.tw, tx = local % vd.tw;
    const int W = vd.p.g.W, H = vd.p.g.H;
    float sum = 0.0f;
    int cnt = 0;
    for (int i = ty * kTile; i < min(H, ty * kTile + kTile); ++i)
        for (int j = tx * kTile; j < min(W, tx * kTile + kTile); ++j) {
            sum += (float)vd.f.out.cost[i * W + j];
            ++cnt;
        }
    T[k] = log2f(1.0f + sum / (float)max(cnt, 1)) * (1.0f / 24.0f);
}

// Shared memory of a training block (128 threads, 128 rows of the minibatch).
// Operands, all K-major: the transposed copies are the weight-gradient
// products' operands (K = the minibatch rows); dz2t / dz1t have 128 rows for
// the M = 128 instruction shape, rows 64..127 zero.
struct __align__(1024) TrainSmem {
    __nv_bfloat16 dz2t[kRows * kRows]; // [out (64 used)][b]
    __nv_bfloat16 dz1t[kRows * kRows]; // [out (64 used)][b]
    __nv_bfloat16 h1[kRows * kHid];    // [b][in]      A of layer 2
    __nv_bfloat16 h1t[kHid * kRows];   // [in][b]      B of dW2
    __nv_bfloat16 dz2[kRows * kHid];   // [b][out]     A of dh1
    __nv_bfloat16 w2[kHid * kHid];     // [out][in]    B of layer 2
    __nv_bfloat16 w2t[kHid * kHid];    // [in][out]    B of dh1
    __nv_bfloat16 x[kRows * kInPad];   // [b][in]      A of layer 1
    __nv_bfloat16 xt[kInPad * kRows];  // [in][b]      B of dW1
    __nv_bfloat16 w1[kHid * kInPad];   // [out][in]    B of layer 1
    float b1[kHid], b2[kHid], w3[kHid];
    float b3;
    float red[4][3 * kHid + 2]; // per-warp partial sums: db1, db2, dw3, db3, loss
    uint64_t mbar;
    uint32_t tmem;
};
// tensor-memory columns of the accumulators
constexpr uint32_t kColD1 = 0, kColD2 = 64, kColDH1 = 128, kColDW2 = 192, kColDW1 = 256, kTrainCols = 512;

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Gradients of mean((y - t)^2) / 2 over a minibatch of `rows` rows starting at
// row `first` (mod n) of the training set, added into grad (zeroed by the
// caller); block b takes rows first + 128 b ... The loss adds into *loss.
__global__ void __launch_bounds__(128) k_grad(const float* P, const __nv_bfloat16* X, const float* T, int n, int first, int rows, float* grad, float* loss,
                                              int* err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>(smem_raw);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    stage_weights(s.w1, s.w2, s.w2t, s.b1, s.b2, s.w3, &s.b3, P);
    for (int k = t; k < kRows * kRows; k += blockDim.x) {
        s.dz2t[k] = __float2bfloat16_rn(0.0f);
        s.dz1t[k] = __float2bfloat16_rn(0.0f);
    }
    const int row_in_batch = blockIdx.x * kRows + t;
    const bool valid = row_in_batch < rows;
    const int gr = (int)(((long long)first + row_in_batch) % n);
    float tgt = 0.0f;
    for (int k = 0; k < kInPad; ++k) {
        const __nv_bfloat16 v = valid ? X[(size_t)gr * kInPad + k] : __float2bfloat16_rn(0.0f);
        s.x[kidx(t, k, kInPad)] = v;
        s.xt[kidx(k, t, kRows)] = v;
    }
    if (valid) tgt = T[gr];
    if (warp == 0) tmem_alloc(&s.tmem, kTrainCols);
    if (t == 0) mbar_init(&s.mbar);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = s.tmem;
    uint32_t phase = 0, last = 0; // parity of the next and of the last committed phase
    bool ok = true;
    auto issue = [&](auto&& body) {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (t == 0 && ok) {
            tc_fence_after();
            body();
            mma_commit(&s.mbar);
        }
        // one verdict for the block: the tensor-memory loads are warp-collective
        if (ok) {
            ok = __syncthreads_and(mbar_wait(&s.mbar, phase) ? 1 : 0) != 0;
            last = phase;
            phase ^= 1u;
        }
        tc_fence_after();
    };
    // layer 1
    issue([&] { mma_rows128(tm + kColD1, s.x, s.w1, kInPad, kHid, false); });
    uint32_t m1[2] = {0u, 0u}; // h1 > 0 per column
    for (int half = 0; half < 2 && ok; ++half) {
        float a[32];
        tmem_ld32(tlane(tm, kColD1 + 32 * half), a);
        for (int j = 0; j < 32; ++j) {
            const int c = 32 * half + j;
            const __nv_bfloat16 h = __float2bfloat16_rn(fmaxf(a[j] + s.b1[c], 0.0f));
            s.h1[kidx(t, c, kHid)] = h;
            s.h1t[kidx(c, t, kRows)] = h;
            if (__bfloat162float(h) > 0.0f) m1[half] |= 1u << j;
        }
    }
    // layer 2, output, and the output-side gradients
    issue([&] { mma_rows128(tm + kColD2, s.h1, s.w2, kHid, kHid, false); });
    float h2[kHid];
    float y = s.b3;
    for (int half = 0; half < 2 && ok; ++half) {
        float a[32];
        tmem_ld32(tlane(tm, kColD2 + 32 * half), a);
        for (int j = 0; j < 32; ++j) {
            h2[32 * half + j] = bf(fmaxf(a[j] + s.b2[32 * half + j], 0.0f));
            y += h2[32 * half + j] * s.w3[32 * half + j];
        }
    }
    const float e = valid ? y - tgt : 0.0f;
    const float dy = e / (float)rows;
    {
        const float l = warp_sum(0.5f * e * e / (float)rows), d3 = warp_sum(dy);
        if (lane == 0) {
            s.red[warp][3 * kHid] = d3;
            s.red[warp][3 * kHid + 1] = l;
        }
    }
    for (int c = 0; c < kHid; ++c) {
        const __nv_bfloat16 d = __float2bfloat16_rn(h2[c] > 0.0f ? dy * s.w3[c] : 0.0f);
        s.dz2[kidx(t, c, kHid)] = d;
        s.dz2t[kidx(c, t, kRows)] = d;
        const float sb = warp_sum(__bfloat162float(d)), sw = warp_sum(dy * h2[c]);
        if (lane == 0) {
            s.red[warp][kHid + c] = sb;
            s.red[warp][2 * kHid + c] = sw;
        }
    }
    // dh1 = dz2 W2 and dW2 = dz2^T h1
    issue([&] {
        mma_rows128(tm + kColDH1, s.dz2, s.w2t, kHid, kHid, false);
        mma_rows128(tm + kColDW2, s.dz2t, s.h1t, kRows, kHid, false);
    });
    for (int half = 0; half < 2 && ok; ++half) {
        float a[32];
        tmem_ld32(tlane(tm, kColDH1 + 32 * half), a);
        for (int j = 0; j < 32; ++j) {
            const int c = 32 * half + j;
            const __nv_bfloat16 d = __float2bfloat16_rn(((m1[half] >> j) & 1u) ? a[j] : 0.0f);
            s.dz1t[kidx(c, t, kRows)] = d;
            const float sb = warp_sum(__bfloat162float(d));
            if (lane == 0) s.red[warp][c] = sb;
        }
    }
    // dW2 rows (out) live in tensor-memory lanes 0..63: warps 0 and 1
    for (int half = 0; half < 2 && ok; ++half) {
        float a[32];
        tmem_ld32(tlane(tm, kColDW2 + 32 * half), a);
        if (warp < 2)
            for (int j = 0; j < 32; ++j) atomicAdd(&grad[SchedLayout::W2 + t * kHid + 32 * half + j], a[j]);
    }
    // dW1 = dz1^T x
    issue([&] { mma_rows128(tm + kColDW1, s.dz1t, s.xt, kRows, kInPad, false); });
    if (ok) {
        float a[32];
        tmem_ld32(tlane(tm, kColDW1), a);
        if (warp < 2)
            for (int j = 0; j < kIn; ++j) atomicAdd(&grad[SchedLayout::W1 + t * kIn + j], a[j]);
    }
    __syncthreads();
    for (int c = t; c < kHid; c += blockDim.x) {
        float g1 = 0.0f, g2 = 0.0f, g3 = 0.0f;
        for (int w = 0; w < 4; ++w) {
            g1 += s.red[w][c];
            g2 += s.red[w][kHid + c];
            g3 += s.red[w][2 * kHid + c];
        }
        atomicAdd(&grad[SchedLayout::B1 + c], g1);
        atomicAdd(&grad[SchedLayout::B2 + c], g2);
        atomicAdd(&grad[SchedLayout::W3 + c], g3);
    }
    if (t == 0) {
        float g = 0.0f, l = 0.0f;
        for (int w = 0; w < 4; ++w) {
            g += s.red[w][3 * kHid];
            l += s.red[w][3 * kHid + 1];
        }
        atomicAdd(&grad[SchedLayout::B3], g);
        if (loss) atomicAdd(loss, l);
    }
    if (!ok) {
        if (t == 0) atomicExch(err, 1);
        (void)mbar_wait(&s.mbar, last); // the instructions that timed out: one more bounded wait
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tm, kTrainCols);
    }
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) on the summed gradients: step k of
// a training call (the call's first step follows the *step_count taken before).
__global__ void k_adam(float* P, float* M, float* V, const float* grad, const int* step_count, int k, float lr) {
    const int it = *step_count + k + 1;
    const float c1 = 1.0f - powf(0.9f, (float)it), c2 = 1.0f - powf(0.999f, (float)it);
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= SchedLayout::N) return;
    const float g = grad[j];
    const float m = 0.9f * M[j] + 0.1f * g, v = 0.999f * V[j] + 0.001f * g * g;
    M[j] = m;
    V[j] = v;
    P[j] -= lr * (m / c1) / (sqrtf(v / c2) + 1e-8f);
}
// after a training call's steps
__global__ void k_adam_done(int* step_count, int* ready, int steps) {
    *step_count += steps;
    *ready = 1;
}

// Initial weights: hidden unit 0 of both layers carries feature 15 (the mean
// of the tile's four probe-cell costs) to the output, so the untrained model
// orders tiles by their probe costs; the other weights are small values from a
// fixed integer hash (He-scaled, times 0.1 into the output), for the training
// to shape.
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
            w = o == 0 ? (in == 15 ? 1.0f : 0.0f) : u * 2.0f * sqrtf(6.0f / kIn);
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
    cudaError_t e = cudaFuncSetAttribute(k_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
    if (e != cudaSuccess) return e;
    k_init<<<8, 256, 0, st>>>(s.params, s.adam_m, s.adam_v, s.ready, s.steps);
    e = cudaMemsetAsync(s.err, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t sched_probe_grid(const ViewDesc* probe, const ViewDesc* main, int nv, unsigned probe_total, cudaStream_t st) {
    if (probe_total == 0) return cudaSuccess;
    k_probe_grid<<<(probe_total + 255) / 256, 256, 0, st>>>(probe, main, nv, probe_total);
    return cudaGetLastError();
}

cudaError_t sched_order(SchedState& s, const ViewDesc* main, int nv, unsigned total, unsigned ntiles, int nsm, uint64_t* out, cudaStream_t st) {
    const unsigned pb = std::max(1u, std::min((ntiles + kRows - 1) / kRows, (unsigned)nsm * 2u));
    unsigned* count = s.hist;
    float* view_cost = reinterpret_cast<float*>(s.hist + kMaxBins);
    int* vrank = reinterpret_cast<int*>(s.hist + kMaxBins + kBatchMaxViews);
    cudaMemsetAsync(s.hist, 0, sizeof(unsigned) * (kMaxBins + kBatchMaxViews), st);
    k_predict<<<pb, kRows, 0, st>>>(main, nv, ntiles, s.params, s.ready, s.tile_bucket, view_cost, s.err);
    k_view_rank<<<1, kBatchMaxViews, 0, st>>>(nv, s.ready, view_cost, vrank);
    k_bins<<<(total + 255) / 256, 256, 0, st>>>(main, nv, total, s.ready, s.tile_bucket, vrank, s.bucket, count);
    k_bin_scan<<<1, 1024, 0, st>>>(s.ready, count);
    k_place<<<(total + 255) / 256, 256, 0, st>>>(total, s.ready, s.bucket, count, out);
    return cudaGetLastError();
}

size_t sched_scratch_words() { return (size_t)kMaxBins + 2 * kBatchMaxViews; }

int sched_train_rows(unsigned ntiles) { return (int)std::min<unsigned>(ntiles, (unsigned)kSchedTiles); }

cudaError_t sched_train(SchedState& s, const ViewDesc* main, int nv, unsigned ntiles, int steps, float lr, cudaStream_t st) {
    const int n = sched_train_rows(ntiles);
    if (n == 0) return cudaSuccess;
    k_collect<<<(n + 255) / 256, 256, 0, st>>>(main, nv, ntiles, s.X, s.T, n);
    const int rows = kTrainBlocks * kRows;
    cudaMemsetAsync(s.loss, 0, sizeof(float), st);
    for (int k = 0; k < steps; ++k) {
        cudaMemsetAsync(s.grad, 0, sizeof(float) * SchedLayout::N, st);
        k_grad<<<kTrainBlocks, kRows, sizeof(TrainSmem), st>>>(s.params, s.X, s.T, n, (int)(((long long)k * rows) % n), rows, s.grad,
                                                              k + 1 == steps ? s.loss : nullptr, s.err);
        k_adam<<<(SchedLayout::N + 255) / 256, 256, 0, st>>>(s.params, s.adam_m, s.adam_v, s.grad, s.steps, k, lr);
    }
    k_adam_done<<<1, 1, 0, st>>>(s.steps, s.ready, steps);
    return cudaGetLastError();
}

cudaError_t sched_gradient(SchedState& s, const __nv_bfloat16* X, const float* T, int n, float* grad_out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(grad_out, 0, sizeof(float) * SchedLayout::N, st);
    if (e != cudaSuccess) return e;
    cudaMemsetAsync(s.loss, 0, sizeof(float), st);
    k_grad<<<(n + kRows - 1) / kRows, kRows, sizeof(TrainSmem), st>>>(s.params, X, T, n, 0, n, grad_out, s.loss, s.err);
    return cudaGetLastError();
}

int sched_train_launches(int steps) { return 2 + 2 * steps; }

} // namespace mbx

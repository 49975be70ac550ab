// Mixed-precision floatexp pass. The bulk delta iteration runs in FP32 on a
// rescaled delta dz = S * w, with S an FP32-mantissa floatexp (float m, int e)
// and w an O(1) float2; the reference orbit is read as float2 from shared
// memory (staged once per block by a TMA bulk copy) or from L1/L2 when it does
// not fit. On GB300 one FP64 instruction costs as much issue time as ~60 FP32
// ones, so FP64 (and FP64-mantissa floatexp) is used only on rare events:
//   * BLA skips: coefficients and validity radii come from the FP64 table;
//     candidates are screened on integer exponents, decided and applied in FP64;
//   * rebasing near |Z + dz| ~ |dz|: screened in FP32, decided in FP64-floatexp;
//   * escape: screened in FP32 with a relative margin, decided and the smooth
//     value computed from an FP64 reconstruction of z;
//   * interior detection: FP32 screen, FP64 at close returns and saves;
//   * steps where the orbit is below FP32's range (exact floatexp step).
// Semantics follow the reference's rescaled loop (mp.cpp:3287-3618); results
// are validated against the arbitrary-precision oracle, not bit-compared.
#include <cuda_runtime.h>

#include "engine.h"
#include "mixed_lane.cuh"

namespace mbx {

namespace {

constexpr double kLn2m = 0x1.62e42fefa39efp-1;

__device__ __forceinline__ bool mcancelled(const DeviceFrame& f) { return f.cancel && *f.cancel; }

template <class T>
__global__ void k_bla_to_lane(const double* r2, const double4* ab, BlaEntry<T>* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = bla_entry<T>(r2[i], ab[i]);
}

// The FP32 lane's per-position radius maxima (BlaMaxR2): the levels lane_bla
// tries at s, startp down to minlevel, as it orders them.
__global__ void k_bla_maxr2(const BlaEntry<float>* t, BlaView b, BlaMaxR2* out, int nq) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int s = (q << b.minlevel) + 1;
    const int maxp = b.nlev - 1;
    int startp = (s == 1) ? maxp : ffs32(s - 1) - 1;
    if (startp > maxp) startp = maxp;
    BlaMaxR2 best{0.0f, 0};
    for (int p = startp; p >= b.minlevel; --p) {
        const int i = (s - 1) >> p;
        if (i >= b.size[p]) continue;
        const BlaEntry<float> e = t[b.off[p] + i];
        if (e.r2m == 0.0f) continue;
        if (best.m == 0.0f || e.r2e > best.e || (e.r2e == best.e && e.r2m > best.m)) best = BlaMaxR2{e.r2m, e.r2e};
    }
    out[q] = best;
}

__device__ __forceinline__ float tlog2(float x) { return log2f(x); }
__device__ __forceinline__ double tlog2(double x) { return log2(x); }
__device__ __forceinline__ float tlog2(df32 x) { return log2f(x.hi + x.lo); }

// Results of a lane (pixelRescaled's outputs, mp.cpp:3498-3528): the smooth
// value N - log2(log2|z|) in the lane type; under DE colourings the distance
// |z| log|z|^2 / (dx |J|) in FP64 floatexp (into the values under EDE, into the
// normal buffer under the DE overlay) or the normal-map angle arg z - arg J;
// EDE takes precedence, then the normal map. The normal buffer holds 0 where
// the exact form writes no angle or distance.
template <bool DE, class T>
__device__ __forceinline__ void lane_write_escape(const Outputs& o, const FrameGeom& g, const MixedParams& p, const Lane<T>& L, T zrad) {
    float v = (float)((T)L.iter - tlog2(T(0.5) * tlog2(zrad)));
    if (DE && g.deriv) {
        float nrm = 0.0f;
        if (g.ede || (g.deovl && !g.normal)) {
            const double zr2 = (double)zrad;
            const double num = sqrt(zr2) * log(zr2);
            const float de = (float)fe_to_double(fe_div(fe_from(num), fe_mul(p.dxfe, lane_j_mag(L))));
            if (g.ede) v = de;
            else nrm = de;
        } else if (g.normal) {
            nrm = (float)(atan2((double)L.ezi, (double)L.ezr) - atan2((double)L.ji, (double)L.jr));
        }
        if ((g.deovl || g.normal) && o.normal) o.normal[L.oidx] = nrm;
    }
    o.iter[L.oidx] = v;
    if (o.escN) o.escN[L.oidx] = L.iter;
}
template <bool DE, class T>
__device__ __forceinline__ void lane_write_interior(const Outputs& o, const FrameGeom& g, const Lane<T>& L) {
    o.iter[L.oidx] = -2.0f;
    if (DE && g.deriv && (g.deovl || g.normal) && o.normal) o.normal[L.oidx] = 0.0f;
    if (o.escN) o.escN[L.oidx] = -1;
}

// Bounded wait on phase 0 of an mbarrier: true once the phase completed, false
// after `limit` polls.
__device__ bool mbar_wait_bounded(unsigned mb, int limit) {
    unsigned done = 0;
    for (int spin = 0; spin < limit && !done; ++spin) {
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mb)
            : "memory");
    }
    return done != 0;
}

// Stage the FP32 orbit into shared memory: bulk TMA copies (cp.async.bulk,
// global -> shared) completing on one mbarrier; the wait is bounded.
__device__ bool stage_orbit(float2* smem, const float2* g, int entries, unsigned long long* mbar) {
    const unsigned bytes = ((unsigned)entries * 8u + 15u) & ~15u;
    const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
        const unsigned chunk = 1u << 15;
        for (unsigned off = 0; off < bytes; off += chunk) {
            unsigned n = bytes - off < chunk ? bytes - off : chunk;
            unsigned dst = (unsigned)__cvta_generic_to_shared((char*)smem + off);
            const char* src = (const char*)g + off;
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst), "l"(src), "r"(n), "r"(mb) : "memory");
        }
    }
    __syncthreads();
    return mbar_wait_bounded(mb, 1 << 22);
}

// Iterations a lane takes per lane_run call between the warp's refill points
// (MixedParams::lane_budget, a tuning axis: the span of the orbit a warp walks
// between refills). Longer calls amortise the warp's reconvergence and refill
// (measured on the 1080p 1e-300 frame: FP32 passes 6.0 ms at 32, 5.4 at 128,
// 4.6 at 256, 4.7 at 1024); finished lanes return at once and wait for the
// warp's next refill. Where a call ends changes no result.

// The lane pass, persistent: warps pull samples from the pass's work counter
// and refill idle lanes together. T = float is the mixed pass (orbit staged in
// shared memory when it fits; samples its error estimate cannot vouch for are
// queued for the FP64 pass); T = double is that FP64 pass over the queue, whose
// length it reads on the device.
// LANES < 32: only the low LANES lanes of a warp take samples. The rerun
// passes are latency-bound (few samples, long dependency chains), so spreading
// their samples over more warps hides more latency than filling each warp.
template <class T, int MAXT, int MINB, int LANES = 32, bool INTR = true, bool FASTI = false, bool DE = false>
__global__ void __launch_bounds__(MAXT, MINB) k_lane_pass(DeviceFrame f, MixedParams p, const BlaEntry<T>* blat, const typename LaneReal<T>::V2* orbit) {
    using V2 = typename LaneReal<T>::V2;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ unsigned long long mbar;
    __shared__ int stage_ok;
    const FrameGeom& g = p.g;
    const V2* orb = orbit;
    const int n = f.px.n_dev ? min((int)*f.px.n_dev, f.px.n) : f.px.n;
    // Of a two-width launch only the variant chosen by the queue length runs.
    if (p.wide_from && ((unsigned)n >= p.wide_from) != (LANES == 32)) return;
    // Blocks past the work leave at once (the work counter hands all n entries
    // to the lower blocks), before any orbit staging.
    if ((long long)blockIdx.x * (MAXT / 32) * LANES >= n) return;
    const unsigned take = LANES == 32 ? 0xffffffffu : ((1u << LANES) - 1u);
    bool stage_late = false;
    if (LaneReal<T>::kTrackError && p.orbit_in_smem) {
        V2* so = reinterpret_cast<V2*>(smem_raw);
        bool ok = stage_orbit(reinterpret_cast<float2*>(so), reinterpret_cast<const float2*>(orbit), p.smem_entries * (int)(sizeof(V2) / sizeof(float2)), &mbar);
        if (threadIdx.x == 0) stage_ok = ok ? 1 : 0;
        __syncthreads();
        if (stage_ok) {
            orb = so;
        } else {
            // the copy did not complete within the wait limit: this block reads
            // the orbit from global memory instead, and waits for the copy
            // again (bounded) before it exits, so that no copy outlives it
            stage_late = true;
            if (threadIdx.x == 0) atomicAdd(&f.ctr->stage_timeouts, 1u);
        }
    }
    const int reflen = p.mx_ref_it + 1;
    const T ESC2f = T(p.esc2f); // (unused by the lanes; no FP64 conversion)
    const int blamask = (1 << f.bla.minlevel) - 1;
    const BlaEntry<T>* bt = f.bla.use ? blat : nullptr;
    const TE<T> dxf = te_from_fe<T>(p.dxfe), dyf = te_from_fe<T>(p.dyfe);
    const unsigned lane_id = threadIdx.x & 31;
    // per-thread counts of one pass (32-bit: a thread executes far fewer than
    // 2^32 steps per pass); skipped and effective iterations stay 64-bit
    unsigned n_steps = 0, n_bla = 0, n_rebase = 0, n_exact = 0, n_ferebase = 0, n_intflag = 0, n_escflag = 0;
    unsigned long long n_skip = 0, n_eff = 0;
    unsigned int n_int = 0, n_fin = 0;
    Lane<T> L;
    unsigned cost0 = 0;
    bool live = false, exhausted = false, stop = false;
    unsigned rounds = 0;
    for (;;) {
        // Warp-synchronous refill: every idle lane takes a new sample together,
        // so the per-sample setup runs once for all of them.
        const unsigned idle = __ballot_sync(0xffffffffu, !live) & take;
        if (idle && !exhausted) {
            int base = 0;
            const int leader = __ffs(idle) - 1;
            if ((int)lane_id == leader) base = (int)atomicAdd(&f.ctr->next, (unsigned)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base >= n) exhausted = true;
            if (!live && ((take >> lane_id) & 1u)) {
                const int i = base + __popc(idle & ((1u << lane_id) - 1u));
                if (i < n && !stop) {
                    lane_setup(L, i, f, p, dxf, dyf, orb);
                    cost0 = (unsigned)(n_steps + 4 * n_bla);
                    live = true;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, live) == 0) break;
        if (p.probe_stop) {
            // the gate's answer is settled once one sample is interior: the
            // probe's samples are rendered again by the main pass
            unsigned hit = 0;
            if (lane_id == 0) hit = *(volatile unsigned*)&f.ctr->probe_hit;
            if (__shfl_sync(0xffffffffu, hit, 0)) {
                exhausted = true;
                live = false;
                break;
            }
        }
        if (live) {
            T zrad = T(0);
            const int st = lane_run<T, INTR, FASTI, DE>(L, p.lane_budget, f, p, bt, orb, reflen, ESC2f, blamask, zrad, n_steps, n_bla, n_skip, n_rebase, n_exact, n_ferebase);
            if (p.probe_stop && (st == 2 || st == 4)) atomicExch(&f.ctr->probe_hit, 1u);
            if (st != 0 && f.out.cost) f.out.cost[L.oidx] = (unsigned)(n_steps + 4 * n_bla) - cost0;
            if (st == 1) {
                lane_write_escape<DE>(f.out, g, p, L, zrad);
                f.out.done[L.i] = 1;
                ++n_fin;
                n_eff += (unsigned long long)L.iter;
                live = false;
            } else if (st == 2) {
                lane_write_interior<DE>(f.out, g, L);
                f.out.done[L.i] = 1;
                ++n_fin;
                n_eff += (unsigned long long)g.mxit;
                ++n_int;
                live = false;
            } else if (LaneReal<T>::kTrackError && st >= 3) { // queued for the next tier
                if (st == 4) ++n_intflag;
                if (st == 5) ++n_escflag;
                const unsigned q = atomicAdd(&f.ctr->rerun_n, 1u);
                if (f.rerun_flag) {
                    f.rerun_flag[L.i] = 1; // queued in entry order after the pass
                } else {
                    int a[4];
                    entry_coords(f.px, L.i, a);
                    f.rerun_keys[q] = key_pack(a[0], a[1], a[2], a[3]);
                }
                f.out.done[L.i] = 1;
                ++n_fin;
                live = false;
            }
        }
        if (((++rounds & 31u) == 0) && mcancelled(f)) {
            stop = true;
            exhausted = true;
            live = false;
        }
    }
    atomicAdd(&f.ctr->steps, (unsigned long long)n_steps);
    atomicAdd(&f.ctr->bla_applies, (unsigned long long)n_bla);
    atomicAdd(&f.ctr->bla_skipped, n_skip);
    atomicAdd(&f.ctr->effective_iters, n_eff);
    atomicAdd(&f.ctr->rebases, (unsigned long long)n_rebase);
    atomicAdd(&f.ctr->exact_steps, (unsigned long long)n_exact);
    atomicAdd(&f.ctr->fe_rebases, (unsigned long long)n_ferebase);
    atomicAdd(&f.ctr->finished, n_fin);
    if (n_intflag) atomicAdd(&f.ctr->interior_flagged, n_intflag);
    if (n_escflag) atomicAdd(&f.ctr->escape_flagged, n_escflag);
    atomicAdd(&f.ctr->interior, n_int);
    if (stage_late && !mbar_wait_bounded((unsigned)__cvta_generic_to_shared(&mbar), 1 << 24) && threadIdx.x == 0) atomicAdd(&f.ctr->stage_timeouts, 1u << 16);
}

// ---- batched passes over several views ------------------------------------
template <class T>
struct ViewTables;
template <>
struct ViewTables<float> {
    __device__ static const Bla32* bla(const ViewDesc& v) { return v.bla32; }
    __device__ static const float2* orb(const ViewDesc& v) { return v.orb32; }
};
template <>
struct ViewTables<df32> {
    __device__ static const BlaDF* bla(const ViewDesc& v) { return v.bladf; }
    __device__ static const df2* orb(const ViewDesc& v) { return v.orbdf; }
};

// One persistent launch over the samples of several views: the FP32 pass takes
// all views' pixel sets back to back (a batch-wide work counter, so SMs that
// finish one view's samples continue with another's), the rerun passes take a
// queue whose keys carry the view index. Each lane reads its view's descriptor
// from device memory; lanes of one warp may work on different views.
template <class T, int MAXT, int MINB, int LANES = 32, bool DE = false>
__global__ void __launch_bounds__(MAXT, MINB) k_batch_pass(BatchArgs a) {
    using V2 = typename LaneReal<T>::V2;
    __shared__ unsigned s_base[kBatchMaxViews];
    const int nv = a.nviews;
    for (int v = threadIdx.x; v < nv; v += MAXT) s_base[v] = a.views[v].base;
    __syncthreads();
    const unsigned n = a.queue ? min(*a.queue_n, a.capacity) : a.total;
    if (a.wide_from && (n >= a.wide_from) != (LANES == 32)) return;
    if ((unsigned long long)blockIdx.x * (MAXT / 32) * LANES >= n) return;
    const unsigned take = LANES == 32 ? 0xffffffffu : ((1u << LANES) - 1u);
    const unsigned lane_id = threadIdx.x & 31;
    // per-thread counts of one pass (32-bit: a thread executes far fewer than
    // 2^32 steps per pass); skipped and effective iterations stay 64-bit
    unsigned n_steps = 0, n_bla = 0, n_rebase = 0, n_exact = 0, n_ferebase = 0, n_intflag = 0;
    unsigned long long n_skip = 0, n_eff = 0;
    unsigned int n_int = 0, n_fin = 0;
    Lane<T> L;
    int view = 0;
    unsigned cost0 = 0, bla0 = 0;
    bool live = false, exhausted = false, stop = false;
    unsigned rounds = 0;
    for (;;) {
        const unsigned idle = __ballot_sync(0xffffffffu, !live) & take;
        if (idle && !exhausted) {
            unsigned base = 0;
            const int leader = __ffs(idle) - 1;
            if ((int)lane_id == leader) base = atomicAdd(&a.ctr->next, (unsigned)__popc(idle));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (base >= n) exhausted = true;
            if (!live && ((take >> lane_id) & 1u)) {
                const unsigned g = base + __popc(idle & ((1u << lane_id) - 1u));
                if (g < n && !stop) {
                    int arr[4];
                    int v;
                    unsigned gn = g; // the sample's batch-wide index in the natural order
                    if (a.queue) {
                        const uint64_t k = a.queue[g];
                        v = (int)(k >> kBatchViewShift);
                        key_unpack(k & ((1ull << kBatchViewShift) - 1ull), arr);
                    } else {
                        if (a.order) gn = (unsigned)a.order[g];
                        int lo = 0, hi = nv - 1; // last view with base <= gn
                        while (lo < hi) {
                            const int mid = (lo + hi + 1) >> 1;
                            if (s_base[mid] <= gn) lo = mid;
                            else hi = mid - 1;
                        }
                        v = lo;
                        entry_coords(a.views[v].f.px, (int)(gn - s_base[v]), arr);
                    }
                    const ViewDesc& vd = a.views[v];
                    if (a.view_interior && !vd.f.out.cost && *(volatile const unsigned*)&a.view_interior[v] != 0u) {
                        // the probe of a view whose gate is settled (an interior
                        // sample found): its samples are rendered again by the main pass
                        ++n_fin;
                    } else {
                        lane_setup_at(L, (int)gn, arr, vd.p, te_from_fe<T>(vd.p.dxfe), te_from_fe<T>(vd.p.dyfe), ViewTables<T>::orb(vd));
                        cost0 = (unsigned)(n_steps + 4 * n_bla);
                        bla0 = n_bla;
                        view = v;
                        live = true;
                    }
                }
            }
        }
        if (__ballot_sync(0xffffffffu, live) == 0) break;
        if (live && a.view_interior && !a.views[view].f.out.cost && *(volatile const unsigned*)&a.view_interior[view] != 0u) {
            ++n_fin; // this view's gate is settled
            live = false;
        }
        if (live) {
            const ViewDesc& vd = a.views[view];
            const BlaEntry<T>* bt = vd.f.bla.use ? ViewTables<T>::bla(vd) : nullptr;
            T zrad = T(0);
            const int st = lane_run<T, true, false, DE>(L, vd.p.lane_budget, vd.f, vd.p, bt, ViewTables<T>::orb(vd), vd.p.mx_ref_it + 1, T(vd.p.esc2f), (1 << vd.f.bla.minlevel) - 1, zrad,
                                                       n_steps, n_bla, n_skip, n_rebase, n_exact, n_ferebase);
            // the learned ordering's costs: the FP32 tier's (the rerun tiers keep them)
            if (std::is_same<T, float>::value && st != 0 && vd.f.out.cost) {
                vd.f.out.cost[L.oidx] = (unsigned)(n_steps + 4 * n_bla) - cost0;
                if (vd.f.out.bla) vd.f.out.bla[L.oidx] = n_bla - bla0;
            }
            if (st == 1) {
                lane_write_escape<DE>(vd.f.out, vd.p.g, vd.p, L, zrad);
                ++n_fin;
                n_eff += (unsigned long long)L.iter;
                live = false;
            } else if (st == 2) {
                lane_write_interior<DE>(vd.f.out, vd.p.g, L);
                if (a.view_interior) atomicAdd(&a.view_interior[view], 1u);
                ++n_fin;
                n_eff += (unsigned long long)vd.p.g.mxit;
                ++n_int;
                live = false;
            } else if (LaneReal<T>::kTrackError && st >= 3) {
                // an unvouched interior decision counts for the probe's gate
                if (st == 4 && a.view_interior) atomicAdd(&a.view_interior[view], 1u);
                int c[4];
                const int row = (L.oidx / (vd.p.g.W * vd.p.g.sub)), col = L.oidx % (vd.p.g.W * vd.p.g.sub);
                c[0] = row / vd.p.g.sub;
                c[1] = col / vd.p.g.sub;
                c[2] = row - c[0] * vd.p.g.sub - vd.p.g.sub / 2;
                c[3] = col - c[1] * vd.p.g.sub - vd.p.g.sub / 2;
                const unsigned q = atomicAdd(&a.ctr->rerun_n, 1u);
                if (a.rerun_flag) a.rerun_flag[L.i] = 1; // queued in the natural order after the pass
                else if (q < a.capacity) a.next_queue[q] = key_pack(c[0], c[1], c[2], c[3]) | ((uint64_t)view << kBatchViewShift);
                ++n_fin;
                live = false;
            }
        }
        if (((++rounds & 31u) == 0) && a.cancel && *a.cancel) {
            stop = true;
            exhausted = true;
            live = false;
        }
    }
    atomicAdd(&a.ctr->steps, (unsigned long long)n_steps);
    atomicAdd(&a.ctr->bla_applies, (unsigned long long)n_bla);
    atomicAdd(&a.ctr->bla_skipped, n_skip);
    atomicAdd(&a.ctr->effective_iters, n_eff);
    atomicAdd(&a.ctr->rebases, (unsigned long long)n_rebase);
    atomicAdd(&a.ctr->exact_steps, (unsigned long long)n_exact);
    atomicAdd(&a.ctr->fe_rebases, (unsigned long long)n_ferebase);
    atomicAdd(&a.ctr->finished, n_fin);
    atomicAdd(&a.ctr->interior, n_int);
}

// Between the probe and the main pass: interior detection of each view follows
// its probe's interior count (mp.cpp:1668-1720).
__global__ void k_batch_gate(ViewDesc* views, int n, const unsigned* view_interior) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n && views[v].interior_gate) views[v].p.use_interior = view_interior[v] > 0 ? 1 : 0;
}

__global__ void k_orbit_to_float(const double2* Z, float2* Zf, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) Zf[i] = make_float2((float)Z[i].x, (float)Z[i].y);
}

// The common-step table of the FP32 lane (MixedParams::Zq).
__global__ void k_orbit_to_q(const double2* Z, float4* Zq, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = (float)Z[i].x, y = (float)Z[i].y;
    constexpr float tiny = LaneReal<float>::kTinyX;
    const float xr2 = fmaf(x, x, y * y);
    const bool in_range = !(fabsf(x) < tiny && fabsf(y) < tiny) && xr2 > tiny * tiny;
    Zq[i] = make_float4(x + x, y + y, in_range ? xr2 : 0.0f, 0.0f);
}

__global__ void k_orbit_to_df(const double2* Z, df2* Zd, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) Zd[i] = df2{df32(Z[i].x), df32(Z[i].y)};
}

__global__ void k_fma_probe_f32(float* out, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = __fmaf_rn(x0, a, b); x1 = __fmaf_rn(x1, a, b); x2 = __fmaf_rn(x2, a, b); x3 = __fmaf_rn(x3, a, b);
        x4 = __fmaf_rn(x4, a, b); x5 = __fmaf_rn(x5, a, b); x6 = __fmaf_rn(x6, a, b); x7 = __fmaf_rn(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void k_fma_probe_f64(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = __fma_rn(x0, a, b); x1 = __fma_rn(x1, a, b); x2 = __fma_rn(x2, a, b); x3 = __fma_rn(x3, a, b);
        x4 = __fma_rn(x4, a, b); x5 = __fma_rn(x5, a, b); x6 = __fma_rn(x6, a, b); x7 = __fma_rn(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

} // namespace

int Engine::measure_fma_peak(int fp64, double* tflops) {
    const int blocks = nsm_ * 8, threads = 256;
    const int iters = fp64 ? 2000 : 40000;
    void* buf = nullptr;
    if (cudaMalloc(&buf, (size_t)blocks * threads * 8) != cudaSuccess) return MBX_E_NOMEM;
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(ev0_, st_);
        if (fp64) k_fma_probe_f64<<<blocks, threads, 0, st_>>>((double*)buf, iters, 0.999999, 1e-7);
        else k_fma_probe_f32<<<blocks, threads, 0, st_>>>((float*)buf, iters, 0.999999f, 1e-7f);
        cudaEventRecord(ev1_, st_);
        cudaError_t e = cudaEventSynchronize(ev1_);
        if (e != cudaSuccess) {
            cudaFree(buf);
            return fail_cuda("fma probe", e);
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, ev0_, ev1_);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaFree(buf);
    *tflops = 2.0 * 8.0 * (double)blocks * threads * iters / (best * 1e-3) / 1e12;
    return MBX_OK;
}

int Engine::prepare_mixed() {
    const int len = orbit_len_;
    {
        // sample offsets from the reference per supersampled column and row
        // (the lane's expression, evaluated here once per frame)
        const int nx = W_ * SUB_, ny = H_ * SUB_;
        hdpxy_.resize((size_t)(nx + ny));
        hdpxyf_.resize((size_t)(nx + ny));
        for (int k = 0; k < nx; ++k) {
            const int a1 = k / SUB_, a3 = k % SUB_ - SUB_ / 2;
            hdpxy_[(size_t)k] = a1 + (double)a3 / SUB_ - ref_x_;
        }
        for (int k = 0; k < ny; ++k) {
            const int a0 = k / SUB_, a2 = k % SUB_ - SUB_ / 2;
            hdpxy_[(size_t)(nx + k)] = a0 + (double)a2 / SUB_ - ref_y_;
        }
        for (size_t k = 0; k < hdpxy_.size(); ++k) hdpxyf_[k] = (float)hdpxy_[k];
        if (!ensure(ddpxy_, hdpxy_.size()) || !ensure(ddpxyf_, hdpxyf_.size())) return MBX_E_NOMEM;
        copy_async(ddpxy_.p, hdpxy_.data(), sizeof(double) * hdpxy_.size(), cudaMemcpyHostToDevice);
        copy_async(ddpxyf_.p, hdpxyf_.data(), sizeof(float) * hdpxyf_.size(), cudaMemcpyHostToDevice);
        dpxy_w_ = nx;
    }
    if (!ensure(dZf_, (size_t)len + 4) || !ensure(dZdf_, (size_t)len + 4) || !ensure(dZq_, (size_t)len + 4)) return MBX_E_NOMEM;
    k_orbit_to_float<<<(len + 255) / 256, 256, 0, st_>>>(dZ_.p, dZf_.p, len);
    k_orbit_to_df<<<(len + 255) / 256, 256, 0, st_>>>(dZ_.p, dZdf_.p, len);
    k_orbit_to_q<<<(len + 255) / 256, 256, 0, st_>>>(dZ_.p, dZq_.p, len);
    stats_.kernel_launches += 3;
    if (bla_.use && bla_.nlev > 0) {
        int n = bla_.off[bla_.nlev - 1] + bla_.size[bla_.nlev - 1];
        if (!ensure(dbla32_, (size_t)n) || !ensure(dbladf_, (size_t)n)) return MBX_E_NOMEM;
        k_bla_to_lane<float><<<(n + 255) / 256, 256, 0, st_>>>(dr2_.p, dab_.p, dbla32_.p, n);
        k_bla_to_lane<df32><<<(n + 255) / 256, 256, 0, st_>>>(dr2_.p, dab_.p, dbladf_.p, n);
        const int nq = (len >> bla_.minlevel) + 2;
        if (!ensure(dblamax_, (size_t)nq)) return MBX_E_NOMEM;
        k_bla_maxr2<<<(nq + 255) / 256, 256, 0, st_>>>(dbla32_.p, bla_, dblamax_.p, nq);
        stats_.kernel_launches += 3;
        blamax_ok_ = true;
    } else {
        blamax_ok_ = false;
    }
    return cuda_ok("mixed preparation");
}

MixedParams Engine::mixed_params() const {
    MixedParams p;
    p.g = geom();
    p.dxfe = dxfe_;
    p.dyfe = dyfe_;
    p.ref_x = ref_x_;
    p.ref_y = ref_y_;
    p.per = ref_period_;
    p.mx_ref_it = ref_period_ > 0 ? ref_period_ : orbit_len_ - 1;
    p.use_interior = use_interior_ ? 1 : 0;
    p.interior_eps2 = interior_eps2_;
    p.interior_confirm = interior_confirm_;
    p.Zf = dZf_.p;
    p.Zq = dZq_.p;
    p.esc2f = (float)p.g.ESC2;
    p.esc2lo = p.esc2f * LaneReal<float>::kEscLo;
    p.Zsmall = nullptr;
    p.orbit_in_smem = 0;
    p.smem_entries = orbit_len_;
    p.wmax2 = mixed_wmax2_;
    p.wmin2 = 1.0f / mixed_wmax2_;
    p.blamax = blamax_ok_ ? dblamax_.p : nullptr;
    if (ddpxy_.p && dpxy_w_ == W_ * SUB_) {
        p.dpx_tab = ddpxy_.p;
        p.dpy_tab = ddpxy_.p + dpxy_w_;
        p.dpx_tabf = ddpxyf_.p;
        p.dpy_tabf = ddpxyf_.p + dpxy_w_;
    }
    p.lane_budget = lane_budget_;
    return p;
}

cudaError_t Engine::run_mixed_pass(const DeviceFrame& f) {
    MixedParams p = mixed_params();
    const size_t bytes = ((size_t)orbit_len_ * 8 + 15) & ~(size_t)15;
    p.orbit_in_smem = (bytes <= (size_t)smem_orbit_limit_) ? 1 : 0;
    const int threads = mixed_threads_;
    const int blocks = std::max(1, std::min((f.px.n + threads - 1) / threads, nsm_ * mixed_blocks_per_sm_));
    const size_t smem = p.orbit_in_smem ? bytes : 0;
    DeviceFrame g = f;
    if (!(bla_.use && dbla32_.p)) g.bla.use = 0;
    // the interior gate's probe stops at its first interior decision (unless
    // its per-sample costs are wanted); it needs no DE values (the main pass
    // renders its samples again)
    p.probe_stop = (probe_gate_only_ && !g.out.cost) ? 1 : 0;
    if (probe_gate_only_) p.g.ede = p.g.deovl = p.g.normal = p.g.deriv = 0;
    auto launch = [&](auto kern) -> cudaError_t {
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        kern<<<blocks, threads, smem, st_>>>(g, p, dbla32_.p, dZf_.p);
        return cudaGetLastError();
    };
    if (probe_gate_only_ && threads == 256 && mixed_blocks_per_sm_ == 3) // the probe: common iterations in the fast loop too
        return launch(k_lane_pass<float, 256, 3, 32, true, true>);
    if (p.g.deriv) { // DE colourings: the lanes carry the derivative (one launch shape)
        if (!p.use_interior) return launch(k_lane_pass<float, 256, 3, 32, false, false, true>);
        return launch(k_lane_pass<float, 256, 3, 32, true, false, true>);
    }
    if (!p.use_interior) { // exterior after the probe: the lane without interior detectors
        if (mixed_blocks_per_sm_ >= 4) return launch(k_lane_pass<float, 256, 4, 32, false>);
        if (mixed_blocks_per_sm_ == 3) return launch(k_lane_pass<float, 256, 3, 32, false>);
        return launch(k_lane_pass<float, 256, 2, 32, false>);
    }
    if (mixed_blocks_per_sm_ >= 4) return launch(k_lane_pass<float, 256, 4>);
    if (mixed_blocks_per_sm_ == 3) return launch(k_lane_pass<float, 256, 3>);
    return launch(k_lane_pass<float, 256, 2>);
}

// The double-float lane pass over the mixed pass's queue (entry count read on
// the device). What it cannot vouch for, it queues for the exact form.
cudaError_t Engine::run_df_pass(const DeviceFrame& f) {
    MixedParams p = mixed_params();
    const size_t bytes = ((size_t)orbit_len_ * 16 + 15) & ~(size_t)15;
    p.orbit_in_smem = (bytes <= (size_t)smem_orbit_limit_) ? 1 : 0;
    const size_t smem = p.orbit_in_smem ? bytes : 0;
    DeviceFrame g = f;
    if (!(bla_.use && dbladf_.p)) g.bla.use = 0;
    const int threads = 128;
    const int blocks = std::max(1, std::min((f.px.n + 31) / 32, nsm_ * 4));
    // the queue length is known only on the device: both widths are launched
    // and the one it selects runs
    p.wide_from = kWideLanesPerSm * (unsigned)nsm_;
    auto narrow = p.g.deriv ? k_lane_pass<df32, 128, 2, 8, true, false, true> : k_lane_pass<df32, 128, 2, 8>;
    auto wide = p.g.deriv ? k_lane_pass<df32, 128, 2, 32, true, false, true> : k_lane_pass<df32, 128, 2, 32>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(narrow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    narrow<<<blocks, threads, smem, st_>>>(g, p, dbladf_.p, dZdf_.p);
    wide<<<std::max(1, std::min((f.px.n + 127) / 128, nsm_ * 4)), threads, smem, st_>>>(g, p, dbladf_.p, dZdf_.p);
    return cudaGetLastError();
}

// Batched passes: one FP32 launch over all views, then the double-float tier
// (what it cannot vouch for goes to each view's exact form on the host side).
cudaError_t launch_batch_pass(int tier, const BatchArgs& a, int nsm, cudaStream_t st) {
    if (tier == 0) {
        if (a.deriv) k_batch_pass<float, 256, 3, 32, true><<<nsm * 3, 256, 0, st>>>(a);
        else k_batch_pass<float, 256, 3><<<nsm * 3, 256, 0, st>>>(a);
    } else {
        BatchArgs b = a;
        b.wide_from = kWideLanesPerSm * (unsigned)nsm;
        if (a.deriv) {
            k_batch_pass<df32, 128, 2, 8, true><<<nsm * 4, 128, 0, st>>>(b);
            k_batch_pass<df32, 128, 2, 32, true><<<nsm * 4, 128, 0, st>>>(b);
        } else {
            // 128 registers without spills: four blocks of 128 per SM (a
            // batch's queue holds many waves of samples; measured on 24
            // tiles of the 1e-500 image, 1.2M queued: 372 -> 332 ms)
            k_batch_pass<df32, 128, 4, 8><<<nsm * 4, 128, 0, st>>>(b);
            k_batch_pass<df32, 128, 4, 32><<<nsm * 4, 128, 0, st>>>(b);
        }
    }
    return cudaGetLastError();
}

// The FP32 pass's leftovers as the next tier's queue in the batch's natural
// order (view by view, rows of samples) rather than the order they failed in:
// neighbouring samples share a warp (their BLA skips and rebases coincide) and
// the lanes read one or two views' orbit and BLA tables at a time (a batch's
// tables together can exceed L2). Measured on 24 tiles of the 1e-500 image at
// maxiter 2e6 (1.2M leftovers): double-float tier 332 ms in failure order,
// 225 ms in the natural order. The order changes no output.
constexpr unsigned kFlagBlock = 4096; // flags per block (1024 threads x 4)

unsigned flag_blocks(unsigned total) { return (total + kFlagBlock - 1) / kFlagBlock; }

__global__ void __launch_bounds__(1024) k_flag_sums(const uint8_t* flag, unsigned total, unsigned* sums) {
    __shared__ unsigned ws[32];
    const unsigned g0 = blockIdx.x * kFlagBlock + threadIdx.x * 4;
    unsigned c = 0;
    for (int k = 0; k < 4; ++k) c += (g0 + k < total && flag[g0 + k]) ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < 32; ++w) t += ws[w];
        sums[blockIdx.x] = t;
    }
}
// exclusive scan of the block sums in place (one block)
__global__ void __launch_bounds__(1024) k_flag_scan(unsigned nb, unsigned* sums) {
    __shared__ unsigned part[1024];
    const unsigned t = threadIdx.x, per = (nb + 1023) / 1024, lo = t * per, hi = min(nb, lo + per);
    unsigned run = 0;
    for (unsigned k = lo; k < hi; ++k) run += sums[k];
    part[t] = run;
    __syncthreads();
    for (unsigned o = 1; o < 1024; o <<= 1) {
        const unsigned add = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    unsigned base = part[t] - run;
    for (unsigned k = lo; k < hi; ++k) {
        const unsigned c = sums[k];
        sums[k] = base;
        base += c;
    }
}
// keys of flagged samples: batch-wide indices over views, or a pass's entries
struct ViewsKeys {
    const ViewDesc* views;
    int nv;
    __device__ uint64_t operator()(unsigned g) const {
        int lo = 0, hi = nv - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (views[mid].base <= g) lo = mid;
            else hi = mid - 1;
        }
        int arr[4];
        entry_coords(views[lo].f.px, (int)(g - views[lo].base), arr);
        return key_pack(arr[0], arr[1], arr[2], arr[3]) | ((uint64_t)lo << kBatchViewShift);
    }
};
struct EntryKeys {
    PixelSet px;
    __device__ uint64_t operator()(unsigned g) const {
        int arr[4];
        entry_coords(px, (int)g, arr);
        return key_pack(arr[0], arr[1], arr[2], arr[3]);
    }
};
template <class Keys>
__global__ void __launch_bounds__(1024) k_flag_emit(Keys keys, const uint8_t* flag, unsigned total, const unsigned* sums, uint64_t* out) {
    __shared__ unsigned ws[32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned g0 = blockIdx.x * kFlagBlock + threadIdx.x * 4;
    bool f[4];
    unsigned c = 0;
    for (int k = 0; k < 4; ++k) {
        f[k] = g0 + k < total && flag[g0 + k];
        c += f[k] ? 1u : 0u;
    }
    // exclusive prefix of c over the block, in thread order
    unsigned x = c;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if ((int)lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if ((int)lane >= o) w += y;
        }
        ws[lane] = w;
    }
    __syncthreads();
    unsigned pos = sums[blockIdx.x] + (warp ? ws[warp - 1] : 0u) + x - c;
    for (int k = 0; k < 4; ++k)
        if (f[k]) out[pos++] = keys(g0 + k);
}

template <class Keys>
cudaError_t flag_compact(Keys keys, unsigned total, const uint8_t* flag, unsigned* sums, uint64_t* out, cudaStream_t st) {
    const unsigned nb = flag_blocks(total);
    if (nb == 0) return cudaSuccess;
    k_flag_sums<<<nb, 1024, 0, st>>>(flag, total, sums);
    k_flag_scan<<<1, 1024, 0, st>>>(nb, sums);
    k_flag_emit<<<nb, 1024, 0, st>>>(keys, flag, total, sums, out);
    return cudaGetLastError();
}
cudaError_t launch_flag_compact(const ViewDesc* views, int nv, unsigned total, const uint8_t* flag, unsigned* sums, uint64_t* out, cudaStream_t st) {
    return flag_compact(ViewsKeys{views, nv}, total, flag, sums, out, st);
}
cudaError_t launch_flag_compact(const PixelSet& px, unsigned total, const uint8_t* flag, unsigned* sums, uint64_t* out, cudaStream_t st) {
    return flag_compact(EntryKeys{px}, total, flag, sums, out, st);
}

cudaError_t launch_batch_gate(ViewDesc* views, int n, const unsigned* view_interior, cudaStream_t st) {
    k_batch_gate<<<(n + 127) / 128, 128, 0, st>>>(views, n, view_interior);
    return cudaGetLastError();
}

} // namespace mbx

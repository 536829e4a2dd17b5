/*
 * wfe_kernels.cu -- the alignment path on sm_103a.
 *
 *   pack_kernel          ASCII -> 2-bit words (src/kernels.cu:313-394)
 *   tier_kernel<Tier>    fused load+pack, wavefront compute+extend, bit-packed
 *                        backtrace store, backtrace and CIGAR replay for one
 *                        pair per group of G lanes (src/kernels.cu:27-310 and
 *                        397-625 in one kernel)
 *   long_kernel<GWF, NT> the same for one pair per CTA of NT threads
 *                        (tiers 5-6), over the target's cone when the pair
 *                        has a distance bound
 *   bound_kernel         distance bounds from a 32-diagonal band, one warp
 *                        per pair; routes tier 5's pairs to distance classes
 *   classify_kernel      length buckets and predicted tiers
 *   history_cigar_kernel CIGARs from the reference's 128-bit histories
 *                        (src/kernels.cu:397-625)
 *
 * Wavefront layout of tier_kernel: lane g of a group holds, in register
 * chunk c (c = 0..2J), diagonal k = G*(c-J) - G/2 + g.  Neighbours k-1 and
 * k+1 come from one rotating shuffle each; the lanes at a chunk edge pick up
 * the neighbouring chunk's value.  A chunk is skipped (warp-uniformly) until
 * the wavefront [-d, d] reaches it; lanes outside [-d, d] hold -1, the
 * reference's sentinel (src/kernels.cu:205-219).
 *
 * Backtrace store: per score d and chunk, two ballots give the low and high
 * bits of the 2-bit operation of every diagonal of the chunk (2 bits per
 * cell).  The chain is then read back from (D, kt) to (0, 0); it equals the
 * reference's forward history, which copies the history of the source
 * diagonal k + op - 2 and adds op at field d-1 (src/kernels.cu:154-171).
 */
#include "wfe_kernels.cuh"

#include <algorithm>
#include <climits>
#include <map>
#include <mutex>
#include <tuple>

namespace wfe {

namespace {

/* Raise, never lower, a kernel's dynamic shared memory limit on the current
 * device.  The limit is a property of the kernel, and a tier launched on the
 * device by one bucket's chain relies on it still covering that bucket after
 * the host has launched the same tier for a smaller bucket. */
cudaError_t allow_smem(const void* fn, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> limit;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = limit[{fn, dev}];
    if (bytes <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;

enum : int { ST_IDLE = 0, ST_RUN, ST_DONE, ST_OVERFLOW, ST_OVERMAX, ST_TOOLONG, ST_BADWALK, ST_RANGE };

__host__ __device__ constexpr size_t round16(size_t x) { return (x + 15u) & ~size_t(15); }

/* Backtrace store entry of one chunk of one score step: the two ballots of
 * the warp -- the low and the high bits of the 2-bit operation of every lane's
 * diagonal -- written by lane 0.  Group grp's diagonal g of the chunk is bit
 * grp * G + g.  A warp of several groups (G < 32) keeps one store for all of
 * them, so the ballots are stored as they come, with no per-group shifting and
 * masking in the score loop; the backtrace picks its group's bits. */
__device__ __forceinline__ int op_of(uint2 e, int bit)
{
    return (int)(((e.x >> bit) & 1u) | (((e.y >> bit) & 1u) << 1));
}

/* One distance tier: G lanes per pair, 2J+1 register chunks, backtrace
 * store in shared (SMEM_OPS) or global memory, sequences of up to RMAX*G
 * aligned 16-byte blocks loaded with all loads in flight at once, at least
 * MINB resident CTAs per SM asked of the register allocator. */
template <int G_, int J_, bool SMEM_OPS_, int RMAX_, int MINB_ = 1>
struct Tier {
    static constexpr int G = G_, J = J_, RMAX = RMAX_, MINB = MINB_;
    static constexpr bool SMEM_OPS = SMEM_OPS_;
    static constexpr int NC = 2 * J + 1;
    static constexpr int DCAP = G * J + G / 2 - 1;
    static constexpr int GPW = 32 / G;
    /* Row d of the backtrace store.  The 32-lane tiers keep only the chunks
     * that score step d touches -- the contiguous range whose diagonals meet
     * [-d, d] -- row after row (a triangle, 55-68 % of DCAP x NC entries),
     * which keeps tier 1's store in shared memory small and tiers 2-4's
     * global scratch mostly in L2.  Tier 0
     * keeps full rows: its occupancy is set by registers, and it is
     * issue-bound, so it saves the index arithmetic instead. */
    static constexpr bool TRI = G == 32;
    static __host__ __device__ constexpr int chunk_lo(int d)
    {
        return !TRI ? 0 : (J - (d - 1 + G / 2) / G < 0 ? 0 : J - (d - 1 + G / 2) / G);
    }
    static __host__ __device__ constexpr int chunk_hi(int d)
    {
        return !TRI ? 2 * J : (J + (d + G / 2) / G > 2 * J ? 2 * J : J + (d + G / 2) / G);
    }
    static __host__ __device__ constexpr int row_entries(int d) { return chunk_hi(d) - chunk_lo(d) + 1; }
    /* entries of rows 1..rows */
    static constexpr int store_entries(int rows = DCAP)
    {
        int t = 0;
        for (int d = 1; d <= rows && d <= DCAP; ++d) t += row_entries(d);
        return t;
    }
    /* a group's share of its warp's store (one 8-byte entry per chunk and
     * score step, shared by the warp's GPW groups) */
    static constexpr size_t ops_bytes = round16((8u * (size_t)store_entries() + GPW - 1) / GPW);
    /* one group's store in global scratch (the 32-lane tiers: one group per
     * warp) for distances up to max_len */
    static size_t store_bytes(uint32_t max_len)
    {
        return round16(8u * (size_t)store_entries((int)std::min<uint32_t>(max_len, (uint32_t)DCAP)));
    }
    static int store_rows(uint32_t max_len) { return (int)std::min<uint32_t>(max_len, (uint32_t)DCAP); }
    static constexpr size_t chain_bytes = round16((size_t)DCAP + 1);
    static constexpr size_t runs_bytes = round16(sizeof(int) * ((size_t)DCAP + 1));
};

inline uint32_t seq_words_for(uint32_t max_len) { return std::max<uint32_t>(1u, (max_len + 15u) / 16u); }

/* Shared memory of one group: both sequences, the operation chain, then one
 * region that first holds the group's share of its warp's backtrace store
 * (when it lives in shared memory) and, once the chains have been read from
 * it, the group's CIGAR stage and the runs of the replay.  Within a warp's
 * block the groups' sequences and chains come first, then their union
 * regions one after another, which together hold the warp's store. */
template <class T>
size_t union_bytes(uint32_t cigar_stride)
{
    const size_t replay = round16(cigar_stride) + T::runs_bytes;
    return T::SMEM_OPS ? std::max(T::ops_bytes, replay) : replay;
}

template <class T>
size_t group_smem_bytes(uint32_t max_len, uint32_t cigar_stride)
{
    return 16u * (size_t)seq_words_for(max_len) + T::chain_bytes + union_bytes<T>(cigar_stride);
}

/* The tiers with several pairs per warp also keep, per warp, the packed
 * blocks of a coalesced span load of the warp's pairs (load_warp_span):
 * 160 blocks, 2,560 bytes of input, enough for 8 pairs of 150 bases stored
 * one after another with their file's line marks. */
constexpr int kSpanWords = 160;

template <class T>
size_t cta_smem_bytes(uint32_t max_len, uint32_t cigar_stride)
{
    const size_t span = T::G < 32 ? (size_t)kWarps * kSpanWords * sizeof(uint32_t) : 0u;
    return group_smem_bytes<T>(max_len, cigar_stride) * (size_t)(kWarps * T::GPW) + span;
}

/* The alignment kernel of a tier, in two forms with one body (tier_body):
 *   tier_kernel_bounded<T, PREDICT>  the 4-lane tier 0 and the prediction
 *       pass, launched from the host only, with launch bounds that set its
 *       register budget for 8 resident CTAs per SM;
 *   tier_kernel<T>  the tiers 1-4 that chains launch from the device, with
 *       no launch bounds: a grid launched from the device whose kernel
 *       declares launch bounds and uses dynamic shared memory was measured
 *       to run one CTA per SM at a time, whatever the bounds say. */
template <class T, bool PREDICT = false>
__global__ void __launch_bounds__(kThreads, T::MINB)
tier_kernel_bounded(const __grid_constant__ AlignLaunch A, uint32_t seq_words, uint32_t gbytes);
template <class T>
__global__ void tier_kernel(const __grid_constant__ AlignLaunch A, uint32_t seq_words, uint32_t gbytes);

/* Tier 0 carries the short-read workloads; its shape is tuned on the GPU
 * (4 lanes per pair, 11 chunks, 8 resident CTAs per SM by default). */
#ifndef WFE_T0_J
#define WFE_T0_J 5
#endif
#ifndef WFE_T0_MINB
#define WFE_T0_MINB 8
#endif
using T0 = Tier<4, WFE_T0_J, true, 5, WFE_T0_MINB>; /* distance <= 4*J + 1 (21) */

/* launched from the device too: no launch bounds (see tier_kernel) */
template <bool GLOBAL_WF, int NT>
__global__ void long_kernel(const __grid_constant__ AlignLaunch A);
__global__ void bound_kernel(const __grid_constant__ AlignLaunch A, uint32_t seq_words, uint32_t unused);
using T1 = Tier<32, 2, true, 1>;   /* distance <= 79  */
using T2 = Tier<32, 4, false, 1>;  /* distance <= 143; backtrace store in global scratch: 8 CTAs per SM */
using T3 = Tier<32, 8, false, 1>;  /* distance <= 271 */
using T4 = Tier<32, 16, false, 1>; /* distance <= 527 */

/* Record that the device-side launch of tier u failed: a plain store of one
 * byte (one per tier, so no two writers share a byte) into host memory that
 * the host reads once the chain has completed. */
__device__ __forceinline__ void note_launch_error(const AlignLaunch& A, int u)
{
    if (A.chain.launch_error) {
        *reinterpret_cast<volatile uint8_t*>(A.chain.launch_error + u) = 1u;
        __threadfence_system();
    }
}

/* Pairs of a chain cut short were deferred: the host aligns them once the
 * deeper tiers' scratch exists.  (Host memory the device writes in place,
 * like the launch failures.) */
__device__ __forceinline__ void note_deferred(const AlignLaunch& A)
{
    if (A.chain.launch_error) {
        *reinterpret_cast<volatile uint8_t*>(A.chain.launch_error + kDeferByte) = 1u;
        __threadfence_system();
    }
}

/* Tail launch of tier u over its list of `count` pairs, built in the launch's
 * own parameter buffer: A (a __grid_constant__ kernel parameter, read in
 * place) is copied word by word and the per-tier fields are patched.  No
 * copy of the launch record is made on the stack -- a kernel whose code
 * holds a large stack frame keeps only a few CTAs resident per SM, and that
 * limit is also what a grid launched from the device runs with. */
template <typename K>
__device__ __forceinline__ void tail_launch(K kernel, const AlignLaunch& A, int u, int grid, int threads,
                                            uint32_t smem, bool tier_args, uint32_t seq_words, uint32_t gbytes)
{
    void* buf = cudaGetParameterBufferV2((void*)kernel, dim3((unsigned)grid), dim3((unsigned)threads), smem);
    if (!buf) {
        note_launch_error(A, u);
        return;
    }
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&A);
    unsigned long long* dst = static_cast<unsigned long long*>(buf);
    static_assert(sizeof(AlignLaunch) % 8 == 0, "launch record is copied in 8-byte words");
#pragma unroll 4
    for (unsigned i = 0; i < sizeof(AlignLaunch) / 8; ++i) dst[i] = src[i];
    AlignLaunch* n = static_cast<AlignLaunch*>(buf);
    n->tier = u;
    n->cls = -1;
    n->work = A.chain.list[u];
    n->work_count = A.chain.counts + u;
    n->retry = u < A.chain.last_tier ? A.chain.list[u + 1] : A.chain.defer;
    n->retry_count = u < A.chain.last_tier ? A.chain.counts + u + 1 : A.chain.defer_count;
    n->passed_total = A.chain.passed ? A.chain.passed + u : nullptr;
    if (tier_args) {
        uint32_t* extra = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(buf) + sizeof(AlignLaunch));
        extra[0] = seq_words;
        extra[1] = gbytes;
    }
    if (cudaLaunchDeviceV2(buf, cudaStreamTailLaunch) != cudaSuccess) {
        note_launch_error(A, u);
        return;
    }
    if (A.chain.launched) atomicAdd(A.chain.launched + u, 1ull);
}

template <class T>
__device__ __forceinline__ void launch_on_device(const AlignLaunch& A, int u, uint32_t count)
{
    const TierShape& sh = A.chain.shape[u];
    const uint32_t per_cta = (uint32_t)(kWarps * T::GPW);
    const int grid = max(1, min(sh.grid, (int)((count + per_cta - 1u) / per_cta)));
    static_assert(T::G == 32, "only the 32-lane tiers are launched from the device");
    tail_launch(tier_kernel<T>, A, u, grid, kThreads, sh.smem, true, sh.seq_words, sh.gbytes);
}

/* Tail launch of distance class c of tier 5 over its list of `count`
 * pairs.  A pair that a class hands on (its bound was not one) goes to the
 * next class; the last class hands on to tier 6. */
__device__ void launch_class_on_device(const AlignLaunch& A, int c, uint32_t count)
{
    const LongClasses& C = A.chain.cls;
    const TierShape& sh = C.shape[c];
    const int grid = max(1, min(sh.grid, (int)count));
    const void* kernel = sh.threads == kLongTinyThreads    ? (const void*)long_kernel<false, kLongTinyThreads>
                         : sh.threads == kLongSmallThreads ? (const void*)long_kernel<false, kLongSmallThreads>
                                                           : (const void*)long_kernel<false, kLongThreads>;
    void* buf = cudaGetParameterBufferV2((void*)kernel, dim3((unsigned)grid), dim3((unsigned)sh.threads), sh.smem);
    if (!buf) {
        note_launch_error(A, 5);
        return;
    }
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(&A);
    unsigned long long* dst = static_cast<unsigned long long*>(buf);
#pragma unroll 4
    for (unsigned i = 0; i < sizeof(AlignLaunch) / 8; ++i) dst[i] = src[i];
    AlignLaunch* n = static_cast<AlignLaunch*>(buf);
    const bool last = c + 1 >= C.n;
    n->tier = 5;
    n->cls = c;
    n->work = C.list[c];
    n->work_count = C.counts + c;
    n->retry = !last ? C.list[c + 1] : (5 < A.chain.last_tier ? A.chain.list[6] : nullptr);
    n->retry_count = !last ? C.counts + c + 1 : A.chain.counts + 6;
    n->passed_total = last && A.chain.passed ? A.chain.passed + 5 : nullptr;
    if (cudaLaunchDeviceV2(buf, cudaStreamTailLaunch) != cudaSuccess) {
        note_launch_error(A, 5);
        return;
    }
    if (A.chain.launched) atomicAdd(A.chain.launched + 5, 1ull);
}

/* Called by the last CTA of tier A.tier: tier u (> A.tier) runs over its
 * list of `count` pairs once this grid has completed.  Tier 5 with
 * distance classes starts with the bound pass, which routes its list into
 * the classes. */
__device__ void launch_tier_on_device(const AlignLaunch& A, int u, uint32_t count)
{
    switch (u) {
    case 1: launch_on_device<T1>(A, u, count); break;
    case 2: launch_on_device<T2>(A, u, count); break;
    case 3: launch_on_device<T3>(A, u, count); break;
    case 4: launch_on_device<T4>(A, u, count); break;
    case 5:
        if (A.bound && A.chain.cls.n > 0) {
            const TierShape& b = A.chain.bound_shape;
            const uint32_t per_cta = (uint32_t)b.threads / 32u;
            const int grid = max(1, min(b.grid, (int)((count + per_cta - 1u) / per_cta)));
            tail_launch(bound_kernel, A, u, grid, b.threads, b.smem, true, b.seq_words, 0u);
        } else {
            const TierShape& sh = A.chain.shape[u];
            tail_launch(long_kernel<false, kLongThreads>, A, u, max(1, min(sh.grid, (int)count)), kLongThreads,
                        sh.smem, false, 0u, 0u);
        }
        break;
    case 6: {
        const TierShape& sh = A.chain.shape[u];
        tail_launch(long_kernel<true, kLongThreads>, A, u, max(1, min(sh.grid, (int)count)), kLongThreads, sh.smem,
                    false, 0u, 0u);
        break;
    }
    default: return;
    }
}

/* The launch that follows this one in the chain: within tier 5 with
 * classes (the bound pass, A.cls == -1, or class A.cls), the next class
 * that has work; else the next tier that has work (pairs handed on, or
 * routed to it up front). */
__device__ void launch_next(const AlignLaunch& A)
{
    if (A.tier == 5 && A.chain.cls.n > 0) {
        for (int c = A.cls + 1; c < A.chain.cls.n; ++c) {
            const uint32_t cnt = *reinterpret_cast<volatile const uint32_t*>(A.chain.cls.counts + c) +
                                 *reinterpret_cast<volatile const uint32_t*>(A.chain.cls.low_counts + c);
            if (cnt > 0u) {
                launch_class_on_device(A, c, cnt);
                return;
            }
        }
    }
    for (int u = A.tier + 1; u <= A.chain.last_tier; ++u) {
        const uint32_t cnt = *reinterpret_cast<volatile const uint32_t*>(A.chain.counts + u);
        if (cnt > 0u) {
            launch_tier_on_device(A, u, cnt);
            return;
        }
    }
}

/* End of a chained kernel: the last CTA to finish starts the next launch. */
__device__ __forceinline__ void chain_next(const AlignLaunch& A)
{
    if (!A.chain.cta_done) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        uint32_t* done = A.cls >= 0 ? A.chain.cls.cta_done + A.cls : A.chain.cta_done + A.tier;
        const unsigned t = atomicAdd(done, 1u);
        if (t == gridDim.x - 1u) {
            __threadfence();
            launch_next(A);
        }
    }
}

template <class T, bool PREDICT>
__device__ __forceinline__ void tier_body(const AlignLaunch& A, uint32_t seq_words, uint32_t gbytes)
{
    constexpr int G = T::G, J = T::J, NC = T::NC, DCAP = T::DCAP, GPW = T::GPW;
    extern __shared__ __align__(16) unsigned char smem[];

    const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5);
    const int g = lane & (G - 1), grp = lane / G;
    const unsigned gmask = (G == 32) ? kFull : (((1u << (G & 31)) - 1u) << (grp * G));
    const int slot = warp * GPW + grp;

    /* the warp's block: GPW x (sequences, chain), then GPW union regions */
    const size_t seqchain = 16u * (size_t)seq_words + T::chain_bytes;
    unsigned char* wblock = smem + (size_t)warp * GPW * gbytes;
    unsigned char* gs = wblock + (size_t)grp * seqchain;
    uint2* QP = reinterpret_cast<uint2*>(gs);
    uint2* QT = QP + seq_words;
    uint8_t* chain = gs + 16u * (size_t)seq_words;
    unsigned char* unis = wblock + (size_t)GPW * seqchain;
    unsigned char* uni = unis + (size_t)grp * (gbytes - seqchain);
    uint2* ops;
    /* last score step the backtrace store holds: a pair that would go past
     * it (never expected: a distance is at most the longest sequence, and
     * the store holds that many rows) goes on to the next tier instead */
    int store_last = DCAP;
    if constexpr (T::SMEM_OPS) {
        ops = reinterpret_cast<uint2*>(unis);
    } else {
        static_assert(T::SMEM_OPS || GPW == 1, "a store in global scratch belongs to one group");
        const TierShape& tsh = A.chain.shape[A.tier];
        const size_t gslot = (size_t)blockIdx.x * (kWarps * GPW) + (size_t)slot;
        ops = reinterpret_cast<uint2*>(A.ops_scratch + gslot * tsh.ops_group_bytes);
        store_last = min(DCAP, tsh.ops_rows);
    }
    int8_t* stage = reinterpret_cast<int8_t*>(uni);
    int* runs = reinterpret_cast<int*>(uni + round16(A.cigar_stride));

    const uint32_t count = A.work_count ? min(*A.work_count, A.n_work) : A.n_work;
    /* work stealing: each warp takes the next GPW items from the launch's
     * counter (or, without one, every gridDim-th block of items) */
    uint32_t* const work_next = A.chain.work_next ? A.chain.work_next + A.tier : nullptr;
    const uint32_t step = gridDim.x * (uint32_t)(kWarps * GPW);
    uint32_t wb = (blockIdx.x * kWarps + (uint32_t)warp) * GPW;
    if (work_next) {
        uint32_t v = 0;
        if (lane == 0) v = atomicAdd(work_next, (uint32_t)GPW);
        wb = __shfl_sync(kFull, v, 0);
    }
    for (; wb < count;) {
        const uint32_t item = wb + (uint32_t)grp;
        int state = ST_IDLE;
        uint32_t pi = 0;
        PairRef pr;
        pr.p = nullptr; pr.t = nullptr; pr.plen = 0; pr.tlen = 0;
        if (item < count) {
            pi = A.work ? A.work[item] : item;
            pr = get_pair(A.L, pi);
            const uint32_t mx = max(pr.plen, pr.tlen);
            state = !pr.in_range ? ST_RANGE
                    : PREDICT ? ST_RUN
                    : (mx > A.max_len || mx > 16u * seq_words) ? ST_TOOLONG : ST_RUN;
        }
        /* a prediction launch aligns only the first kPredictPrefix bases */
        const uint32_t lp = state == ST_RUN ? (PREDICT ? min(pr.plen, (uint32_t)kPredictPrefix) : pr.plen) : 0u;
        const uint32_t lt = state == ST_RUN ? (PREDICT ? min(pr.tlen, (uint32_t)kPredictPrefix) : pr.tlen) : 0u;
        if constexpr (G < 32) {
            /* the warp's 8 pairs in one coalesced span when they lie together */
            uint32_t* span = reinterpret_cast<uint32_t*>(smem + (size_t)(kWarps * GPW) * gbytes) + warp * kSpanWords;
            const uintptr_t a0 = load_warp_span<kSpanWords>(pr.p, lp, pr.t, lt, span, lane);
            if (a0) {
                pack_from_span<G>(span, a0, pr.p, lp, QP, g);
                pack_from_span<G>(span, a0, pr.t, lt, QT, g);
            } else {
                load_packed<G, T::RMAX>(pr.p, lp, QP, g, gmask);
                load_packed<G, T::RMAX>(pr.t, lt, QT, g, gmask);
            }
        } else {
            load_packed<G, T::RMAX>(pr.p, lp, QP, g, gmask);
            load_packed<G, T::RMAX>(pr.t, lt, QT, g, gmask);
        }
        __syncwarp();

        const int plen = (int)lp, tlen = (int)lt, kt = tlen - plen;
        int O[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) O[c] = -1;
        int D = 0;
        /* score 0: the lane of diagonal 0 extends from the origin
         * (src/kernels.cu:249-258) */
        if (state == ST_RUN && g == G / 2) O[J] = extend_lane(QP, QT, plen, tlen, 0, 0);
        {
            const bool hit = state == ST_RUN && g == G / 2 && kt == 0 && O[J] == tlen;
            if (__ballot_sync(kFull, hit) & gmask) state = ST_DONE;
        }
        int rowbase = 0;  /* first store entry of step d's row (the same for every group) */
        int rowD = 0;     /* ... of step D's row */
        for (int d = 1;; rowbase += T::row_entries(d), ++d) {
            const bool run = state == ST_RUN;
            if (!__any_sync(kFull, run)) break;
            if (d > store_last || (A.max_distance > 0 && d > A.max_distance)) {
                if (run) state = (A.max_distance > 0 && d > A.max_distance) ? ST_OVERMAX : ST_OVERFLOW;
                break;
            }
            const int clo = T::chunk_lo(d);
            int N[NC];
            /* compute (src/kernels.cu:129-152) */
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const int lo_k = G * (c - J) - G / 2;
                N[c] = -1;
                if (lo_k <= d && lo_k + G - 1 >= -d) {
                    const int upsrc = (c + 1 < NC) ? O[(c + 1 < NC) ? c + 1 : 0] : -1;
                    const int dnsrc = (c > 0) ? O[(c > 0) ? c - 1 : 0] : -1;
                    const int up = __shfl_sync(kFull, g == 0 ? upsrc : O[c], (g + 1) & (G - 1), G);
                    const int dn = __shfl_sync(kFull, g == G - 1 ? dnsrc : O[c], (g + G - 1) & (G - 1), G);
                    const int m = piggyback_max(up, O[c], dn);
                    const unsigned blo = __ballot_sync(kFull, m & 1);
                    const unsigned bhi = __ballot_sync(kFull, m & 2);
                    if (!PREDICT && lane == 0) ops[rowbase + c - clo] = make_uint2(blo, bhi);
                    const int k = lo_k + g;
                    N[c] = (run && k >= -d && k <= d) ? (m >> 2) : -1;
                }
            }
            /* extend and test the target (src/kernels.cu:173-176, 268) */
            bool hit = false;
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const int lo_k = G * (c - J) - G / 2;
                if (lo_k <= d && lo_k + G - 1 >= -d) {
                    const int k = lo_k + g;
                    if (N[c] >= 0) {
                        N[c] = extend_lane(QP, QT, plen, tlen, k, N[c]);
                        hit |= (k == kt) && (N[c] == tlen);
                    }
                    O[c] = N[c];
                }
            }
            if ((__ballot_sync(kFull, hit) & gmask) && run) {
                state = ST_DONE;
                D = d;
                rowD = rowbase;
            }
        }

        if constexpr (PREDICT) {
            if (g == 0 && item < count)
                A.pred[pi] = (uint16_t)(state == ST_DONE ? D : (state == ST_OVERFLOW ? DCAP + 1 : 0xffff));
            state = ST_IDLE;
        }
        if (state == ST_DONE) {
            /* backtrace: from (D, kt) back to (0, 0); a walk that leaves the
             * wavefront (never expected) is reported, not followed */
            int walk_ok = 1;
            if (g == 0) {
                int k = kt;
                int row = rowD;
                for (int s = D; s >= 1; --s) {
                    if (k < -s || k > s) { walk_ok = 0; break; }
                    const int idx = k + G / 2 + G * J;
                    const int op = op_of(ops[row + idx / G - T::chunk_lo(s)], grp * G + (idx & (G - 1)));
                    chain[s - 1] = (uint8_t)op;
                    k += op - 2;
                    if (s > 1) row -= T::row_entries(s - 1);
                }
                if (k != 0) walk_ok = 0;
            }
            walk_ok = __shfl_sync(gmask, walk_ok, 0, G);
            if (!walk_ok) state = ST_BADWALK;
        }
        /* the warp's store is read by every group's walk before any group's
         * replay reuses its union region */
        if constexpr (T::SMEM_OPS && GPW > 1) __syncwarp();
        if (state == ST_DONE) {
            __syncwarp(gmask);
            const int len = replay_chain<G>(QP, QT, plen, tlen, chain, D, runs, stage, A.cigar_stride,
                                            g, grp, gmask);
            if (A.cigar_stride)
                store_cigar<G>(stage, (uint32_t)len, A.cigar_stride,
                               A.cigar + (size_t)pi * A.cigar_stride, g, gmask);
            if (g == 0) {
                A.dist[pi] = D;
                if (A.status)
                    A.status[pi] = (uint32_t)len > A.cigar_stride ? (uint8_t)WFE_PAIR_CIGAR_TRUNCATED
                                                                  : (uint8_t)WFE_PAIR_OK;
            }
        } else if (state == ST_OVERFLOW && A.retry) {
            /* hand the pair to the next tier, or defer it (a chain cut short) */
            if (g == 0) {
                const uint32_t s = atomicAdd(A.retry_count, 1u);
                if (A.retry != A.chain.defer) {
                    A.retry[s] = pi;
                } else {
                    if (s < A.chain.defer_cap) A.retry[s] = A.chain.defer_base + pi;
                    note_deferred(A);
                }
                if (A.passed_total) atomicAdd(A.passed_total, 1ull);
            }
        } else if (state == ST_OVERFLOW || state == ST_OVERMAX || state == ST_TOOLONG ||
                   state == ST_BADWALK || state == ST_RANGE) {
            if (g == 0) {
                A.dist[pi] = state == ST_OVERMAX ? A.max_distance + 1 : -1;
                if (A.status)
                    A.status[pi] = state == ST_OVERMAX  ? (uint8_t)WFE_PAIR_OVER_MAX_DISTANCE
                                   : state == ST_BADWALK ? (uint8_t)WFE_PAIR_BAD_HISTORY
                                   : state == ST_RANGE   ? (uint8_t)WFE_PAIR_OUT_OF_RANGE
                                                         : (uint8_t)WFE_PAIR_TOO_LONG;
                if (A.cigar_stride) A.cigar[(size_t)pi * A.cigar_stride] = 0;
            }
        }
        __syncwarp();
        if (work_next) {
            uint32_t v = 0;
            if (lane == 0) v = atomicAdd(work_next, (uint32_t)GPW);
            wb = __shfl_sync(kFull, v, 0);
        } else {
            wb += step;
        }
    }

    /* the last CTA to finish starts the next tier that has work */
    if constexpr (!PREDICT) chain_next(A);
}

template <class T, bool PREDICT>
__global__ void __launch_bounds__(kThreads, T::MINB)
tier_kernel_bounded(const __grid_constant__ AlignLaunch A, uint32_t seq_words, uint32_t gbytes)
{
    tier_body<T, PREDICT>(A, seq_words, gbytes);
}

template <class T>
__global__ void tier_kernel(const __grid_constant__ AlignLaunch A, uint32_t seq_words, uint32_t gbytes)
{
    tier_body<T, false>(A, seq_words, gbytes);
}

/* ------------------------------------------------------------------------ */
/* Tiers 5 and 6: one CTA of NT threads (128 or 256) per pair, for distances
 * beyond the register tiers.  Step d computes the 2d+1 cells of [-d, d] in
 * 32-cell chunks, one warp per chunk (src/kernels.cu:111-180 with every
 * thread of the CTA); a barrier separates the steps and every thread then
 * tests the target cell (src/kernels.cu:268).  The wavefront's two buffers
 * live in shared memory (tier 5, distances up to kLongSmemDistance, or up
 * to the limit of the launch's distance class) or in the CTA's global
 * scratch (tier 6).  Each step also writes -1 two cells beyond its
 * range, so the next step reads the reference's sentinel there.  The 2-bit
 * backtrace store is in global scratch, row d holding ceil((2d+1)/32) 64-bit
 * entries (low and high operation bits of 32 diagonals). */

/* first entry of row d (d >= 1) of the long-tier backtrace store:
 * sum over e in [1, d-1] of ceil((2e+1)/32) = floor(e/16) + 1 */
__host__ __device__ __forceinline__ uint64_t long_row(int d)
{
    const uint64_t n = (uint64_t)(d - 1);
    const uint64_t a = n >> 4, b = n & 15u;
    return n + 8u * a * (a >= 1 ? a - 1 : 0) + a * (b + 1);
}

template <bool GLOBAL_WF, int NT>
__global__ void long_kernel(const __grid_constant__ AlignLaunch A)
{
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int kW = NT / 32;
    static_assert(kW >= 1, "at least one warp");
    const bool in_class = A.cls >= 0;
    const TierShape& sh = in_class ? A.chain.cls.shape[A.cls] : A.chain.shape[A.tier];
    const int dlim = sh.dlim;
    const int W = 2 * dlim + 5; /* entries per wavefront buffer, centre dlim + 2 */
    const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5);
    const uint32_t seq_words = sh.seq_words;
    uint2* QP = reinterpret_cast<uint2*>(smem);
    uint2* QT = QP + seq_words;
    unsigned char* slab = sh.scratch + (size_t)blockIdx.x * sh.slab;
    uint2* ops = reinterpret_cast<uint2*>(slab);
    const uint64_t ops_entries = long_row(dlim + 1);
    uint8_t* chain = slab + ops_entries * 8u;
    int* runs = reinterpret_cast<int*>(chain + ((dlim + 16) & ~15));
    int* wf;
    if constexpr (GLOBAL_WF)
        wf = runs + ((dlim + 4) & ~3);
    else
        wf = reinterpret_cast<int*>(QT + seq_words);
    int* bufA = wf + dlim + 2;     /* centred */
    int* bufB = wf + W + dlim + 2;

    /* a class list: its front part, then its back part from the end */
    const uint32_t front = A.work_count ? *A.work_count : A.n_work;
    const uint32_t count = min(front + (in_class ? A.chain.cls.low_counts[A.cls] : 0u), A.n_work);
    __shared__ uint32_t s_item;
    uint32_t* const work_next = !A.chain.work_next ? nullptr
                                : in_class ? A.chain.cls.work_next + A.cls : A.chain.work_next + A.tier;
    uint32_t item = blockIdx.x;
    if (work_next) {
        if (threadIdx.x == 0) s_item = atomicAdd(work_next, 1u);
        __syncthreads();
        item = s_item;
    }
    while (item < count) {
        const uint32_t pi = !A.work ? item : item < front ? A.work[item] : A.work[A.chain.cls.cap - 1u - (item - front)];
        const PairRef pr = get_pair(A.L, pi);
        const uint32_t mx = max(pr.plen, pr.tlen);
        int state = !pr.in_range ? ST_RANGE : (mx > A.max_len || mx > 16u * seq_words) ? ST_TOOLONG : ST_RUN;
        const int plen = state == ST_RUN ? (int)pr.plen : 0, tlen = state == ST_RUN ? (int)pr.tlen : 0;
        const int kt = tlen - plen;
        /* warps 0 and 1 load the two sequences (warp 0 both, in a one-warp CTA) */
        if (warp == 0) load_packed<32, 4>(pr.p, (uint32_t)plen, QP, lane, kFull);
        if (warp == (kW > 1 ? 1 : 0)) load_packed<32, 4>(pr.t, (uint32_t)tlen, QT, lane, kFull);
        __syncthreads();
        int D = 0;
        /* last step: the tier's limit or the caller's cap */
        const int dstop = A.max_distance > 0 ? min(dlim, A.max_distance) : dlim;
        /* Cone of the target.  Cell (d, kt) depends only on the cells
         * (s, k) with |k - kt| <= d - s, so the cells that any step up to
         * dub depends on are those with |k - kt| <= dub - s: a step computes
         * [-d, d] cut to [kt - (dub - d), kt + (dub - d)], and every cell
         * it reads lies in the previous step's cut range or on the -1
         * sentinels just beyond [-(d-1), d-1].  Each cell computed holds the
         * full recurrence's value, so the first hit at a step <= dub, and
         * the walk back from it (which stays in the cone), are exactly the
         * full recurrence's.  dub is dstop, or the pair's bound when one was
         * computed below it; a pair with no hit by a bound below dstop (the
         * bound was not one) is aligned again with dub = dstop. */
        int dub = dstop;
        if (state == ST_RUN && A.bound) {
            const int bnd = A.bound[pi];
            if (bnd >= 0 && bnd < dstop)
                dub = max(bnd, abs(kt));
            else if (bnd > dstop && A.retry && (A.max_distance <= 0 || A.max_distance > dlim))
                state = ST_OVERFLOW; /* past this tier: straight to the next */
        }
        while (state == ST_RUN) {
            /* score 0 (src/kernels.cu:249-258) */
            if (threadIdx.x == 0) {
                bufA[0] = extend_lane(QP, QT, plen, tlen, 0, 0);
                bufA[1] = bufA[-1] = bufA[2] = bufA[-2] = -1;
            }
            __syncthreads();
            int* prev = bufA;
            int* next = bufB;
            bool again = false;
            if (!(kt == 0 && prev[0] == tlen)) {
                uint2* row = ops; /* row d of the backtrace store: long_row(d), kept running */
                for (int d = 1;; ++d) {
                    if (d > dub) {
                        if (dub < dstop)
                            again = true;
                        else
                            state = (A.max_distance > 0 && d > A.max_distance) ? ST_OVERMAX : ST_OVERFLOW;
                        break;
                    }
                    const int ncell = 2 * d + 1;
                    const int nchunk = (ncell + 31) >> 5;
                    /* cells i = k + d of [ilo, ihi] */
                    const int ilo = max(0, kt - dub + 2 * d), ihi = min(2 * d, kt + dub);
                    for (int q = (ilo >> 5) + warp; q <= (ihi >> 5); q += kW) {
                        const int i = 32 * q + lane;
                        const int k = i - d;
                        const bool valid = i >= ilo && i <= ihi;
                        int m = 0;
                        if (valid) {
                            m = piggyback_max(prev[k + 1], prev[k], prev[k - 1]);
                            next[k] = extend_lane(QP, QT, plen, tlen, k, m >> 2);
                        }
                        const unsigned lo = __ballot_sync(kFull, m & 1);
                        const unsigned hi = __ballot_sync(kFull, m & 2);
                        if (lane == 0) row[q] = make_uint2(lo, hi);
                    }
                    if (threadIdx.x == 0) next[d + 1] = next[-d - 1] = next[d + 2] = next[-d - 2] = -1;
                    __syncthreads();
                    if (kt >= -d && kt <= d && next[kt] == tlen) { D = d; break; }
                    int* t = prev; prev = next; next = t;
                    row += nchunk;
                }
            }
            if (!again) {
                if (state == ST_RUN) state = ST_DONE;
                break;
            }
            /* every thread has read the last step's target cell before
             * thread 0 rewrites the buffers */
            __syncthreads();
            dub = dstop;
        }
        if (state == ST_DONE && warp == 0) {
            /* backtrace, 32 rows per round: lane r fetches row s-r's entries
             * around the walk (it moves 0-2 positions down per row), then
             * all lanes walk them through shuffles */
            int p = kt + D;
            int s = D;
            bool ok = true;
            while (s >= 1 && ok) {
                const int ctop = p >> 5;
                const int sr = s - lane;
                uint2 e0 = make_uint2(0, 0), e1 = e0, e2 = e0;
                if (sr >= 1) {
                    const uint2* rw = ops + long_row(sr);
                    const int last = (2 * sr) >> 5;
                    if (ctop - 2 >= 0 && ctop - 2 <= last) e0 = rw[ctop - 2];
                    if (ctop - 1 >= 0 && ctop - 1 <= last) e1 = rw[ctop - 1];
                    if (ctop <= last) e2 = rw[ctop];
                }
                const int steps = min(32, s);
                for (int r = 0; r < steps; ++r) {
                    const int sel = (p >> 5) - (ctop - 2);
                    const uint2 mine = sel == 0 ? e0 : (sel == 1 ? e1 : e2);
                    const unsigned lo = __shfl_sync(kFull, mine.x, r);
                    const unsigned hi = __shfl_sync(kFull, mine.y, r);
                    const int bit = p & 31;
                    const int op = (int)(((lo >> bit) & 1u) | (((hi >> bit) & 1u) << 1));
                    const int row = s - r;
                    if (op == 0 || sel < 0 || sel > 2 || p < 0 || p > 2 * row) { ok = false; break; }
                    if (lane == 0) chain[row - 1] = (uint8_t)op;
                    p += op - 3;
                }
                s -= steps;
            }
            if (ok && p != 0) ok = false;
            if (!ok) state = ST_BADWALK;
            __syncwarp();
            if (state == ST_DONE) {
                int8_t* dst = A.cigar_stride ? A.cigar + (size_t)pi * A.cigar_stride : nullptr;
                const int len = replay_chain<32>(QP, QT, plen, tlen, chain, D, runs, dst, dst ? A.cigar_stride : 0u,
                                                 lane, 0, kFull);
                if (lane == 0) {
                    if (dst && (uint32_t)len < A.cigar_stride) dst[len] = 0;
                    A.dist[pi] = D;
                    if (A.status)
                        A.status[pi] = (uint32_t)len > A.cigar_stride ? (uint8_t)WFE_PAIR_CIGAR_TRUNCATED
                                                                      : (uint8_t)WFE_PAIR_OK;
                }
            }
        }
        if (threadIdx.x == 0 && state != ST_DONE && state != ST_IDLE) {
            if (state == ST_OVERFLOW && A.retry) {
                const uint32_t s = atomicAdd(A.retry_count, 1u);
                A.retry[s] = pi;
                if (A.passed_total) atomicAdd(A.passed_total, 1ull);
            } else {
                A.dist[pi] = state == ST_OVERMAX ? A.max_distance + 1 : -1;
                if (A.status)
                    A.status[pi] = state == ST_OVERMAX  ? (uint8_t)WFE_PAIR_OVER_MAX_DISTANCE
                                   : state == ST_BADWALK ? (uint8_t)WFE_PAIR_BAD_HISTORY
                                   : state == ST_RANGE   ? (uint8_t)WFE_PAIR_OUT_OF_RANGE
                                                         : (uint8_t)WFE_PAIR_TOO_LONG;
                if (A.cigar_stride) A.cigar[(size_t)pi * A.cigar_stride] = 0;
            }
        }
        __syncthreads();
        if (work_next) {
            if (threadIdx.x == 0) s_item = atomicAdd(work_next, 1u);
            __syncthreads();
            item = s_item;
        } else {
            item += gridDim.x;
        }
    }

    chain_next(A);
}

/* ------------------------------------------------------------------------ */
/* Distance bounds for the CTA-per-pair tiers, one warp per pair.  The warp
 * runs the recurrence of the tiers restricted to a band of 32 diagonals
 * (lane l: diagonal b + l) that follows the cell furthest along its
 * antidiagonal (largest min(h, t_len) + min(v, p_len): offsets the
 * recurrence carries past a sequence's end count that end, so that the band
 * turns towards the target diagonal once one sequence is consumed): one
 * score step after it is seen the band moves one
 * diagonal towards that cell when it lies outside lanes 15-16.  Cells
 * outside the band count as the -1 sentinel, and a cell whose offset would
 * put its pattern position below 0 is dropped.  Every offset the band
 * computes is reached by some path of cost d and is at most the full
 * recurrence's offset (the three-way maximum and the extend are both
 * monotone), so the first step at which the band's cell (d, kt) reaches the
 * end is an upper bound on the edit distance: bound[pi] is that step, or -1
 * if the band has not reached it after max(p_len, t_len) + 1 steps.  On the
 * synthetic workloads the bound equals the distance for all but a handful
 * of pairs; the long tiers then compute only the target's cone (about half
 * of the cells), and a bound that is not one costs a second pass, never a
 * wrong result.  Each warp keeps its pair as plain packed words (16 bases
 * per 32-bit word, src/kernels.cu:313-394) in shared memory, followed by
 * zero words. */

/* 16-base window of plain packed words starting at base v (words w and
 * w + 1 of v's word w) */
__device__ __forceinline__ uint32_t window_words(const uint32_t* W, int v)
{
    const int w = v >> 4;
    return __funnelshift_l(W[w + 1], W[w], (uint32_t)(v & 15) << 1);
}

/* extend_lane over plain packed words */
__device__ __forceinline__ int extend_words(const uint32_t* P, const uint32_t* T, int plen, int tlen, int k, int off)
{
    int v = off - k, h = off;
    while ((unsigned)v < (unsigned)plen && (unsigned)h < (unsigned)tlen) {
        const uint32_t x = window_words(P, v) ^ window_words(T, h);
        int n = __clz(x) >> 1;
        n = min(n, min(plen - v, tlen - h));
        v += n;
        h += n;
        if (n < 16) break;
    }
    return h;
}

/* words per sequence in the bound kernel's shared memory: the packed words
 * and at least one zero word after them, rounded to 16 bytes */
__host__ __device__ __forceinline__ uint32_t bound_words(uint32_t seq_words) { return (seq_words + 4u) & ~3u; }

__device__ __forceinline__ void bound_body(const AlignLaunch& A, uint32_t seq_words)
{
    extern __shared__ __align__(16) unsigned char smem[];
    /* tier 5 with classes: route every pair to a class, then start them */
    const bool route = A.tier == 5 && A.chain.cls.n > 0;
    constexpr int kW = kLongThreads / 32;
    constexpr int kHalf = 15;
    const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5);
    const uint32_t bw = bound_words(seq_words);
    uint32_t* WP = reinterpret_cast<uint32_t*>(smem) + (size_t)warp * 2u * bw;
    uint32_t* WT = WP + bw;
    const uint32_t count = A.work_count ? min(*A.work_count, A.n_work) : A.n_work;
    for (uint32_t item = blockIdx.x * kW + (uint32_t)warp; item < count; item += gridDim.x * kW) {
        const uint32_t pi = A.work ? A.work[item] : item;
        const PairRef pr = get_pair(A.L, pi);
        const uint32_t mx = max(pr.plen, pr.tlen);
        int bound = -1;
        int need = INT_MAX; /* steps the pair's class must hold */
        if (pr.in_range && mx <= A.max_len && mx <= 16u * seq_words) {
            const int plen = (int)pr.plen, tlen = (int)pr.tlen, kt = tlen - plen;
            /* words 0..bw-1 of each sequence: packed_word gives 0 past the end */
            for (uint32_t w0 = 0; w0 < bw; w0 += 32u) {
                const uint32_t wp = packed_word<32>(pr.p, pr.plen, w0, lane, kFull);
                const uint32_t wt = packed_word<32>(pr.t, pr.tlen, w0, lane, kFull);
                if (w0 + (uint32_t)lane < bw) {
                    WP[w0 + lane] = wp;
                    WT[w0 + lane] = wt;
                }
            }
            __syncwarp();
            int b = -kHalf;
            int O = lane == kHalf ? extend_words(WP, WT, plen, tlen, 0, 0) : -1;
            if (__ballot_sync(kFull, lane == kHalf && kt == 0 && O == tlen)) bound = 0;
            const int limit = (int)mx + 1;
            int delta_next = 0;
            for (int d = 1; bound < 0 && d <= limit; ++d) {
                /* The band's leader after step d-1 -- the cell that has
                 * consumed the most bases of both sequences (offsets past an
                 * end count the end) -- moves the band of step d+1: the
                 * reduction then runs beside step d instead of before it. */
                const int delta = delta_next;
                const int prog = O >= 0 ? min(O, tlen) + min(O - (b + lane), plen) : INT_MIN;
                const int best = __reduce_max_sync(kFull, prog);
                const int lead = __ffs((int)__ballot_sync(kFull, prog == best)) - 1 - delta;
                delta_next = (lead > kHalf + 1) - (lead < kHalf);
                b += delta;
                const int k = b + lane;
                /* diagonals k+1, k, k-1 of step d-1 were on lanes s+1, s, s-1 */
                const int s = lane + delta;
                int up = __shfl_sync(kFull, O, (s + 1) & 31);
                int self = __shfl_sync(kFull, O, s & 31);
                int dn = __shfl_sync(kFull, O, (s - 1) & 31);
                if ((unsigned)(s + 1) > 31u) up = -1;
                if ((unsigned)s > 31u) self = -1;
                if ((unsigned)(s - 1) > 31u) dn = -1;
                int N = -1;
                if (k >= -d && k <= d) {
                    const int off = piggyback_max(up, self, dn) >> 2;
                    if (off >= k) N = extend_words(WP, WT, plen, tlen, k, off);
                }
                O = N;
                if (__ballot_sync(kFull, k == kt && N == tlen)) bound = d;
            }
            if (bound >= 0) need = max(bound, abs(kt));
            if (A.max_distance > 0) need = min(need, A.max_distance);
        }
        if (lane == 0) {
            A.bound[pi] = bound;
            if (route) {
                const LongClasses& C = A.chain.cls;
                const int top = C.shape[C.n - 1].dlim;
                if (bound > top && need > top && A.retry) {
                    /* past tier 5 (with no cap below its limit): straight on */
                    A.retry[atomicAdd(A.retry_count, 1u)] = pi;
                    if (A.passed_total) atomicAdd(A.passed_total, 1ull);
                } else {
                    int c = 0;
                    while (c + 1 < C.n && C.shape[c].dlim < need) ++c;
                    const int below = c > 0 ? C.shape[c - 1].dlim : 0;
                    if (2 * need >= below + C.shape[c].dlim)
                        C.list[c][atomicAdd(C.counts + c, 1u)] = pi;
                    else
                        C.list[c][C.cap - 1u - atomicAdd(C.low_counts + c, 1u)] = pi;
                }
            }
        }
        __syncwarp();
    }
    if (route) chain_next(A);
}

/* The bound pass in two forms with one body, as the tier kernels: launched
 * from the host with launch bounds for 6 resident CTAs per SM, and from the
 * device (a chain entering tier 5) without. */
__global__ void __launch_bounds__(kLongThreads, 6)
bound_kernel_host(const __grid_constant__ AlignLaunch A, uint32_t seq_words, uint32_t /* unused */)
{
    bound_body(A, seq_words);
}

__global__ void bound_kernel(const __grid_constant__ AlignLaunch A, uint32_t seq_words, uint32_t /* unused */)
{
    bound_body(A, seq_words);
}

const TierInfo kTiers[kNumTiers] = {
    {T0::G, T0::J, T0::DCAP, T0::SMEM_OPS},
    {T1::G, T1::J, T1::DCAP, T1::SMEM_OPS},
    {T2::G, T2::J, T2::DCAP, T2::SMEM_OPS},
    {T3::G, T3::J, T3::DCAP, T3::SMEM_OPS},
    {T4::G, T4::J, T4::DCAP, T4::SMEM_OPS},
    {kLongThreads, 0, kLongSmemDistance, false},
    {kLongThreads, 0, 0x7fffffff, false},
};

/* The kernel a tier's host launches use (see tier_kernel_bounded). */
template <class T>
const void* host_kernel()
{
    if constexpr (T::G == 32) return (const void*)tier_kernel<T>;
    else return (const void*)tier_kernel_bounded<T, false>;
}

template <class T>
TierShape shape_of(uint32_t max_len, uint32_t cigar_stride, int sm_count)
{
    TierShape sh{};
    const size_t smem = cta_smem_bytes<T>(max_len, cigar_stride);
    if (smem > 227u * 1024u) return sh;
    const void* fn = host_kernel<T>();
    if (allow_smem(fn, smem) != cudaSuccess)
        return sh;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kThreads, smem) != cudaSuccess)
        return sh;
    sh.grid = std::max(1, nb) * sm_count;
    sh.smem = (uint32_t)smem;
    sh.seq_words = seq_words_for(max_len);
    sh.gbytes = (uint32_t)group_smem_bytes<T>(max_len, cigar_stride);
    if (!T::SMEM_OPS) {
        sh.ops_group_bytes = (uint32_t)T::store_bytes(max_len);
        sh.ops_rows = T::store_rows(max_len);
    }
    return sh;
}

template <class T>
int grid_of(uint32_t max_len, uint32_t cigar_stride, int sm_count)
{
    return shape_of<T>(max_len, cigar_stride, sm_count).grid;
}

template <class T>
cudaError_t launch(const AlignLaunch& a, int grid, cudaStream_t s)
{
    const uint32_t sw = seq_words_for(a.max_len);
    const size_t gb = group_smem_bytes<T>(a.max_len, a.cigar_stride);
    const size_t smem = cta_smem_bytes<T>(a.max_len, a.cigar_stride);
    if (smem > 227u * 1024u) return cudaErrorInvalidValue;
    if (!T::SMEM_OPS) {
        const TierShape& tsh = a.chain.shape[a.tier];
        if (tsh.ops_group_bytes == 0 || tsh.ops_rows <= 0 ||
            a.ops_scratch_bytes < (size_t)tsh.ops_group_bytes * (size_t)grid * (kWarps * T::GPW))
            return cudaErrorInvalidValue;
    }
    cudaError_t e = allow_smem(host_kernel<T>(), smem);
    if (e != cudaSuccess) return e;
    if constexpr (T::G == 32)
        tier_kernel<T><<<grid, kThreads, smem, s>>>(a, sw, (uint32_t)gb);
    else
        tier_kernel_bounded<T><<<grid, kThreads, smem, s>>>(a, sw, (uint32_t)gb);
    return cudaGetLastError();
}

/* ------------------------------------------------------------------------ */
/* Routing: one thread per pair.  The length bucket is the first whose
 * max_len holds max(p_len, t_len).  The tier is the bucket's first tier, or,
 * with predictions, the first tier whose distance limit covers the
 * prediction: the prefix distance scaled by max length / prefix length,
 * plus 25 % and 2, up to tier 5 (a prediction only chooses where a pair
 * starts; a pair above its tier's limit still moves up).  Appends are warp-aggregated: one
 * atomic per (bucket, tier) present in the warp. */
__global__ void __launch_bounds__(256) classify_kernel(Layout L, uint32_t n, Buckets B)
{
    const int lane = (int)(threadIdx.x & 31u);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lim = (n + 31u) & ~31u; /* whole warps iterate together */
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < lim; i += stride) {
        int key = -1;
        if (i < n) {
            const PairRef pr = get_pair(L, i);
            const uint32_t len = max(pr.plen, pr.tlen);
            int b = B.n - 1;
            for (int j = 0; j < B.n; ++j)
                if (len <= B.max_len[j]) { b = j; break; }
            int t = B.first_tier[b];
            if (B.pred && len > 0) {
                const uint32_t pref = min(max(pr.plen, pr.tlen), (uint32_t)kPredictPrefix);
                const uint32_t pd = B.pred[i];
                if (pd != 0xffff) {
                    const float scale = (float)len / (float)max(pref, 1u);
                    const float est = ((float)pd + 1.0f) * scale * 1.25f + 2.0f;
                    /* never past tier 5: the global-wavefront tier only
                     * takes pairs that tier 5 hands on */
                    const int top = min(B.last_tier[b], 5);
                    while (t < top && (float)B.dcap[t] < est) ++t;
                }
            }
            key = b * kListsPerBucket + t;
        }
        const unsigned same = __match_any_sync(kFull, key);
        const int leader = __ffs((int)same) - 1;
        uint32_t base = 0;
        if (key >= 0 && lane == leader) {
            const int b = key / kListsPerBucket, t = key % kListsPerBucket;
            base = atomicAdd(B.counts + (size_t)b * B.count_stride + t, (uint32_t)__popc(same));
            if (B.totals) atomicAdd(B.totals + b, (unsigned long long)__popc(same));
        }
        base = __shfl_sync(kFull, base, leader);
        if (key >= 0) {
            const uint32_t rank = (uint32_t)__popc(same & ((1u << lane) - 1u));
            B.lists[(size_t)key * B.stride + base + rank] = i;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Standalone packer (src/kernels.cu:313-394): one thread per kPackWords
 * output words.  Thread t writes words kPackWords*j .. kPackWords*j +
 * kPackWords-1 of sequence t / ceil(wps/kPackWords) (pattern of pair i at
 * 2i, text at 2i+1), j = t % ceil(wps/kPackWords), from the kPackWords+1
 * aligned 16-byte blocks that hold their bases, each packed once; the
 * threads of a sequence read its blocks and descriptor through L1, so the
 * ASCII is read from DRAM about once and the words are written with
 * coalesced stores.  For 2 n ceil(wps/kPackWords) < 2^32. */
constexpr int kPackWords = 4;
__global__ void __launch_bounds__(256)
pack_words_kernel(Layout L, uint32_t n, uint32_t* out, uint32_t wps)
{
    const uint32_t gps = (wps + kPackWords - 1u) / kPackWords;
    const uint32_t total = 2u * n * gps;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const uint32_t sidx = t / gps, w0 = kPackWords * (t - sidx * gps);
        const PairRef pr = get_pair(L, sidx >> 1);
        const char* s = (sidx & 1u) ? pr.t : pr.p;
        const uint32_t len = (sidx & 1u) ? pr.tlen : pr.plen;
        const uint32_t nw = (len + 15u) >> 4;
        const uintptr_t a = reinterpret_cast<uintptr_t>(s);
        const uint32_t sh = (uint32_t)(a & 15u);
        const uint4* base = reinterpret_cast<const uint4*>(a - sh);
        const uint32_t nblk = (sh + len + 15u) >> 4;
        uint4 v[kPackWords + 1];
#pragma unroll
        for (int r = 0; r <= kPackWords; ++r) v[r] = w0 + r < nblk ? __ldg(base + w0 + r) : make_uint4(0u, 0u, 0u, 0u);
        uint32_t x[kPackWords + 1];
#pragma unroll
        for (int r = 0; r <= kPackWords; ++r) x[r] = pack16(v[r]);
        uint32_t* dst = out + (size_t)sidx * wps;
#pragma unroll
        for (int r = 0; r < kPackWords; ++r) {
            const uint32_t w = w0 + (uint32_t)r;
            if (w >= wps) break;
            uint32_t W = 0;
            if (w < nw) {
                W = sh ? __funnelshift_l(x[r + 1], x[r], 2u * sh) : x[r];
                const uint32_t rem = len - 16u * w;
                if (rem < 16u) W &= ~0u << (2u * (16u - rem));
            }
            dst[w] = W;
        }
    }
}

/* The same words, one warp per sequence: for outputs of 2^32 words or more. */
__global__ void __launch_bounds__(256)
pack_kernel(Layout L, uint32_t n, uint32_t* out, uint32_t wps)
{
    const int lane = (int)(threadIdx.x & 31u);
    const uint32_t wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarp = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t sidx = wid; sidx < 2u * n; sidx += nwarp) {
        const PairRef pr = get_pair(L, sidx >> 1);
        const char* s = (sidx & 1u) ? pr.t : pr.p;
        const uint32_t len = (sidx & 1u) ? pr.tlen : pr.plen;
        uint32_t* dst = out + (size_t)sidx * wps;
        const uint32_t nw = (len + 15u) >> 4;
        for (uint32_t w0 = 0; w0 < wps; w0 += 32u) {
            uint32_t W = 0;
            if (w0 < nw) W = packed_word<32>(s, len, w0, lane, kFull);
            if (w0 + (uint32_t)lane < wps) dst[w0 + lane] = W;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* CIGARs from 128-bit histories (src/kernels.cu:397-625): one group of 4
 * lanes per pair, 8 pairs per warp (a history holds at most 63 operations,
 * and 4 lanes extend 64 bases per trip). */
constexpr int kHG = 4;

__global__ void __launch_bounds__(kThreads)
history_cigar_kernel(Layout L, uint32_t n, uint32_t max_len, const int32_t* dist,
                     const uint64_t* hist, int8_t* cigar, uint32_t stride, uint8_t* status,
                     uint32_t seq_words, uint32_t gbytes)
{
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int G = kHG, GPW = 32 / G;
    const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5);
    const int g = lane & (G - 1), grp = lane / G;
    const unsigned gmask = ((1u << G) - 1u) << (grp * G);
    unsigned char* gs = smem + (size_t)(warp * GPW + grp) * gbytes;
    uint2* QP = reinterpret_cast<uint2*>(gs);
    uint2* QT = QP + seq_words;
    uint8_t* chain = gs + 16u * (size_t)seq_words;
    int* runs = reinterpret_cast<int*>(chain + 64);
    int8_t* stage = reinterpret_cast<int8_t*>(chain + 64 + 256);
    const uint32_t step = gridDim.x * (uint32_t)(kWarps * GPW);
    for (uint32_t wb = (blockIdx.x * kWarps + (uint32_t)warp) * GPW; wb < n; wb += step) {
        const uint32_t pi = wb + (uint32_t)grp;
        if (pi >= n) continue; /* whole group leaves together */
        const PairRef pr = get_pair(L, pi);
        const int D = dist[pi];
        const bool toolong = max(pr.plen, pr.tlen) > max_len || max(pr.plen, pr.tlen) > 16u * seq_words;
        if (toolong || D < 0 || D > 63) {
            if (g == 0) {
                if (status)
                    status[pi] = toolong ? (uint8_t)WFE_PAIR_TOO_LONG : (uint8_t)WFE_PAIR_OVER_MAX_DISTANCE;
                if (stride) cigar[(size_t)pi * stride] = 0;
            }
            continue;
        }
        load_packed<G, (G == 4 ? 5 : 3)>(pr.p, pr.plen, QP, g, gmask);
        load_packed<G, (G == 4 ? 5 : 3)>(pr.t, pr.tlen, QT, g, gmask);
        const uint64_t w0 = hist[2u * pi], w1 = hist[2u * pi + 1u];
        for (int d = g; d < D; d += G)
            chain[d] = (uint8_t)(((d < 32 ? w0 : w1) >> (2 * (d & 31))) & 3u);
        __syncwarp(gmask);
        int len = replay_chain<G>(QP, QT, (int)pr.plen, (int)pr.tlen, chain, D, runs, stage, stride, g,
                                  grp, gmask);
        const bool bad = len < 0;
        if (bad) len = -1 - len;
        if (stride) store_cigar<G>(stage, (uint32_t)len, stride, cigar + (size_t)pi * stride, g, gmask);
        if (g == 0 && status)
            status[pi] = bad ? (uint8_t)WFE_PAIR_BAD_HISTORY
                             : ((uint32_t)len > stride ? (uint8_t)WFE_PAIR_CIGAR_TRUNCATED
                                                       : (uint8_t)WFE_PAIR_OK);
        __syncwarp(gmask);
    }
}

}  // namespace

const TierInfo& tier_info(int t) { return kTiers[t]; }

size_t tier_scratch_bytes(int tier, int grid, uint32_t max_len)
{
    switch (tier) {
    case 2: return T2::store_bytes(max_len) * (size_t)grid * (kWarps * T2::GPW);
    case 3: return T3::store_bytes(max_len) * (size_t)grid * (kWarps * T3::GPW);
    case 4: return T4::store_bytes(max_len) * (size_t)grid * (kWarps * T4::GPW);
    default: return 0;
    }
}

uint64_t long_slab_bytes(int dlim, bool global_wavefront)
{
    uint64_t b = long_row(dlim + 1) * 8u;              /* backtrace store */
    b += (uint64_t)((dlim + 16) & ~15);                 /* chain */
    b += 4u * (uint64_t)((dlim + 4) & ~3);              /* runs */
    if (global_wavefront) b += 8u * (uint64_t)(2 * dlim + 5); /* two wavefront buffers */
    return (b + 255u) & ~uint64_t(255);
}

namespace {

/* Shape of a CTA-per-pair launch of NT threads for sequences up to max_len
 * and distances up to dlim (global wavefront: GWF). */
template <bool GWF, int NT>
TierShape long_shape_for(uint32_t max_len, int dlim, int sm_count)
{
    TierShape sh{};
    const uint32_t sw = seq_words_for(max_len);
    const size_t smem = 16u * (size_t)sw + (GWF ? 0u : 8u * (size_t)(2 * dlim + 5));
    if (smem > 227u * 1024u) return sh;
    if (allow_smem((const void*)long_kernel<GWF, NT>, smem) != cudaSuccess)
        return sh;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, long_kernel<GWF, NT>, NT, smem) != cudaSuccess)
        return sh;
    sh.grid = std::max(1, nb) * sm_count;
    sh.smem = (uint32_t)smem;
    sh.seq_words = sw;
    sh.dlim = dlim;
    sh.slab = long_slab_bytes(dlim, GWF);
    sh.threads = NT;
    return sh;
}

template <bool GWF>
TierShape long_shape_of(uint32_t max_len, int sm_count)
{
    const int dlim = GWF ? (int)max_len : (int)std::min<uint32_t>(max_len, kLongSmemDistance);
    return long_shape_for<GWF, kLongThreads>(max_len, dlim, sm_count);
}

template <bool GWF>
cudaError_t launch_long(const AlignLaunch& a, int grid, cudaStream_t s)
{
    const TierShape& sh = a.chain.shape[a.tier];
    if (!sh.scratch || sh.smem == 0) return cudaErrorInvalidValue;
    cudaError_t e = allow_smem((const void*)long_kernel<GWF, kLongThreads>, sh.smem);
    if (e != cudaSuccess) return e;
    long_kernel<GWF, kLongThreads><<<grid, kLongThreads, sh.smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

namespace {

TierShape compute_tier_shape(int tier, uint32_t max_len, uint32_t cigar_stride, int sm_count)
{
    switch (tier) {
    case 0: return shape_of<T0>(max_len, cigar_stride, sm_count);
    case 1: return shape_of<T1>(max_len, cigar_stride, sm_count);
    case 2: return shape_of<T2>(max_len, cigar_stride, sm_count);
    case 3: return shape_of<T3>(max_len, cigar_stride, sm_count);
    case 4: return shape_of<T4>(max_len, cigar_stride, sm_count);
    case 5: return long_shape_of<false>(max_len, sm_count);
    case 6: return max_len > (uint32_t)kLongSmemDistance ? long_shape_of<true>(max_len, sm_count) : TierShape{};
    default: return TierShape{};
    }
}

}  // namespace

/* Shapes depend only on the device and the arguments; each occupancy query
 * costs tens of microseconds the first time, and a context asks for every
 * tier's shape at creation and again for its first bucket, so results are
 * kept per device for the life of the process. */
TierShape tier_shape(int tier, uint32_t max_len, uint32_t cigar_stride, int sm_count)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TierShape{};
    static std::mutex mu;
    static std::map<std::tuple<int, int, uint32_t, uint32_t, int>, TierShape> known;
    const auto key = std::make_tuple(dev, tier, max_len, cigar_stride, sm_count);
    std::lock_guard<std::mutex> lock(mu);
    const auto it = known.find(key);
    if (it != known.end()) return it->second;
    const TierShape sh = compute_tier_shape(tier, max_len, cigar_stride, sm_count);
    known.emplace(key, sh);
    return sh;
}

int tier_grid(int tier, uint32_t max_len, uint32_t cigar_stride, int sm_count)
{
    return tier_shape(tier, max_len, cigar_stride, sm_count).grid;
}

/* cached per (device, max_len, SMs), as tier_shape */
TierShape bound_shape(uint32_t max_len, int sm_count)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TierShape{};
    static std::mutex mu;
    static std::map<std::tuple<int, uint32_t, int>, TierShape> known;
    const auto key = std::make_tuple(dev, max_len, sm_count);
    std::lock_guard<std::mutex> lock(mu);
    const auto it = known.find(key);
    if (it != known.end()) return it->second;
    TierShape sh{};
    const uint32_t sw = seq_words_for(max_len);
    const size_t smem = (size_t)(kLongThreads / 32) * 2u * bound_words(sw) * sizeof(uint32_t);
    int nb = 0;
    if (smem <= 227u * 1024u && allow_smem((const void*)bound_kernel, smem) == cudaSuccess &&
        allow_smem((const void*)bound_kernel_host, smem) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, bound_kernel_host, kLongThreads, smem) == cudaSuccess) {
        sh.grid = std::max(1, nb) * sm_count;
        sh.smem = (uint32_t)smem;
        sh.seq_words = sw;
        sh.threads = kLongThreads;
    }
    cudaGetLastError();
    known.emplace(key, sh);
    return sh;
}

cudaError_t launch_bound(const AlignLaunch& a, cudaStream_t s)
{
    const TierShape& sh = a.chain.bound_shape;
    if (sh.grid <= 0 || !a.bound || sh.seq_words != seq_words_for(a.max_len)) return cudaErrorInvalidValue;
    cudaError_t e = allow_smem((const void*)bound_kernel_host, sh.smem);
    if (e != cudaSuccess) return e;
    const uint32_t per_cta = (uint32_t)sh.threads / 32u;
    int grid = sh.grid;
    if (!a.work_count) grid = (int)std::min<uint64_t>((uint64_t)grid, ((uint64_t)a.n_work + per_cta - 1) / per_cta);
    bound_kernel_host<<<std::max(grid, 1), sh.threads, sh.smem, s>>>(a, sh.seq_words, 0u);
    return cudaGetLastError();
}

namespace {

LongClasses compute_long_classes(uint32_t max_len, int sm_count, uint64_t scratch_bytes)
{
    LongClasses C{};
    const int top = (int)std::min<uint32_t>(max_len, kLongSmemDistance);
    int lim[kLongClasses];
    int n = 0;
    for (int c = 0; c < kLongClasses - 1; ++c)
        if (2 * kLongClassLimit[c] < top) lim[n++] = kLongClassLimit[c];
    lim[n++] = top;
    for (int c = 0; c < n; ++c) {
        TierShape sh = lim[c] <= kLongTinyDistance    ? long_shape_for<false, kLongTinyThreads>(max_len, lim[c], sm_count)
                     : lim[c] <= kLongSmallDistance ? long_shape_for<false, kLongSmallThreads>(max_len, lim[c], sm_count)
                                                    : long_shape_for<false, kLongThreads>(max_len, lim[c], sm_count);
        if (sh.grid <= 0) return LongClasses{};
        /* the class's slabs share tier 5's scratch: one class runs at a time */
        const uint64_t fit = sh.slab ? scratch_bytes / sh.slab : 0u;
        if (fit == 0) return LongClasses{};
        sh.grid = (int)std::min<uint64_t>((uint64_t)sh.grid, fit);
        C.shape[c] = sh;
    }
    C.n = n;
    return C;
}

}  // namespace

/* cached per (device, max_len, SMs, scratch), as tier_shape */
LongClasses long_classes(uint32_t max_len, int sm_count, uint64_t scratch_bytes)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return LongClasses{};
    static std::mutex mu;
    static std::map<std::tuple<int, uint32_t, int, uint64_t>, LongClasses> known;
    const auto key = std::make_tuple(dev, max_len, sm_count, scratch_bytes);
    std::lock_guard<std::mutex> lock(mu);
    const auto it = known.find(key);
    if (it != known.end()) return it->second;
    const LongClasses C = compute_long_classes(max_len, sm_count, scratch_bytes);
    cudaGetLastError();
    known.emplace(key, C);
    return C;
}

cudaError_t launch_tier(int tier, const AlignLaunch& a, int grid, cudaStream_t s)
{
    if (grid <= 0) return cudaErrorInvalidConfiguration;
    switch (tier) {
    case 0: return launch<T0>(a, grid, s);
    case 1: return launch<T1>(a, grid, s);
    case 2: return launch<T2>(a, grid, s);
    case 3: return launch<T3>(a, grid, s);
    case 4: return launch<T4>(a, grid, s);
    case 5: return launch_long<false>(a, grid, s);
    case 6: return launch_long<true>(a, grid, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_classify(const Layout& L, uint32_t n, const Buckets& B, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, 4096u);
    classify_kernel<<<blocks, 256, 0, s>>>(L, n, B);
    return cudaGetLastError();
}

cudaError_t launch_predict(const Layout& L, uint32_t n, uint32_t max_len, uint16_t* pred, int grid, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const uint32_t plen = std::min<uint32_t>(max_len, (uint32_t)kPredictPrefix);
    const size_t gb = group_smem_bytes<T0>(plen, 0);
    const size_t smem = cta_smem_bytes<T0>(plen, 0);
    cudaError_t e = allow_smem((const void*)tier_kernel_bounded<T0, true>, smem);
    if (e != cudaSuccess) return e;
    AlignLaunch a{};
    a.L = L;
    a.n_work = n;
    a.max_len = max_len;
    a.pred = pred;
    a.tier = 0;
    const uint32_t per_cta = kWarps * T0::GPW;
    grid = std::max(1, std::min(grid, (int)((n + per_cta - 1) / per_cta)));
    tier_kernel_bounded<T0, true><<<grid, kThreads, smem, s>>>(a, seq_words_for(plen), (uint32_t)gb);
    return cudaGetLastError();
}

cudaError_t launch_pack(const Layout& L, uint32_t n, uint32_t* words, uint32_t wps, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const uint64_t total = 2ull * n * ((wps + kPackWords - 1u) / kPackWords);
    if (total < (1ull << 32)) {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                      cudaSuccess)
            return cudaErrorInvalidValue;
        /* 8 blocks of 256 per SM, each thread looping over words */
        const uint32_t blocks = (uint32_t)std::max<uint64_t>(
            1u, std::min<uint64_t>((total + 255u) / 256u, (uint64_t)sms * 8u));
        pack_words_kernel<<<blocks, 256, 0, s>>>(L, n, words, wps);
        return cudaGetLastError();
    }
    const uint32_t warps = 2u * n;
    const uint32_t blocks = std::min<uint32_t>((warps + 7u) / 8u, 65535u * 16u);
    pack_kernel<<<blocks, 256, 0, s>>>(L, n, words, wps);
    return cudaGetLastError();
}

cudaError_t launch_cigar_from_history(const Layout& L, uint32_t n, uint32_t max_len,
                                      const int32_t* dist, const uint64_t* hist, int8_t* cigar,
                                      uint32_t stride, uint8_t* status, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const uint32_t sw = seq_words_for(max_len);
    const size_t gb = 16u * (size_t)sw + 64u + 256u + round16(stride);
    const size_t smem = gb * (size_t)(kWarps * (32 / kHG));
    if (smem > 227u * 1024u) return cudaErrorInvalidValue;
    cudaError_t e = allow_smem((const void*)history_cigar_kernel, smem);
    if (e != cudaSuccess) return e;
    const uint32_t per_cta = kWarps * (32 / kHG);
    const uint32_t blocks = std::min<uint32_t>((n + per_cta - 1u) / per_cta, 1u << 20);
    history_cigar_kernel<<<blocks, kThreads, smem, s>>>(L, n, max_len, dist, hist, cigar, stride, status,
                                                        sw, (uint32_t)gb);
    return cudaGetLastError();
}

}  // namespace wfe

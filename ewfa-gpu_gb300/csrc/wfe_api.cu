/*
 * wfe_api.cu -- the C ABI of libwfe (include/wfe.h): contexts, the batch
 * pipeline of the host-buffer calls, and the device-buffer calls.
 *
 * The reference's batch loop (src/wavefront.cu:127-330) runs, per host
 * thread, one batch at a time: H2D of the next batch on a second stream
 * overlaps the current kernels, then a synchronous D2H of the CIGARs.  Here
 * a context keeps two pipeline stages, each with its own stream and device
 * buffers, so the copies in and out of one batch overlap the kernels of the
 * other; the tier chain of each batch runs on its stage's stream with no host
 * synchronisation between kernels.
 */
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <thread>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "wfe.h"
#include "wfe_internal.h"
#include "wfe_kernels.cuh"

using namespace wfe;

namespace {

constexpr int kStages = 2;

struct Stage {
    cudaStream_t stream = nullptr;
    /* device buffers of host calls that stage, carved from one allocation
     * (staging_arena) made by the first such call */
    unsigned char* staging_arena = nullptr;
    char* d_ascii = nullptr;
    size_t ascii_cap = 0;
    wfe_pair* d_pairs = nullptr;
    uint32_t* d_plen = nullptr;
    uint32_t* d_tlen = nullptr;
    int32_t* d_dist = nullptr;
    int8_t* d_cigar = nullptr;
    uint8_t* d_status = nullptr;
    /* in the context's arena: */
    uint32_t* d_lists = nullptr;  /* a work list of batch_size entries per bucket and tier */
    uint32_t* d_counts = nullptr; /* per bucket: list counts, finished CTAs, work counters */
    uint16_t* d_pred = nullptr;   /* predicted prefix distances */
    int32_t* d_bound = nullptr;   /* distance bounds of the pairs of the CTA-per-pair tiers */
    char* h_stage = nullptr;      /* pinned gather buffer for scattered inputs */
    wfe_pair* h_pairs = nullptr;  /* pinned descriptors of a gathered batch */
    /* Scratch of tiers 2-6 owned by this stage (stage 1 only; stage 0 uses
     * the context's): the chains of the two stages run at the same time, and
     * a tier's CTAs index their scratch by blockIdx, so two grids of one tier
     * must not share it.  One allocation, scratch_arena. */
    unsigned char* scratch_arena = nullptr;
    unsigned char* own_ops_scratch = nullptr;
    unsigned char* own_long_scratch[kNumTiers] = {};
    bool own_scratch = false;
};

/* Sub-buffers carved from one device allocation, each 256-byte aligned: a
 * cudaMalloc or cudaFree costs 40-140 us on this path (plus ~0.4 us per MB
 * freed), so a context makes one at creation -- and one more for tiers
 * 2-6's scratch, when a call first needs it -- and frees them at teardown. */
struct Carve {
    size_t used = 0;
    size_t take(size_t bytes)
    {
        const size_t at = used;
        used += (bytes + 255u) & ~size_t(255);
        return at;
    }
};

thread_local int g_last_create_error = 0;

}  // namespace

struct TimedLaunch {
    int tier;
    cudaEvent_t start, stop;
};

/* How the pairs of one length bucket are aligned: the first tier and the
 * launch shape of every tier for sequences up to max_len. */
struct BucketPlan {
    uint32_t max_len = 0;
    int first_tier = 0;
    int last_tier = 0;
    TierShape shape[kNumTiers] = {};
    LongClasses cls{};      /* tier 5's distance classes (n == 0: none) */
    TierShape bound{};      /* the bound pass (grid 0: none) */
};

struct wfe_ctx {
    wfe_config cfg{};
    int sm_count = 0;
    bool host_page_tables = false;             /* the device reads pageable memory through the CPU's page tables */
    int nbuckets = 1;
    BucketPlan bucket[kMaxBuckets];
    bool predict = false;                      /* route pairs by predicted distance */
    bool bound = true;                         /* bound distances before chains that start at tier 5-6 */
    int scratch_ctas[kNumTiers] = {};          /* CTAs whose global scratch is allocated */
    unsigned char* d_arena = nullptr;          /* the one allocation holding the buffers below, both
                                                  stages' work lists, counters and predictions and,
                                                  for host calls, stage 1's own tier scratch */
    int lists_buckets = 1;                     /* length buckets the stages' work lists have room for */
    uint32_t* d_lists_ext = nullptr;           /* work lists of more buckets (wfe_set_policy) */
    /* The global scratch of tiers 2-6 (both stages') is a second allocation,
     * made when a call first needs it (deep_ready): until then host calls
     * run their chains as far as tier 1 and defer the pairs that go further
     * (see finish_deferred).  Short reads never reach tier 2, and a context
     * for them holds ~10 MB instead of ~200. */
    bool deep_ready = false;
    unsigned char* d_deep = nullptr;
    size_t deep_bytes = 0;
    bool defer_dirty = false;                  /* a host call with a cut chain did not finish */
    uint32_t* d_defer = nullptr;               /* deferred pairs (index in the call) */
    uint32_t* d_defer_count = nullptr;
    uint32_t defer_cap = 0;
    unsigned char* d_ops_scratch = nullptr;    /* tiers 2-4 backtrace stores */
    size_t ops_scratch_bytes = 0;              /* their size (also before they are allocated) */
    unsigned char* d_long_scratch[kNumTiers] = {}; /* tiers 5-6 slabs */
    uint64_t long_slab[kNumTiers] = {};
    unsigned long long* d_passed = nullptr;    /* pairs each tier handed on, running total */
    unsigned long long* d_launched = nullptr;  /* tier launches made on the device */
    unsigned long long* d_bucket_total = nullptr; /* pairs classified into each bucket */
    uint8_t* h_launch_error = nullptr;         /* byte t: a device-side launch of tier t failed */
    uint8_t* d_launch_error = nullptr;         /* its device address */
    bool launch_error_pinned = false;          /* from cudaHostAlloc (else new[]: pageable memory the
                                                  device reaches through the CPU's page tables) */
    uint64_t single_entered[kNumTiers] = {};   /* first-tier entries of one-bucket batches */
    Stage st[kStages];
    int last_cuda_error = 0;
    wfe_stats stats{};
    std::vector<TimedLaunch> timed;            /* launches whose events are not read yet */
    std::vector<cudaEvent_t> event_pool;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr; /* device calls of several batches: stage 1's stream
                                                         after the caller's, and back */
};

namespace {

int fail_cuda(wfe_ctx* ctx, cudaError_t e)
{
    if (ctx) ctx->last_cuda_error = (int)e;
    /* the error is reported here: clear the runtime's record of it (a failed
     * allocation is not sticky), so that a later cudaGetLastError -- ours or
     * the caller's -- does not report it again */
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? WFE_ERR_OUT_OF_MEMORY : WFE_ERR_CUDA;
}

#define WFE_CUDA(ctx, call)                                        \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return fail_cuda((ctx), e_);        \
    } while (0)

/* Device-side tier launches that failed (their pairs were left unaligned)
 * since the last call, reported once as a CUDA launch failure.  Read after
 * the work in question has completed. */
int pop_launch_error(wfe_ctx* ctx)
{
    volatile uint8_t* f = ctx->h_launch_error;
    if (!f) return WFE_OK;
    bool failed = false;
    for (int t = 0; t < kNumTiers; ++t)
        if (f[t]) {
            failed = true;
            f[t] = 0u;
        }
    return failed ? fail_cuda(ctx, cudaErrorLaunchFailure) : WFE_OK;
}

/* byte t < kNumTiers: a device-side launch of tier t failed; byte
 * kDeferByte: a chain cut short deferred pairs */
constexpr size_t kLaunchErrorBytes = 8;
static_assert(kDeferByte < (int)kLaunchErrorBytes, "one launch-error byte per tier and the deferral byte");

void free_launch_error(wfe_ctx* ctx)
{
    if (ctx->launch_error_pinned)
        cudaFreeHost(ctx->h_launch_error);
    else
        delete[] reinterpret_cast<uint64_t*>(ctx->h_launch_error);
    ctx->h_launch_error = ctx->d_launch_error = nullptr;
}

uint32_t default_cigar_stride(uint32_t max_seq_len)
{
    /* src/wavefront.cuh:48-50: seq_len + (4 - seq_len % 4) */
    return max_seq_len + (4u - max_seq_len % 4u);
}

/* First tier by sequence length, used until a policy says otherwise: short
 * reads almost always finish in the 4-lane tier; longer ones start at the
 * CTA-per-pair tier, whose bound pass sends each pair to the distance class
 * that fits it (on 1,000-base reads at 10% edits 25M alignments/s against
 * 20.7M from tier 2; at 2% edits tier 1 is faster, 125M against 91M). */
int default_first_tier(uint32_t max_len)
{
    if (max_len <= 1200) return 0;
    return 5;
}

/* per-stage counters, per bucket: the count of every tier's list, finished
 * CTAs and work counters of every tier; per-stage lists: one per bucket and
 * tier */
/* per bucket: list counts (one more for the last tier's hand-on), finished
 * CTAs and work counters of every tier, then, for every class of tier 5,
 * front and back list counts, finished CTAs and work counters */
constexpr size_t kChainWords = 3 * kNumTiers + 1 + 4 * kLongClasses;
constexpr size_t kCountWords = kMaxBuckets * kChainWords;

/* What a stage owns itself: its staging and scratch allocations, pinned
 * gather buffers and stream (its lists live in the context's arena). */
void free_stage(Stage& s)
{
    cudaFree(s.staging_arena);
    cudaFree(s.scratch_arena);
    cudaFreeHost(s.h_stage);
    cudaFreeHost(s.h_pairs);
    if (s.stream) cudaStreamDestroy(s.stream);
    s = Stage();
}

/* Launch shapes of every tier for sequences up to max_len, within the
 * scratch the context holds. */
void plan_bucket(wfe_ctx* ctx, BucketPlan& b)
{
    const wfe_config& c = ctx->cfg;
    b.last_tier = b.max_len > (uint32_t)kLongSmemDistance ? 6 : 5;
    for (int t = 0; t < kNumTiers; ++t) {
        TierShape sh = tier_shape(t, b.max_len, c.cigar_stride, ctx->sm_count);
        if (t >= 2 && sh.grid > 0) sh.grid = std::min(sh.grid, ctx->scratch_ctas[t]);
        if (t >= 5 && sh.grid > 0) {
            sh.slab = ctx->long_slab[t];
            sh.scratch = ctx->d_long_scratch[t];
        }
        b.shape[t] = sh;
    }
    /* The bound pass and tier 5's classes (shapes cached per process, like
     * the tiers'); the autotuner also tries tier 5 first on buckets whose
     * pairs would not reach it otherwise. */
    b.cls = LongClasses{};
    b.bound = TierShape{};
    if (b.shape[5].grid > 0) {
        b.bound = bound_shape(b.max_len, ctx->sm_count);
        if (b.bound.grid > 0 && ctx->d_long_scratch[5]) {
            b.cls = long_classes(b.max_len, ctx->sm_count, ctx->long_slab[5] * (uint64_t)ctx->scratch_ctas[5]);
            for (int k = 0; k < b.cls.n; ++k) b.cls.shape[k].scratch = ctx->d_long_scratch[5];
        }
    }
}

bool bucket_usable(const BucketPlan& b)
{
    for (int t = b.first_tier; t <= b.last_tier; ++t)
        if (b.shape[t].grid <= 0) return false;
    return true;
}

/* The global scratch of tiers 2-6 (wfe_ctx::deep_ready): tiers 2-4's
 * backtrace stores and tiers 5-6's slabs, and, for a context whose host
 * calls keep two batches in flight, stage 1's own copy of both, in one
 * allocation.  The buckets' launch plans are made again with it.  The
 * chains enqueued before it all ended at tier 1, so none used it. */
int ensure_deep(wfe_ctx* ctx)
{
    if (ctx->deep_ready) return WFE_OK;
    const bool two = !(ctx->cfg.flags & (WFE_FLAG_DEVICE_ONLY | WFE_FLAG_NO_PIPELINE));
    const int copies = two ? 2 : 1;
    Carve k;
    size_t ops_at[2] = {}, long_at[2][kNumTiers] = {}; /* + 1: 0 means none */
    for (int i = 0; i < copies; ++i) {
        if (ctx->ops_scratch_bytes) ops_at[i] = k.take(ctx->ops_scratch_bytes) + 1u;
        for (int t = 5; t < kNumTiers; ++t)
            if (ctx->long_slab[t] && ctx->scratch_ctas[t])
                long_at[i][t] = k.take((size_t)ctx->long_slab[t] * (size_t)ctx->scratch_ctas[t]) + 1u;
    }
    if (k.used) {
        unsigned char* p = nullptr;
        const cudaError_t e = cudaMalloc(&p, k.used);
        if (e != cudaSuccess) return fail_cuda(ctx, e);
        ctx->d_deep = p;
        ctx->deep_bytes = k.used;
        if (ops_at[0]) ctx->d_ops_scratch = p + (ops_at[0] - 1u);
        for (int t = 5; t < kNumTiers; ++t)
            if (long_at[0][t]) ctx->d_long_scratch[t] = p + (long_at[0][t] - 1u);
        if (two) {
            Stage& s1 = ctx->st[1];
            if (ops_at[1]) s1.own_ops_scratch = p + (ops_at[1] - 1u);
            for (int t = 5; t < kNumTiers; ++t)
                if (long_at[1][t]) s1.own_long_scratch[t] = p + (long_at[1][t] - 1u);
        }
    }
    if (two) ctx->st[1].own_scratch = true;
    ctx->deep_ready = true;
    for (int b = 0; b < ctx->nbuckets; ++b) plan_bucket(ctx, ctx->bucket[b]);
    return WFE_OK;
}

TimedLaunch* begin_timing(wfe_ctx* ctx, int t, cudaStream_t s, int* rc)
{
    *rc = WFE_OK;
    if (!(ctx->cfg.flags & WFE_FLAG_KERNEL_TIMING)) return nullptr;
    TimedLaunch tl{t, nullptr, nullptr};
    for (cudaEvent_t* ev : {&tl.start, &tl.stop}) {
        if (!ctx->event_pool.empty()) {
            *ev = ctx->event_pool.back();
            ctx->event_pool.pop_back();
        } else if (cudaEventCreate(ev) != cudaSuccess) {
            *rc = WFE_ERR_CUDA;
            return nullptr;
        }
    }
    cudaEventRecord(tl.start, s);
    ctx->timed.push_back(tl);
    return &ctx->timed.back();
}

/* Last tier of a chain from tier `first`: a distance cap at or below a
 * tier's capacity ends the chain there. */
int chain_end(const wfe_config& c, int first, int last)
{
    if (c.max_distance > 0)
        for (int u = first; u <= last; ++u)
            if (c.max_distance <= tier_info(u).dcap) return u;
    return last;
}

/* Last tier of a chain while the context has no scratch for tiers 2-6:
 * the chain stops there and defers the pairs it would hand on. */
constexpr int kShallowLastTier = 1;

/* Last tier a chain from `first` runs to now (see chain_end and
 * kShallowLastTier), and whether that cuts it short. */
int chain_last(const wfe_ctx* ctx, int first, int last, bool* cut)
{
    const int end = chain_end(ctx->cfg, first, last);
    *cut = !ctx->deep_ready && end > kShallowLastTier;
    return *cut ? kShallowLastTier : end;
}

/* Launch the first tier of one bucket's chain over `work` (NULL: pairs
 * 0..n-1); the last CTA of every tier starts the next tier with work, on the
 * device.  `base` is the index of the batch's first pair in the call (the
 * deferred pairs of a chain cut short are recorded by it). */
int launch_bucket(wfe_ctx* ctx, Stage& st, const BucketPlan& bp, int bucket_index, int first_tier,
                  const Layout& L, bool listed, uint32_t n, int32_t* dist, int8_t* cigar, uint8_t* status,
                  cudaStream_t s, uint32_t base)
{
    const wfe_config& c = ctx->cfg;
    const uint32_t B = c.batch_size;
    const int t = first_tier;
    uint32_t* words = st.d_counts + (size_t)bucket_index * kChainWords;
    uint32_t* lists = st.d_lists + (size_t)bucket_index * kListsPerBucket * B;
    AlignLaunch a{};
    a.L = L;
    a.work = listed ? lists + (size_t)t * B : nullptr;
    a.work_count = listed ? words + t : nullptr;
    a.n_work = n;
    a.dist = dist;
    a.cigar = cigar;
    a.cigar_stride = c.cigar_stride;
    a.status = status;
    a.max_distance = c.max_distance;
    a.max_len = bp.max_len;
    a.ops_scratch = st.own_ops_scratch ? st.own_ops_scratch : ctx->d_ops_scratch;
    a.ops_scratch_bytes = ctx->ops_scratch_bytes;
    a.tier = t;
    bool cut = false;
    const int last = chain_last(ctx, t, bp.last_tier, &cut);
    if (t > last) return WFE_ERR_INTERNAL; /* a first tier past 1 gets its scratch before it launches */
    a.chain.last_tier = last;
    for (int u = 0; u < kNumTiers; ++u) {
        a.chain.shape[u] = bp.shape[u];
        if (st.own_long_scratch[u]) a.chain.shape[u].scratch = st.own_long_scratch[u];
        a.chain.list[u] = lists + (size_t)u * B;
    }
    a.chain.counts = words;
    a.chain.cta_done = words + kNumTiers + 1;
    a.chain.work_next = words + 2 * kNumTiers + 1;
    a.chain.launched = ctx->d_launched;
    a.chain.passed = ctx->d_passed;
    a.chain.launch_error = ctx->d_launch_error;
    if (cut) {
        a.chain.defer = ctx->d_defer;
        a.chain.defer_count = ctx->d_defer_count;
        a.chain.defer_cap = ctx->defer_cap;
        a.chain.defer_base = base;
    }
    a.retry = t < last ? a.chain.list[t + 1] : a.chain.defer;
    a.retry_count = t < last ? words + t + 1 : a.chain.defer_count;
    a.passed_total = ctx->d_passed + t;
    a.cls = -1;
    /* Distance bounds (and with them tier 5's classes) for every chain that
     * can reach the CTA-per-pair tiers: pairs that enter tier 5 -- first or
     * handed on -- go through the bound pass, which routes them into the
     * classes. */
    const bool bounded = ctx->bound && st.d_bound && bp.bound.grid > 0 && last >= 5;
    if (bounded) {
        a.bound = st.d_bound;
        a.chain.bound_shape = bp.bound;
        a.chain.cls = bp.cls;
        uint32_t* cw = words + 3 * kNumTiers + 1;
        for (int k = 0; k < a.chain.cls.n; ++k) {
            a.chain.cls.list[k] = lists + (size_t)(kNumTiers + k) * B;
            if (st.own_long_scratch[5]) a.chain.cls.shape[k].scratch = st.own_long_scratch[5];
        }
        a.chain.cls.cap = B;
        a.chain.cls.counts = cw;
        a.chain.cls.low_counts = cw + kLongClasses;
        a.chain.cls.cta_done = cw + 2 * kLongClasses;
        a.chain.cls.work_next = cw + 3 * kLongClasses;
    }
    int grid = bp.shape[t].grid;
    if (!listed) {
        const uint32_t per_cta = t >= 5 ? 1u : 4u * (32u / (uint32_t)tier_info(t).G);
        grid = (int)std::min<uint64_t>((uint64_t)grid, ((uint64_t)n + per_cta - 1) / per_cta);
    }
    grid = std::max(grid, 1);
    int rc = WFE_OK;
    TimedLaunch* tl = begin_timing(ctx, t, s, &rc);
    if (rc != WFE_OK) return rc;
    if (bounded && t == 5 && a.chain.cls.n > 0) {
        /* tier 5 starts with the bound pass, which starts the classes */
        WFE_CUDA(ctx, launch_bound(a, s));
    } else {
        if (bounded && t == 6) {
            /* bounds only, then tier 6 */
            WFE_CUDA(ctx, launch_bound(a, s));
            ctx->stats.kernel_launches++;
        }
        WFE_CUDA(ctx, launch_tier(t, a, grid, s));
    }
    if (tl) WFE_CUDA(ctx, cudaEventRecord(tl->stop, s));
    ctx->stats.kernel_launches++;
    ctx->stats.tier_launches[t]++;
    return WFE_OK;
}

/* Enqueue the alignment of pairs 0..n-1 of one batch on stream s: with one
 * bucket and no prediction the batch goes straight to its first tier; else
 * the pairs are routed on the device -- by length to a bucket whose launch
 * shapes fit its longest sequence, and by predicted distance to a tier --
 * and every bucket's chain runs from its first tier. */
int run_chain(wfe_ctx* ctx, Stage& st, const Layout& L, uint32_t n, int32_t* dist, int8_t* cigar,
              uint8_t* status, cudaStream_t s, const int* first_override = nullptr, uint32_t base = 0)
{
    if (n == 0) return WFE_OK;
    const uint32_t B = ctx->cfg.batch_size;
    WFE_CUDA(ctx, cudaMemsetAsync(st.d_counts, 0, sizeof(uint32_t) * kCountWords, s));
    if (ctx->nbuckets == 1 && !ctx->predict) {
        const BucketPlan& bp = ctx->bucket[0];
        const int t = first_override ? first_override[0] : bp.first_tier;
        ctx->single_entered[t] += n;
        return launch_bucket(ctx, st, bp, 0, t, L, false, n, dist, cigar, status, s, base);
    }
    Buckets bk{};
    bk.n = ctx->nbuckets;
    for (int b = 0; b < ctx->nbuckets; ++b) {
        bk.max_len[b] = ctx->bucket[b].max_len;
        bk.first_tier[b] = first_override ? first_override[b] : ctx->bucket[b].first_tier;
        /* routing never goes past the end of the bucket's chain */
        bool cut = false;
        bk.last_tier[b] = chain_last(ctx, bk.first_tier[b], ctx->bucket[b].last_tier, &cut);
    }
    for (int t = 0; t < kNumTiers; ++t) bk.dcap[t] = tier_info(t).dcap;
    /* predictions only move pairs of buckets that start below tier 5 */
    bool predict = false;
    for (int b = 0; b < ctx->nbuckets; ++b) predict |= ctx->predict && bk.first_tier[b] < 5;
    if (predict) {
        WFE_CUDA(ctx, launch_predict(L, n, ctx->cfg.max_seq_len, st.d_pred, ctx->bucket[0].shape[0].grid > 0
                                         ? ctx->bucket[0].shape[0].grid : ctx->sm_count * 8, s));
        ctx->stats.kernel_launches++;
        bk.pred = st.d_pred;
    }
    bk.lists = st.d_lists;
    bk.stride = B;
    bk.counts = st.d_counts;
    bk.count_stride = (uint32_t)kChainWords;
    bk.totals = ctx->d_bucket_total;
    WFE_CUDA(ctx, launch_classify(L, n, bk, s));
    ctx->stats.kernel_launches++;
    /* longest bucket first: its chains take longest */
    for (int b = ctx->nbuckets - 1; b >= 0; --b) {
        const int r =
            launch_bucket(ctx, st, ctx->bucket[b], b, bk.first_tier[b], L, true, n, dist, cigar, status, s, base);
        if (r != WFE_OK) return r;
    }
    return WFE_OK;
}

}  // namespace

extern "C" {

const char* wfe_strerror(int status)
{
    switch (status) {
    case WFE_OK: return "success";
    case WFE_ERR_INVALID_ARGUMENT: return "invalid argument";
    case WFE_ERR_OUT_OF_MEMORY: return "out of memory";
    case WFE_ERR_SEQ_TOO_LONG: return "sequence longer than the context's max_seq_len";
    case WFE_ERR_CUDA: return "CUDA runtime error";
    case WFE_ERR_NO_DEVICE: return "no CUDA device";
    case WFE_ERR_TIMEOUT: return "timed out";
    case WFE_ERR_BUSY: return "not enough free device memory";
    case WFE_ERR_INTERNAL: return "internal consistency check failed";
    case WFE_ERR_NOT_FOUND: return "unknown ticket";
    default: return "unknown status";
    }
}

int wfe_last_cuda_error(const wfe_ctx* ctx) { return ctx ? ctx->last_cuda_error : g_last_create_error; }

}  // extern "C"

namespace wfe {
int take_launch_error(wfe_ctx* ctx) { return pop_launch_error(ctx); }

/* wfe_create with the slab budgets of tiers 5 and 6 (0: 2 GiB and 8 GiB):
 * a smaller budget only lowers how many long pairs run at once. */
int create_context(const wfe_config* cfg, uint64_t budget5, uint64_t budget6, wfe_ctx** out)
{
    if (!cfg || !out) return WFE_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (cfg->max_seq_len == 0 || cfg->max_distance < 0) return WFE_ERR_INVALID_ARGUMENT;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        g_last_create_error = (int)e;
        return WFE_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev) return WFE_ERR_INVALID_ARGUMENT;
    e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) { g_last_create_error = (int)e; return WFE_ERR_CUDA; }

    wfe_ctx* ctx = new (std::nothrow) wfe_ctx();
    if (!ctx) return WFE_ERR_OUT_OF_MEMORY;
    ctx->cfg = *cfg;
    wfe_config& c = ctx->cfg;
    if (c.batch_size == 0) c.batch_size = 100000;
    if (c.cigar_stride == 0) c.cigar_stride = default_cigar_stride(c.max_seq_len);

    auto bail = [&](cudaError_t err) {
        g_last_create_error = (int)err;
        cudaGetLastError(); /* reported here, not to a later call */
        for (auto& s : ctx->st) free_stage(s);
        cudaFree(ctx->d_arena);
        cudaFree(ctx->d_deep);
        free_launch_error(ctx);
        delete ctx;
        return err == cudaErrorMemoryAllocation ? WFE_ERR_OUT_OF_MEMORY : WFE_ERR_CUDA;
    };

    e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, c.device);
    if (e != cudaSuccess) return bail(e);
    int hpt = 0;
    e = cudaDeviceGetAttribute(&hpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, c.device);
    if (e != cudaSuccess) return bail(e);
    ctx->host_page_tables = hpt != 0;
    /* Global scratch is sized for the longest sequences (max_seq_len); a
     * bucket of shorter sequences has more resident CTAs and uses at most
     * the CTAs that scratch was sized for.  Tiers 2-6's scratch is one
     * allocation (ensure_deep), made here when the first tier is past 1 or
     * the context is for device calls only, else by the first call that
     * needs it; everything else the context keeps on the device is carved
     * from another. */
    size_t scratch = 0;
    Carve arena;
    const int last = c.max_seq_len > (uint32_t)kLongSmemDistance ? 6 : 5;
    for (int t = 0; t <= last; ++t) {
        const TierShape sh = tier_shape(t, c.max_seq_len, c.cigar_stride, ctx->sm_count);
        if (sh.grid <= 0) continue;
        if (t >= 2 && t <= 4) {
            ctx->scratch_ctas[t] = sh.grid;
            scratch = std::max(scratch, tier_scratch_bytes(t, sh.grid, c.max_seq_len));
        } else if (t >= 5) {
            /* a slab per resident CTA (backtrace store, chain, runs; tier 6
             * also its wavefront), the grid trimmed to a budget */
            const uint64_t budget = t == 5 ? (budget5 ? budget5 : (2ull << 30)) : (budget6 ? budget6 : (8ull << 30));
            const int grid = (int)std::min<uint64_t>((uint64_t)sh.grid, std::max<uint64_t>(1, budget / sh.slab));
            ctx->scratch_ctas[t] = grid;
            ctx->long_slab[t] = sh.slab;
        }
    }
    ctx->ops_scratch_bytes = scratch;
    const size_t nctr = 2 * kNumTiers + kMaxBuckets;
    const size_t passed_at = arena.take(sizeof(unsigned long long) * nctr);
    const size_t B = c.batch_size;
    size_t lists_at[kStages], counts_at[kStages], pred_at[kStages], bound_at[kStages];
    for (int i = 0; i < kStages; ++i) {
        /* a work list per tier of one length bucket; wfe_set_policy adds
         * room for more buckets */
        lists_at[i] = arena.take((size_t)kListsPerBucket * B * sizeof(uint32_t));
        counts_at[i] = arena.take(sizeof(uint32_t) * kCountWords);
        pred_at[i] = arena.take(B * sizeof(uint16_t));
        bound_at[i] = arena.take(B * sizeof(int32_t));
    }
    /* pairs deferred by host calls that run before tiers 2-6 have scratch */
    const size_t defer_at = arena.take(B * sizeof(uint32_t));
    const size_t defer_count_at = arena.take(sizeof(uint32_t));
    if ((e = cudaMalloc(&ctx->d_arena, arena.used)) != cudaSuccess) return bail(e);
    unsigned char* A0 = ctx->d_arena;
    ctx->d_defer = reinterpret_cast<uint32_t*>(A0 + defer_at);
    ctx->d_defer_count = reinterpret_cast<uint32_t*>(A0 + defer_count_at);
    ctx->defer_cap = (uint32_t)B;
    ctx->d_passed = reinterpret_cast<unsigned long long*>(A0 + passed_at);
    for (int i = 0; i < kStages; ++i) {
        Stage& s = ctx->st[i];
        s.d_lists = reinterpret_cast<uint32_t*>(A0 + lists_at[i]);
        s.d_counts = reinterpret_cast<uint32_t*>(A0 + counts_at[i]);
        s.d_pred = reinterpret_cast<uint16_t*>(A0 + pred_at[i]);
        s.d_bound = reinterpret_cast<int32_t*>(A0 + bound_at[i]);
    }
    ctx->nbuckets = 1;
    ctx->bucket[0].max_len = c.max_seq_len;
    ctx->bucket[0].first_tier = default_first_tier(c.max_seq_len);
    plan_bucket(ctx, ctx->bucket[0]);
    if (!bucket_usable(ctx->bucket[0])) return bail(cudaErrorInvalidValue); /* sequences too long for shared memory */

    ctx->d_launched = ctx->d_passed + kNumTiers;
    ctx->d_bucket_total = ctx->d_passed + 2 * kNumTiers;
    /* The record of failed device-side launches is host memory the kernels
     * write in place.  A device that reads the CPU's page tables (ATS over
     * NVLink-C2C) writes ordinary heap memory; elsewhere it is a mapped
     * page-locked word (cudaHostAlloc costs ~0.15 ms, and as much to free). */
    if (ctx->host_page_tables) {
        uint64_t* w = new (std::nothrow) uint64_t[1];
        if (!w) return bail(cudaErrorMemoryAllocation);
        *w = 0u; /* the page is present before the device can write it */
        ctx->h_launch_error = ctx->d_launch_error = reinterpret_cast<uint8_t*>(w);
    } else {
        if ((e = cudaHostAlloc(&ctx->h_launch_error, kLaunchErrorBytes, cudaHostAllocMapped)) != cudaSuccess)
            return bail(e);
        ctx->launch_error_pinned = true;
        std::memset(ctx->h_launch_error, 0, kLaunchErrorBytes);
        if ((e = cudaHostGetDevicePointer(&ctx->d_launch_error, ctx->h_launch_error, 0)) != cudaSuccess)
            return bail(e);
    }
    const bool host_calls = !(c.flags & WFE_FLAG_DEVICE_ONLY);
    for (auto& s : ctx->st) {
        if ((e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
        /* the staging buffers of host calls are allocated by the first call
         * that stages (see ensure_staging) */
        if (host_calls) s.ascii_cap = B * 2u * (size_t)c.max_seq_len + 64u;
    }
    /* the counters start at zero; both stages' streams come after this */
    if ((e = cudaMemsetAsync(ctx->d_passed, 0, sizeof(unsigned long long) * nctr, ctx->st[0].stream)) != cudaSuccess)
        return bail(e);
    if ((e = cudaMemsetAsync(ctx->d_defer_count, 0, sizeof(uint32_t), ctx->st[0].stream)) != cudaSuccess)
        return bail(e);
    if ((e = cudaStreamSynchronize(ctx->st[0].stream)) != cudaSuccess) return bail(e);
    if ((c.flags & WFE_FLAG_DEVICE_ONLY) || ctx->bucket[0].first_tier > kShallowLastTier)
        if (ensure_deep(ctx) != WFE_OK) return bail((cudaError_t)ctx->last_cuda_error);
    *out = ctx;
    return WFE_OK;
}

}  // namespace wfe

namespace {
int ensure_stage_scratch(wfe_ctx* ctx, Stage& s);
}  // namespace

extern "C" {

int wfe_create(const wfe_config* cfg, wfe_ctx** out) { return wfe::create_context(cfg, 0, 0, out); }

int wfe_create_with_scratch(const wfe_config* cfg, uint64_t tier5_bytes, uint64_t tier6_bytes, wfe_ctx** out)
{
    return wfe::create_context(cfg, tier5_bytes, tier6_bytes, out);
}

int wfe_set_policy(wfe_ctx* ctx, uint32_t nbuckets, const uint32_t* bucket_max_len, const int32_t* first_tier,
                   uint32_t flags)
{
    if (!ctx || nbuckets < 1 || nbuckets > (uint32_t)kMaxBuckets || !bucket_max_len) return WFE_ERR_INVALID_ARGUMENT;
    if (flags & ~(uint32_t)(WFE_POLICY_PREDICT | WFE_POLICY_NO_BOUND)) return WFE_ERR_INVALID_ARGUMENT;
    BucketPlan plan[kMaxBuckets];
    for (uint32_t b = 0; b < nbuckets; ++b) {
        uint32_t m = bucket_max_len[b];
        if (b + 1 == nbuckets) m = ctx->cfg.max_seq_len; /* the last bucket holds everything */
        if (m == 0 || m > ctx->cfg.max_seq_len || (b > 0 && m <= plan[b - 1].max_len))
            return WFE_ERR_INVALID_ARGUMENT;
        plan[b].max_len = m;
        const int32_t ft = first_tier ? first_tier[b] : -1;
        if (ft >= kNumTiers) return WFE_ERR_INVALID_ARGUMENT;
        plan[b].first_tier = ft < 0 ? default_first_tier(m) : ft;
        plan_bucket(ctx, plan[b]);
        if (plan[b].first_tier > plan[b].last_tier || !bucket_usable(plan[b])) return WFE_ERR_INVALID_ARGUMENT;
    }
    WFE_CUDA(ctx, cudaSetDevice(ctx->cfg.device));
    for (auto& s : ctx->st) WFE_CUDA(ctx, cudaStreamSynchronize(s.stream));
    /* a first tier past 1, or routing by predicted distance, needs tiers
     * 2-6's scratch from the start */
    bool deep = (flags & WFE_POLICY_PREDICT) != 0;
    for (uint32_t b = 0; b < nbuckets; ++b) deep |= plan[b].first_tier > kShallowLastTier;
    if (deep && !ctx->deep_ready) {
        if (const int r = ensure_deep(ctx)) return r;
        for (uint32_t b = 0; b < nbuckets; ++b) plan_bucket(ctx, plan[b]);
    }
    if ((int)nbuckets > ctx->lists_buckets) {
        /* work lists for every tier of every bucket, both stages */
        const size_t per_stage = (size_t)nbuckets * kListsPerBucket * ctx->cfg.batch_size;
        uint32_t* lists = nullptr;
        WFE_CUDA(ctx, cudaMalloc(&lists, kStages * per_stage * sizeof(uint32_t)));
        cudaFree(ctx->d_lists_ext);
        ctx->d_lists_ext = lists;
        for (int i = 0; i < kStages; ++i) ctx->st[i].d_lists = lists + (size_t)i * per_stage;
        ctx->lists_buckets = (int)nbuckets;
    }
    ctx->nbuckets = (int)nbuckets;
    for (uint32_t b = 0; b < nbuckets; ++b) ctx->bucket[b] = plan[b];
    ctx->predict = (flags & WFE_POLICY_PREDICT) != 0;
    ctx->bound = (flags & WFE_POLICY_NO_BOUND) == 0;
    return WFE_OK;
}

int wfe_get_policy(const wfe_ctx* ctx, uint32_t* nbuckets, uint32_t* bucket_max_len, int32_t* first_tier,
                   uint32_t* flags)
{
    if (!ctx || !nbuckets) return WFE_ERR_INVALID_ARGUMENT;
    *nbuckets = (uint32_t)ctx->nbuckets;
    if (flags) *flags = (ctx->predict ? WFE_POLICY_PREDICT : 0u) | (ctx->bound ? 0u : WFE_POLICY_NO_BOUND);
    for (int b = 0; b < ctx->nbuckets; ++b) {
        if (bucket_max_len) bucket_max_len[b] = ctx->bucket[b].max_len;
        if (first_tier) first_tier[b] = ctx->bucket[b].first_tier;
    }
    return WFE_OK;
}

void wfe_destroy(wfe_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->cfg.device);
    for (auto& s : ctx->st)
        if (s.stream) cudaStreamSynchronize(s.stream);
    for (auto& s : ctx->st) free_stage(s);
    cudaFree(ctx->d_arena);
    cudaFree(ctx->d_deep);
    cudaFree(ctx->d_lists_ext);
    free_launch_error(ctx);
    for (auto& t : ctx->timed) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    for (auto ev : ctx->event_pool) cudaEventDestroy(ev);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    delete ctx;
}

int wfe_get_stats(wfe_ctx* ctx, wfe_stats* out)
{
    if (!ctx || !out) return WFE_ERR_INVALID_ARGUMENT;
    WFE_CUDA(ctx, cudaSetDevice(ctx->cfg.device));
    for (auto& s : ctx->st) WFE_CUDA(ctx, cudaStreamSynchronize(s.stream));
    for (auto& t : ctx->timed) {
        WFE_CUDA(ctx, cudaEventSynchronize(t.stop));
        float ms = 0.f;
        WFE_CUDA(ctx, cudaEventElapsedTime(&ms, t.start, t.stop));
        ctx->stats.tier_ms[t.tier] += ms;
        ctx->event_pool.push_back(t.start);
        ctx->event_pool.push_back(t.stop);
    }
    ctx->timed.clear();
    unsigned long long dev[2 * kNumTiers + kMaxBuckets] = {};
    WFE_CUDA(ctx, cudaMemcpy(dev, ctx->d_passed, sizeof(dev), cudaMemcpyDeviceToHost));
    *out = ctx->stats;
    out->deep_scratch_bytes = ctx->deep_bytes;
    for (int t = 0; t < kNumTiers; ++t) {
        out->tier_passed[t] = dev[t];
        out->tier_entered[t] = ctx->single_entered[t] + (t > 0 ? dev[t - 1] : 0);
        out->tier_launches[t] += dev[kNumTiers + t];
        out->kernel_launches += dev[kNumTiers + t];
    }
    for (int b = 0; b < ctx->nbuckets; ++b) out->tier_entered[ctx->bucket[b].first_tier] += dev[2 * kNumTiers + b];
    return WFE_OK;
}

int wfe_reset_stats(wfe_ctx* ctx)
{
    if (!ctx) return WFE_ERR_INVALID_ARGUMENT;
    wfe_stats tmp;
    const int r = wfe_get_stats(ctx, &tmp); /* drains pending timings */
    if (r != WFE_OK) return r;
    ctx->stats = wfe_stats{};
    for (auto& x : ctx->single_entered) x = 0;
    WFE_CUDA(ctx, cudaMemset(ctx->d_passed, 0, sizeof(unsigned long long) * (2 * kNumTiers + kMaxBuckets)));
    return WFE_OK;
}

int wfe_align_device(wfe_ctx* ctx, const char* d_ascii, const wfe_pair* d_pairs, size_t n,
                     uint32_t max_len, int32_t* d_dist, int8_t* d_cigar, uint8_t* d_status,
                     void* stream)
{
    if (!ctx || (n && (!d_ascii || !d_pairs || !d_dist || (!d_cigar && ctx->cfg.cigar_stride))))
        return WFE_ERR_INVALID_ARGUMENT;
    if (max_len > ctx->cfg.max_seq_len) return WFE_ERR_SEQ_TOO_LONG;
    WFE_CUDA(ctx, cudaSetDevice(ctx->cfg.device));
    /* an earlier asynchronous call whose device-side launch failed */
    if (const int r = pop_launch_error(ctx)) return r;
    /* a device call returns before its chains end, so they run whole: the
     * first one allocates tiers 2-6's scratch if no call has yet */
    if (const int r = ensure_deep(ctx)) return r;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->st[0].stream;
    const size_t B = ctx->cfg.batch_size;
    /* Several batches alternate between `stream` (stage 0) and stage 1's
     * stream, which first waits for the work already on `stream` and which
     * `stream` waits for at the end: the last CTAs of one batch then share
     * the GPU with the first of the next, and the call stays ordered on
     * `stream`.  Stage 1 has its own work lists and tier scratch (allocated
     * by the first call that needs them); without them the batches run one
     * after another. */
    int nstages = 1;
    if (n > B && !(ctx->cfg.flags & WFE_FLAG_NO_PIPELINE)) {
        const int seen = ctx->last_cuda_error;
        if (ensure_stage_scratch(ctx, ctx->st[1]) == WFE_OK) {
            if (!ctx->ev_fork) WFE_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
            if (!ctx->ev_join) WFE_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
            WFE_CUDA(ctx, cudaEventRecord(ctx->ev_fork, s));
            WFE_CUDA(ctx, cudaStreamWaitEvent(ctx->st[1].stream, ctx->ev_fork, 0));
            nstages = 2;
        } else {
            ctx->last_cuda_error = seen; /* no failure of the call: its batches run on `stream` alone */
        }
    }
    int rc = WFE_OK;
    size_t bi = 0;
    for (size_t b0 = 0; b0 < n && rc == WFE_OK; b0 += B, ++bi) {
        const uint32_t nb = (uint32_t)std::min(B, n - b0);
        const int si = (int)(bi % (size_t)nstages);
        Layout L{};
        L.ascii = d_ascii;
        L.pairs = d_pairs + b0;
        L.base_off = 0;
        rc = run_chain(ctx, ctx->st[si], L, nb, d_dist + b0, d_cigar ? d_cigar + b0 * ctx->cfg.cigar_stride : nullptr,
                       d_status ? d_status + b0 : nullptr, si ? ctx->st[1].stream : s);
        if (rc != WFE_OK) break;
        ctx->stats.batches++;
        ctx->stats.pairs += nb;
    }
    if (nstages == 2) {
        /* also after a failed enqueue: nothing on `stream` may overtake stage 1 */
        WFE_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->st[1].stream));
        WFE_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_join, 0));
    }
    return rc;
}

}  // extern "C"

namespace {

/* Host-buffer pipeline shared by wfe_align and wfe_align_strided. */
struct HostJob {
    const char* ascii;
    size_t ascii_bytes;
    const wfe_pair* pairs;   /* descriptor layout */
    size_t stride;           /* strided layout when pairs == NULL */
    const uint32_t* p_len;
    const uint32_t* t_len;
};

/* A pageable host range that the device reaches through the CPU's page
 * tables.  Its pages are made present on the host before the device touches
 * them: a page the device finds missing is filled by a fault that costs ~5x
 * the host's own first touch (152 MB of fresh output: 33 ms from the GPU,
 * 6.4 ms from one host thread, 1.3 ms from eight).  One byte per page is
 * touched.  Input pages are read.  Output pages that were missing get a 0
 * written (no read first: a read maps the shared zero page, and the write
 * after it costs a copy-on-write fault, 40x slower); present ones are read
 * and written back, which also shows that they are writable.  Every byte
 * touched lies inside the sub-range being touched, so touching one batch's
 * outputs never writes bytes of a batch the device is already writing. */
struct HostRange {
    char* p = nullptr;
    size_t bytes = 0;
    bool write = false;
    uintptr_t lo = 0;                    /* first page */
    std::vector<unsigned char> resident; /* per page, when the call started */
    size_t missing = 0;                  /* pages not present then */

    static size_t page()
    {
        static const size_t pg = (size_t)sysconf(_SC_PAGESIZE);
        return pg;
    }

    /* false when part of the range is not mapped at all (mincore fails) */
    bool map(const void* q, size_t n, bool w)
    {
        p = (char*)q;
        bytes = n;
        write = w;
        lo = (uintptr_t)q & ~(uintptr_t)(page() - 1);
        const uintptr_t hi = (uintptr_t)q + n;
        resident.assign((hi - lo + page() - 1) / page(), 0);
        if (mincore((void*)lo, hi - lo, resident.data()) != 0) return false;
        missing = 0;
        for (unsigned char r : resident) missing += (r & 1u) ? 0u : 1u;
        return true;
    }

    /* touch the pages that overlap bytes [off0, off1) of the range */
    void touch(size_t off0, size_t off1) const
    {
        if (off0 >= off1) return;
        const uintptr_t a0 = (uintptr_t)p + off0, a1 = (uintptr_t)p + off1;
        for (size_t k = (a0 - lo) / page(); k <= (a1 - 1 - lo) / page(); ++k) {
            volatile char* q = (volatile char*)std::max<uintptr_t>(a0, lo + k * page());
            if (write && !(resident[k] & 1u)) {
                *q = 0;
            } else {
                const char v = *q;
                if (write) *q = v;
            }
        }
    }
};

/* Device address of a host buffer that the kernels can use in place, or
 * NULL when it has to be staged.  Pinned, device-mapped memory is always
 * used in place.  Pageable memory is used in place when `pageable` (the
 * caller's WFE_FLAG_PAGEABLE_IN_PLACE on a device that reads the CPU's page
 * tables) and all of it is mapped; an input's missing pages are read here,
 * an output's are left to the caller (range filled in). */
void* mapped_address(const void* p, size_t bytes, bool write, bool pageable, HostRange* range)
{
    if (!p) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError(); /* pageable memory of an older driver: not mapped */
        return nullptr;
    }
    if (at.type == cudaMemoryTypeHost) return at.devicePointer;
    if (at.type != cudaMemoryTypeUnregistered || !pageable || bytes == 0) return nullptr;
    try {
        HostRange r;
        if (!r.map(p, bytes, write)) return nullptr;
        if (write) {
            *range = std::move(r);
        } else if (r.missing) {
            r.touch(0, bytes);
        }
    } catch (const std::bad_alloc&) {
        return nullptr; /* no room for the page map: staged */
    }
    return const_cast<void*>(p);
}

/* The output pages of a call's batches, touched in batch order by helper
 * threads while the device aligns the earlier batches; the host launches
 * batch b once its pages are done.  Threads are used only when more than
 * 8 MB of output pages are missing; otherwise ready() touches the batch
 * itself. */
class OutputPages {
public:
    OutputPages(std::vector<HostRange> ranges, std::vector<size_t> unit, size_t batch, size_t n)
        : r_(std::move(ranges)), unit_(std::move(unit)), batch_(batch), n_(n)
    {
        size_t missing = 0;
        for (const HostRange& r : r_) missing += r.missing;
        nb_ = batch_ ? (n_ + batch_ - 1) / batch_ : 0;
        if (r_.empty() || missing * HostRange::page() < (8u << 20) || nb_ == 0) return;
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const unsigned want = std::min(8u, hw);
        left_.reset(new (std::nothrow) std::atomic<unsigned>[nb_]);
        if (!left_) return;
        /* the helpers wait for `go_`, so that the stripes are cut for the
         * threads that could actually be started (none: ready() touches) */
        for (unsigned t = 0; t < want; ++t) {
            try {
                th_.emplace_back([this, t] { run(t); });
            } catch (...) {
                break;
            }
        }
        nthreads_ = (unsigned)th_.size();
        for (size_t b = 0; b < nb_; ++b) left_[b].store(nthreads_);
        go_.store(true, std::memory_order_release);
    }
    ~OutputPages()
    {
        stop_.store(true);
        go_.store(true, std::memory_order_release);
        for (auto& x : th_) x.join();
    }
    /* batch b's output pages are present */
    void ready(size_t b)
    {
        if (r_.empty() || b >= nb_) return;
        if (th_.empty()) {
            stripe(b, 0, 1);
            return;
        }
        while (left_[b].load(std::memory_order_acquire) != 0) std::this_thread::yield();
    }

private:
    void stripe(size_t b, unsigned t, unsigned T) const
    {
        const size_t i0 = b * batch_, i1 = std::min(n_, i0 + batch_);
        for (size_t k = 0; k < r_.size(); ++k) {
            const size_t o0 = i0 * unit_[k], o1 = i1 * unit_[k];
            r_[k].touch(o0 + (o1 - o0) * t / T, o0 + (o1 - o0) * (t + 1) / T);
        }
    }
    void run(unsigned t)
    {
        while (!go_.load(std::memory_order_acquire)) std::this_thread::yield();
        for (size_t b = 0; b < nb_ && !stop_.load(std::memory_order_relaxed); ++b) {
            stripe(b, t, nthreads_);
            left_[b].fetch_sub(1, std::memory_order_release);
        }
    }
    std::vector<HostRange> r_;
    std::vector<size_t> unit_; /* bytes per pair in each range */
    size_t batch_, n_, nb_ = 0;
    unsigned nthreads_ = 0;
    std::unique_ptr<std::atomic<unsigned>[]> left_;
    std::atomic<bool> stop_{false};
    std::atomic<bool> go_{false};
    std::vector<std::thread> th_;
};

/* The device buffers a stage needs to stage a batch of host inputs in and
 * results out, allocated when a host call first stages (pinned and, with
 * WFE_FLAG_PAGEABLE_IN_PLACE, pageable buffers are used in place and never
 * need them).  A failed allocation leaves none of them behind. */
int ensure_staging(wfe_ctx* ctx, Stage& s)
{
    if (s.staging_arena) return WFE_OK;
    const size_t B = ctx->cfg.batch_size;
    Carve c;
    const size_t ascii_at = c.take(s.ascii_cap), pairs_at = c.take(B * sizeof(wfe_pair));
    const size_t plen_at = c.take(B * sizeof(uint32_t)), tlen_at = c.take(B * sizeof(uint32_t));
    const size_t dist_at = c.take(B * sizeof(int32_t));
    const size_t cigar_at = c.take(B * (size_t)ctx->cfg.cigar_stride + 16u), status_at = c.take(B);
    const cudaError_t e = cudaMalloc(&s.staging_arena, c.used);
    if (e != cudaSuccess) {
        s.staging_arena = nullptr;
        return fail_cuda(ctx, e);
    }
    unsigned char* a = s.staging_arena;
    s.d_ascii = reinterpret_cast<char*>(a + ascii_at);
    s.d_pairs = reinterpret_cast<wfe_pair*>(a + pairs_at);
    s.d_plen = reinterpret_cast<uint32_t*>(a + plen_at);
    s.d_tlen = reinterpret_cast<uint32_t*>(a + tlen_at);
    s.d_dist = reinterpret_cast<int32_t*>(a + dist_at);
    s.d_cigar = reinterpret_cast<int8_t*>(a + cigar_at);
    s.d_status = reinterpret_cast<uint8_t*>(a + status_at);
    return WFE_OK;
}

/* Stage 1's own scratch of tiers 2-6, the size of the context's, allocated
 * when a device call first runs two batches at once on a context for
 * device calls only (other contexts get it with the context's, in
 * ensure_deep; before that their chains need none).  A failed allocation
 * leaves none of it behind. */
int ensure_stage_scratch(wfe_ctx* ctx, Stage& s)
{
    if (s.own_scratch || !ctx->deep_ready) return WFE_OK;
    Carve c;
    const size_t ops_at = ctx->d_ops_scratch ? c.take(ctx->ops_scratch_bytes) : 0u;
    size_t long_at[kNumTiers] = {};
    for (int t = 5; t < kNumTiers; ++t)
        if (ctx->d_long_scratch[t])
            long_at[t] = c.take((size_t)ctx->long_slab[t] * (size_t)ctx->scratch_ctas[t]) + 1u; /* 0: none */
    if (c.used) {
        const cudaError_t e = cudaMalloc(&s.scratch_arena, c.used);
        if (e != cudaSuccess) {
            s.scratch_arena = nullptr;
            return fail_cuda(ctx, e);
        }
        if (ctx->d_ops_scratch) s.own_ops_scratch = s.scratch_arena + ops_at;
        for (int t = 5; t < kNumTiers; ++t)
            if (long_at[t]) s.own_long_scratch[t] = s.scratch_arena + (long_at[t] - 1u);
    }
    s.own_scratch = true;
    return WFE_OK;
}

int align_host_checked(wfe_ctx* ctx, const HostJob& job, size_t n, int32_t* dist_out, int8_t* cigar_out,
                       uint8_t* status_out);
int finish_deferred(wfe_ctx* ctx, const HostJob& job, size_t n, int32_t* dist_out, int8_t* cigar_out,
                    uint8_t* status_out);

/* The host-buffer calls: no C++ exception crosses the C ABI. */
int align_host(wfe_ctx* ctx, const HostJob& job, size_t n, int32_t* dist_out, int8_t* cigar_out,
               uint8_t* status_out)
{
    try {
        return align_host_checked(ctx, job, n, dist_out, cigar_out, status_out);
    } catch (const std::bad_alloc&) {
        return WFE_ERR_OUT_OF_MEMORY;
    } catch (...) {
        return WFE_ERR_INTERNAL;
    }
}

int align_host_checked(wfe_ctx* ctx, const HostJob& job, size_t n, int32_t* dist_out, int8_t* cigar_out,
                       uint8_t* status_out)
{
    const wfe_config& c = ctx->cfg;
    if (c.flags & WFE_FLAG_DEVICE_ONLY) return WFE_ERR_INVALID_ARGUMENT;
    WFE_CUDA(ctx, cudaSetDevice(c.device));
    const bool want_cigar = cigar_out && c.cigar_stride;
    if (!ctx->deep_ready) {
        /* Without tiers 2-6's scratch the chains stop at tier 1 and defer
         * what they would hand on, recorded by the pair's index in the call.
         * A first tier past 1, or more pairs than those indices hold, needs
         * the scratch now. */
        bool deep = n > (size_t)UINT32_MAX;
        for (int b = 0; b < ctx->nbuckets; ++b) deep |= ctx->bucket[b].first_tier > kShallowLastTier;
        if (deep) {
            if (const int r = ensure_deep(ctx)) return r;
        } else {
            if (ctx->defer_dirty) {
                /* an earlier call that deferred pairs did not finish */
                WFE_CUDA(ctx, cudaMemset(ctx->d_defer_count, 0, sizeof(uint32_t)));
                reinterpret_cast<volatile uint8_t*>(ctx->h_launch_error)[kDeferByte] = 0u;
            }
            ctx->defer_dirty = true;
        }
    }

    /* pinned inputs are read in place, pinned outputs written in place, and
     * so are pageable ones when asked for on a device that can */
    const bool pg = (c.flags & WFE_FLAG_PAGEABLE_IN_PLACE) && ctx->host_page_tables && n > 0;
    HostRange r_dist, r_cigar, r_status, unused;
    const char* m_ascii = (const char*)mapped_address(job.ascii, job.ascii_bytes, false, pg, &unused);
    const wfe_pair* m_pairs =
        job.pairs ? (const wfe_pair*)mapped_address(job.pairs, n * sizeof(wfe_pair), false, pg, &unused) : nullptr;
    const uint32_t* m_plen =
        job.pairs ? nullptr : (const uint32_t*)mapped_address(job.p_len, n * 4u, false, pg, &unused);
    const uint32_t* m_tlen =
        job.pairs ? nullptr : (const uint32_t*)mapped_address(job.t_len, n * 4u, false, pg, &unused);
    const bool in_place = m_ascii && job.ascii_bytes > 0 && (job.pairs ? m_pairs != nullptr : (m_plen && m_tlen));
    int32_t* m_dist = (int32_t*)mapped_address(dist_out, n * 4u, true, pg, &r_dist);
    int8_t* m_cigar =
        want_cigar ? (int8_t*)mapped_address(cigar_out, n * (size_t)c.cigar_stride, true, pg, &r_cigar) : nullptr;
    uint8_t* m_status = status_out ? (uint8_t*)mapped_address(status_out, n, true, pg, &r_status) : nullptr;
    const bool out_in_place = m_dist && (!want_cigar || m_cigar) && (!status_out || m_status);

    size_t B = c.batch_size;
    if (!job.pairs && !in_place) {
        /* strided slots may be wider than max_seq_len: fewer pairs per batch */
        const size_t fit = (ctx->st[0].ascii_cap - 32u) / (2u * job.stride);
        if (fit == 0) return WFE_ERR_SEQ_TOO_LONG;
        B = std::min(B, fit);
    }
    /* pageable outputs written in place: their pages are made present batch
     * by batch, ahead of the device */
    std::vector<HostRange> pages;
    std::vector<size_t> unit;
    if (out_in_place) {
        if (r_dist.p) pages.push_back(std::move(r_dist)), unit.push_back(4u);
        if (r_cigar.p) pages.push_back(std::move(r_cigar)), unit.push_back(c.cigar_stride);
        if (r_status.p) pages.push_back(std::move(r_status)), unit.push_back(1u);
    }
    OutputPages out_pages(std::move(pages), std::move(unit), B, n);
    int nstages = (c.flags & WFE_FLAG_NO_PIPELINE) ? 1 : kStages;
    /* a second batch in flight needs the second stage's own tier scratch;
     * without it the call runs one batch at a time */
    if (nstages > 1 && n > B && ensure_stage_scratch(ctx, ctx->st[1]) != WFE_OK) nstages = 1;
    if (n > 0 && (!in_place || !out_in_place))
        for (int i = 0; i < nstages; ++i) {
            const int r = ensure_staging(ctx, ctx->st[i]);
            if (r != WFE_OK) return r;
        }
    size_t bi = 0;
    size_t nb = 0;
    for (size_t b0 = 0; b0 < n; b0 += nb, ++bi) {
        Stage& st = ctx->st[bi % nstages];
        cudaStream_t s = st.stream;
        nb = std::min(B, n - b0);
        Layout L{};
        if (in_place) {
            /* the kernels read the pinned inputs over the CPU-GPU link and
             * check every pair against the buffer */
            L.ascii = m_ascii;
            L.ascii_bytes = job.ascii_bytes;
            if (job.pairs) {
                L.pairs = m_pairs + b0;
            } else {
                L.ascii = m_ascii + 2u * b0 * job.stride;
                L.ascii_bytes = 2u * nb * job.stride;
                L.plen = m_plen + b0;
                L.tlen = m_tlen + b0;
                L.stride = job.stride;
            }
            ctx->stats.mapped_batches++;
        } else if (job.pairs) {
            const wfe_pair* P = job.pairs + b0;
            uint64_t lo = UINT64_MAX, hi = 0;
            for (size_t i = 0; i < nb; ++i) {
                if (P[i].p_len > c.max_seq_len || P[i].t_len > c.max_seq_len) return WFE_ERR_SEQ_TOO_LONG;
                const uint64_t pe = P[i].p_off + P[i].p_len, te = P[i].t_off + P[i].t_len;
                if (pe > job.ascii_bytes || te > job.ascii_bytes || pe < P[i].p_off || te < P[i].t_off)
                    return WFE_ERR_INVALID_ARGUMENT;
                lo = std::min(lo, std::min(P[i].p_off, P[i].t_off));
                hi = std::max(hi, std::max(pe, te));
            }
            if (nb == 0 || hi <= lo) lo = hi = 0;
            if (hi - lo + 32u <= st.ascii_cap) {
                /* one contiguous copy of the batch's span */
                WFE_CUDA(ctx, cudaMemcpyAsync(st.d_ascii, job.ascii + lo, hi - lo, cudaMemcpyHostToDevice, s));
                WFE_CUDA(ctx, cudaMemcpyAsync(st.d_pairs, P, nb * sizeof(wfe_pair), cudaMemcpyHostToDevice, s));
                ctx->stats.h2d_bytes += (hi - lo) + nb * sizeof(wfe_pair);
                L.base_off = lo;
            } else {
                /* scattered inputs: gather this batch through pinned memory */
                WFE_CUDA(ctx, cudaStreamSynchronize(s));
                if (!st.h_stage) {
                    WFE_CUDA(ctx, cudaMallocHost(&st.h_stage, st.ascii_cap));
                    WFE_CUDA(ctx, cudaMallocHost(&st.h_pairs, c.batch_size * sizeof(wfe_pair)));
                }
                uint64_t pos = 0;
                for (size_t i = 0; i < nb; ++i) {
                    wfe_pair q = P[i];
                    std::memcpy(st.h_stage + pos, job.ascii + q.p_off, q.p_len);
                    q.p_off = pos;
                    pos += q.p_len;
                    std::memcpy(st.h_stage + pos, job.ascii + q.t_off, q.t_len);
                    q.t_off = pos;
                    pos += q.t_len;
                    st.h_pairs[i] = q;
                }
                WFE_CUDA(ctx, cudaMemcpyAsync(st.d_ascii, st.h_stage, pos, cudaMemcpyHostToDevice, s));
                WFE_CUDA(ctx, cudaMemcpyAsync(st.d_pairs, st.h_pairs, nb * sizeof(wfe_pair), cudaMemcpyHostToDevice, s));
                ctx->stats.h2d_bytes += pos + nb * sizeof(wfe_pair);
                L.base_off = 0;
            }
            L.ascii = st.d_ascii;
            L.pairs = st.d_pairs;
        } else {
            for (size_t i = 0; i < nb; ++i)
                if (job.p_len[b0 + i] > job.stride || job.t_len[b0 + i] > job.stride ||
                    job.p_len[b0 + i] > c.max_seq_len || job.t_len[b0 + i] > c.max_seq_len)
                    return WFE_ERR_SEQ_TOO_LONG;
            const size_t bytes = 2u * nb * job.stride;
            if (bytes + 32u > st.ascii_cap) return WFE_ERR_INVALID_ARGUMENT;
            WFE_CUDA(ctx, cudaMemcpyAsync(st.d_ascii, job.ascii + 2u * b0 * job.stride, bytes,
                                          cudaMemcpyHostToDevice, s));
            WFE_CUDA(ctx, cudaMemcpyAsync(st.d_plen, job.p_len + b0, nb * 4u, cudaMemcpyHostToDevice, s));
            WFE_CUDA(ctx, cudaMemcpyAsync(st.d_tlen, job.t_len + b0, nb * 4u, cudaMemcpyHostToDevice, s));
            ctx->stats.h2d_bytes += bytes + nb * 8u;
            L.ascii = st.d_ascii;
            L.pairs = nullptr;
            L.plen = st.d_plen;
            L.tlen = st.d_tlen;
            L.stride = job.stride;
        }
        if (out_in_place) {
            out_pages.ready(bi);
            const int r = run_chain(ctx, st, L, (uint32_t)nb, m_dist + b0,
                                    want_cigar ? m_cigar + b0 * c.cigar_stride : nullptr,
                                    status_out ? m_status + b0 : nullptr, s, nullptr, (uint32_t)b0);
            if (r != WFE_OK) return r;
        } else {
            const int r = run_chain(ctx, st, L, (uint32_t)nb, st.d_dist, st.d_cigar, st.d_status, s, nullptr,
                                    (uint32_t)b0);
            if (r != WFE_OK) return r;
            WFE_CUDA(ctx, cudaMemcpyAsync(dist_out + b0, st.d_dist, nb * 4u, cudaMemcpyDeviceToHost, s));
            ctx->stats.d2h_bytes += nb * 4u;
            if (status_out) {
                WFE_CUDA(ctx, cudaMemcpyAsync(status_out + b0, st.d_status, nb, cudaMemcpyDeviceToHost, s));
                ctx->stats.d2h_bytes += nb;
            }
            if (want_cigar) {
                WFE_CUDA(ctx, cudaMemcpyAsync(cigar_out + b0 * c.cigar_stride, st.d_cigar,
                                              nb * c.cigar_stride, cudaMemcpyDeviceToHost, s));
                ctx->stats.d2h_bytes += nb * c.cigar_stride;
            }
        }
        ctx->stats.batches++;
        ctx->stats.pairs += nb;
    }
    for (int i = 0; i < nstages; ++i) WFE_CUDA(ctx, cudaStreamSynchronize(ctx->st[i].stream));
    if (const int r = pop_launch_error(ctx)) return r;
    if (ctx->defer_dirty) {
        if (reinterpret_cast<volatile uint8_t*>(ctx->h_launch_error)[kDeferByte])
            return finish_deferred(ctx, job, n, dist_out, cigar_out, status_out);
        ctx->defer_dirty = false; /* nothing deferred, the count is still 0 */
    }
    return WFE_OK;
}

/* A host call whose chains stopped at tier 1 deferred some pairs: allocate
 * tiers 2-6's scratch, then align those pairs as a call of their own (from
 * tier 0 again: a few of a call's pairs at most, as a rule) and put their
 * results in place.  When more were deferred than the list holds, the
 * whole call runs again. */
int finish_deferred(wfe_ctx* ctx, const HostJob& job, size_t n, int32_t* dist_out, int8_t* cigar_out,
                    uint8_t* status_out)
{
    const wfe_config& c = ctx->cfg;
    uint32_t cnt = 0;
    WFE_CUDA(ctx, cudaMemcpy(&cnt, ctx->d_defer_count, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    std::vector<uint32_t> idx;
    if (cnt <= ctx->defer_cap) {
        idx.resize(cnt);
        if (cnt) WFE_CUDA(ctx, cudaMemcpy(idx.data(), ctx->d_defer, cnt * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    }
    WFE_CUDA(ctx, cudaMemset(ctx->d_defer_count, 0, sizeof(uint32_t)));
    reinterpret_cast<volatile uint8_t*>(ctx->h_launch_error)[kDeferByte] = 0u;
    ctx->defer_dirty = false;
    if (const int r = ensure_deep(ctx)) return r;
    ctx->stats.deferred_pairs += cnt;
    if (cnt > ctx->defer_cap) return align_host_checked(ctx, job, n, dist_out, cigar_out, status_out);
    std::vector<wfe_pair> sub(cnt);
    for (uint32_t k = 0; k < cnt; ++k) {
        const uint32_t j = idx[k];
        if (j >= n) return WFE_ERR_INTERNAL;
        if (job.pairs) {
            sub[k] = job.pairs[j];
        } else {
            /* the strided layout as descriptors: pattern, then text, in slot j */
            const uint64_t o = 2ull * j * job.stride;
            sub[k].p_off = o;
            sub[k].t_off = o + job.stride;
            sub[k].p_len = job.p_len[j];
            sub[k].t_len = job.t_len[j];
        }
    }
    const size_t stride = c.cigar_stride;
    const bool want_cigar = cigar_out && stride;
    std::vector<int32_t> d(cnt);
    std::vector<int8_t> cg(want_cigar ? (size_t)cnt * stride : 0u);
    std::vector<uint8_t> st(cnt);
    const HostJob sj{job.ascii, job.ascii_bytes, sub.data(), 0, nullptr, nullptr};
    if (const int r = align_host_checked(ctx, sj, cnt, d.data(), want_cigar ? cg.data() : nullptr, st.data()))
        return r;
    for (uint32_t k = 0; k < cnt; ++k) {
        const uint32_t j = idx[k];
        dist_out[j] = d[k];
        if (want_cigar) std::memcpy(cigar_out + (size_t)j * stride, cg.data() + (size_t)k * stride, stride);
        if (status_out) status_out[j] = st[k];
    }
    return WFE_OK;
}

}  // namespace

extern "C" {

int wfe_align(wfe_ctx* ctx, const char* ascii, size_t ascii_bytes, const wfe_pair* pairs, size_t n,
              int32_t* dist_out, int8_t* cigar_out, uint8_t* status_out)
{
    if (!ctx || (n && (!ascii || !pairs || !dist_out))) return WFE_ERR_INVALID_ARGUMENT;
    HostJob j{ascii, ascii_bytes, pairs, 0, nullptr, nullptr};
    return align_host(ctx, j, n, dist_out, cigar_out, status_out);
}

int wfe_align_strided(wfe_ctx* ctx, const char* ascii, size_t stride, const uint32_t* p_len,
                      const uint32_t* t_len, size_t n, int32_t* dist_out, int8_t* cigar_out,
                      uint8_t* status_out)
{
    if (!ctx || (n && (!ascii || !p_len || !t_len || !dist_out || stride == 0)))
        return WFE_ERR_INVALID_ARGUMENT;
    HostJob j{ascii, 2u * n * stride, nullptr, stride, p_len, t_len};
    return align_host(ctx, j, n, dist_out, cigar_out, status_out);
}

int wfe_pack_device(const char* d_ascii, const wfe_pair* d_pairs, size_t n, uint32_t* d_words,
                    uint32_t words_per_seq, void* stream)
{
    if (n && (!d_ascii || !d_pairs || !d_words || words_per_seq == 0)) return WFE_ERR_INVALID_ARGUMENT;
    Layout L{};
    L.ascii = d_ascii;
    L.pairs = d_pairs;
    const cudaError_t e = launch_pack(L, (uint32_t)n, d_words, words_per_seq, (cudaStream_t)stream);
    return e == cudaSuccess ? WFE_OK : WFE_ERR_CUDA;
}

int wfe_cigar_from_history_device(const char* d_ascii, const wfe_pair* d_pairs, size_t n,
                                  uint32_t max_len, const int32_t* d_dist, const uint64_t* d_history,
                                  int8_t* d_cigar, uint32_t cigar_stride, uint8_t* d_status,
                                  void* stream)
{
    if (n && (!d_ascii || !d_pairs || !d_dist || !d_history || (!d_cigar && cigar_stride)))
        return WFE_ERR_INVALID_ARGUMENT;
    Layout L{};
    L.ascii = d_ascii;
    L.pairs = d_pairs;
    const cudaError_t e = launch_cigar_from_history(L, (uint32_t)n, max_len, d_dist, d_history, d_cigar,
                                                    cigar_stride, d_status, (cudaStream_t)stream);
    return e == cudaSuccess ? WFE_OK : WFE_ERR_CUDA;
}

}  // extern "C"

extern "C" {

int wfe_device_count(int* count)
{
    if (!count) return WFE_ERR_INVALID_ARGUMENT;
    *count = 0;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return WFE_ERR_NO_DEVICE;
    }
    *count = n;
    return n > 0 ? WFE_OK : WFE_ERR_NO_DEVICE;
}

int wfe_device_name(int device, char* name, size_t cap, int* cc_major, int* cc_minor)
{
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        cudaGetLastError();
        return WFE_ERR_NO_DEVICE;
    }
    if (name && cap) {
        std::strncpy(name, prop.name, cap - 1);
        name[cap - 1] = 0;
    }
    if (cc_major) *cc_major = prop.major;
    if (cc_minor) *cc_minor = prop.minor;
    return WFE_OK;
}

int wfe_host_alloc(void** p, size_t bytes)
{
    if (!p) return WFE_ERR_INVALID_ARGUMENT;
    *p = nullptr;
    const cudaError_t e = cudaMallocHost(p, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? WFE_ERR_OUT_OF_MEMORY : WFE_ERR_CUDA;
    }
    return WFE_OK;
}

void wfe_host_free(void* p)
{
    if (p) cudaFreeHost(p);
}

}  // extern "C"

/* ---- autotuner ------------------------------------------------------------ */

namespace {

/* One cache line per tuned context, JSON:
 * {"gpu": "...", "max_seq_len": L, "cigar_stride": S, "buckets": [...], "first_tier": [...]} */
std::string cache_key(const wfe_ctx* ctx, const char* gpu, uint32_t nb, const uint32_t* bmax, uint32_t flags)
{
    std::ostringstream k;
    k << "{\"gpu\": \"" << gpu << "\", \"max_seq_len\": " << ctx->cfg.max_seq_len
      << ", \"cigar_stride\": " << ctx->cfg.cigar_stride << ", \"flags\": " << flags << ", \"buckets\": [";
    for (uint32_t b = 0; b < nb; ++b) k << (b ? ", " : "") << (b + 1 == nb ? ctx->cfg.max_seq_len : bmax[b]);
    k << "], \"first_tier\": [";
    return k.str();
}

bool cache_lookup(const char* path, const std::string& key, uint32_t nb, int32_t* tiers)
{
    if (!path) return false;
    std::ifstream f(path);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        if (line.compare(0, key.size(), key) != 0) continue;
        std::istringstream in(line.substr(key.size()));
        uint32_t b = 0;
        for (; b < nb; ++b) {
            int v = -1;
            char sep = 0;
            if (!(in >> v)) break;
            tiers[b] = v;
            in >> sep;
        }
        found = (b == nb); /* the last matching line wins */
    }
    return found;
}

void cache_store(const char* path, const std::string& key, uint32_t nb, const int32_t* tiers)
{
    if (!path) return;
    std::ofstream f(path, std::ios::app);
    f << key;
    for (uint32_t b = 0; b < nb; ++b) f << (b ? ", " : "") << tiers[b];
    f << "]}\n";
}

}  // namespace

extern "C" int wfe_autotune(wfe_ctx* ctx, const char* d_ascii, const wfe_pair* d_pairs, size_t n,
                            uint32_t nbuckets, const uint32_t* bucket_max_len, uint32_t flags,
                            const char* cache_path, int32_t* first_tier_out)
{
    if (!ctx || !d_ascii || !d_pairs || n == 0 || nbuckets < 1 || nbuckets > (uint32_t)kMaxBuckets ||
        !bucket_max_len)
        return WFE_ERR_INVALID_ARGUMENT;
    const wfe_config& c = ctx->cfg;
    WFE_CUDA(ctx, cudaSetDevice(c.device));
    cudaDeviceProp prop{};
    WFE_CUDA(ctx, cudaGetDeviceProperties(&prop, c.device));
    const std::string key = cache_key(ctx, prop.name, nbuckets, bucket_max_len, flags);
    int32_t best[kMaxBuckets];
    if (cache_lookup(cache_path, key, nbuckets, best)) {
        const int r = wfe_set_policy(ctx, nbuckets, bucket_max_len, best, flags);
        if (r == WFE_OK && first_tier_out)
            for (uint32_t b = 0; b < nbuckets; ++b) first_tier_out[b] = best[b];
        if (r == WFE_OK) return WFE_OK; /* a stale entry falls through to tuning */
    }
    /* start from the length defaults, then time every usable first tier of
     * every bucket on up to kSample of the given pairs that fall in it, run
     * through the same routing and chains as a real batch */
    int r = wfe_set_policy(ctx, nbuckets, bucket_max_len, nullptr, flags);
    if (r != WFE_OK) return r;
    /* the trials start chains at every tier */
    if ((r = ensure_deep(ctx)) != WFE_OK) return r;
    constexpr size_t kSample = 4096;
    const size_t ns = std::min<size_t>(n, std::max<size_t>(kSample * nbuckets, 65536));
    std::vector<wfe_pair> host(ns);
    WFE_CUDA(ctx, cudaMemcpy(host.data(), d_pairs, ns * sizeof(wfe_pair), cudaMemcpyDeviceToHost));
    std::vector<std::vector<wfe_pair>> sample(nbuckets);
    for (size_t i = 0; i < ns; ++i) {
        const uint32_t len = std::max(host[i].p_len, host[i].t_len);
        if (len > c.max_seq_len) continue;
        uint32_t b = 0;
        while (b + 1 < nbuckets && len > ctx->bucket[b].max_len) ++b;
        if (sample[b].size() < std::min<size_t>(kSample, c.batch_size)) sample[b].push_back(host[i]);
    }
    wfe_pair* d_sample = nullptr;
    int32_t* d_dist = nullptr;
    int8_t* d_cigar = nullptr;
    uint8_t* d_status = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    Stage& st = ctx->st[0];
    cudaStream_t s = st.stream;
    auto cleanup = [&]() {
        cudaFree(d_sample); cudaFree(d_dist); cudaFree(d_cigar); cudaFree(d_status);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t e = cudaSuccess;
    if ((e = cudaMalloc(&d_sample, kSample * sizeof(wfe_pair))) != cudaSuccess ||
        (e = cudaMalloc(&d_dist, kSample * sizeof(int32_t))) != cudaSuccess ||
        (e = cudaMalloc(&d_cigar, kSample * (size_t)c.cigar_stride + 16)) != cudaSuccess ||
        (e = cudaMalloc(&d_status, kSample)) != cudaSuccess || (e = cudaEventCreate(&e0)) != cudaSuccess ||
        (e = cudaEventCreate(&e1)) != cudaSuccess) {
        cleanup();
        return fail_cuda(ctx, e);
    }
    /* tuning runs do not count in the statistics */
    const wfe_stats saved = ctx->stats;
    uint64_t saved_entered[kNumTiers];
    std::copy(ctx->single_entered, ctx->single_entered + kNumTiers, saved_entered);
    unsigned long long saved_dev[2 * kNumTiers + kMaxBuckets];
    if ((e = cudaMemcpy(saved_dev, ctx->d_passed, sizeof saved_dev, cudaMemcpyDeviceToHost)) != cudaSuccess) {
        cleanup();
        return fail_cuda(ctx, e);
    }
    int tiers[kMaxBuckets];
    for (uint32_t b = 0; b < nbuckets; ++b) best[b] = tiers[b] = ctx->bucket[b].first_tier;
    for (uint32_t b = 0; b < nbuckets; ++b) {
        if (sample[b].empty()) continue;
        const uint32_t m = (uint32_t)sample[b].size();
        e = cudaMemcpy(d_sample, sample[b].data(), m * sizeof(wfe_pair), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { cleanup(); return fail_cuda(ctx, e); }
        Layout L{};
        L.ascii = d_ascii;
        L.pairs = d_sample;
        const BucketPlan& bp = ctx->bucket[b];
        float best_ms = 1e30f;
        for (int t = 0; t <= bp.last_tier; ++t) {
            BucketPlan trial = bp;
            trial.first_tier = t;
            if (!bucket_usable(trial)) continue;
            tiers[b] = t;
            float ms_min = 1e30f;
            for (int rep = 0; rep < 3; ++rep) {
                cudaEventRecord(e0, s);
                r = run_chain(ctx, st, L, m, d_dist, d_cigar, d_status, s, tiers);
                cudaEventRecord(e1, s);
                if (r != WFE_OK || cudaEventSynchronize(e1) != cudaSuccess) { r = WFE_ERR_CUDA; break; }
                if ((r = pop_launch_error(ctx)) != WFE_OK) break;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0) ms_min = std::min(ms_min, ms); /* the first run warms up */
            }
            if (r != WFE_OK) { cleanup(); return r; }
            if (ms_min < best_ms) {
                best_ms = ms_min;
                best[b] = t;
            }
        }
        tiers[b] = best[b];
    }
    cleanup();
    ctx->stats = saved;
    std::copy(saved_entered, saved_entered + kNumTiers, ctx->single_entered);
    WFE_CUDA(ctx, cudaMemcpy(ctx->d_passed, saved_dev, sizeof saved_dev, cudaMemcpyHostToDevice));
    for (auto& t : ctx->timed) { ctx->event_pool.push_back(t.start); ctx->event_pool.push_back(t.stop); }
    ctx->timed.clear();
    r = wfe_set_policy(ctx, nbuckets, bucket_max_len, best, flags);
    if (r != WFE_OK) return r;
    cache_store(cache_path, key, nbuckets, best);
    if (first_tier_out)
        for (uint32_t b = 0; b < nbuckets; ++b) first_tier_out[b] = best[b];
    return WFE_OK;
}

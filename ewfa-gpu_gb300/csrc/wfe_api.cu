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
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "wfe.h"
#include "wfe_kernels.cuh"

using namespace wfe;

namespace {

constexpr int kStages = 2;

struct Stage {
    cudaStream_t stream = nullptr;
    char* d_ascii = nullptr;
    size_t ascii_cap = 0;
    wfe_pair* d_pairs = nullptr;
    uint32_t* d_plen = nullptr;
    uint32_t* d_tlen = nullptr;
    int32_t* d_dist = nullptr;
    int8_t* d_cigar = nullptr;
    uint8_t* d_status = nullptr;
    uint32_t* d_lists = nullptr;  /* two retry lists of batch_size entries */
    uint32_t* d_counts = nullptr; /* one retry counter per tier */
    char* h_stage = nullptr;      /* pinned gather buffer for scattered inputs */
    wfe_pair* h_pairs = nullptr;  /* pinned descriptors of a gathered batch */
};

thread_local int g_last_create_error = 0;

}  // namespace

struct TimedLaunch {
    int tier;
    cudaEvent_t start, stop;
};

struct wfe_ctx {
    wfe_config cfg{};
    int sm_count = 0;
    int first_tier = 0;
    int last_tier = 0;      /* 5, or 6 when sequences can be longer than kLongSmemDistance */
    int grid[kNumTiers] = {};
    TierShape shape[kNumTiers] = {};
    unsigned char* d_ops_scratch = nullptr;
    size_t ops_scratch_bytes = 0;
    unsigned long long* d_passed = nullptr;   /* pairs each tier handed on, running total */
    unsigned long long* d_launched = nullptr; /* tier launches made on the device */
    Stage st[kStages];
    int last_cuda_error = 0;
    wfe_stats stats{};
    std::vector<TimedLaunch> timed;      /* launches whose events are not read yet */
    std::vector<cudaEvent_t> event_pool;
};

namespace {

int fail_cuda(wfe_ctx* ctx, cudaError_t e)
{
    if (ctx) ctx->last_cuda_error = (int)e;
    return e == cudaErrorMemoryAllocation ? WFE_ERR_OUT_OF_MEMORY : WFE_ERR_CUDA;
}

#define WFE_CUDA(ctx, call)                                        \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return fail_cuda((ctx), e_);        \
    } while (0)

uint32_t default_cigar_stride(uint32_t max_seq_len)
{
    /* src/wavefront.cuh:48-50: seq_len + (4 - seq_len % 4) */
    return max_seq_len + (4u - max_seq_len % 4u);
}

/* First tier by sequence length: short reads almost always finish in the
 * 8-lane tier; long reads start where their distances usually are. */
int default_first_tier(uint32_t max_len)
{
    if (max_len <= 1200) return 0;
    if (max_len <= 2000) return 2;
    return 3;
}

void free_stage(Stage& s)
{
    cudaFree(s.d_ascii);
    cudaFree(s.d_pairs);
    cudaFree(s.d_plen);
    cudaFree(s.d_tlen);
    cudaFree(s.d_dist);
    cudaFree(s.d_cigar);
    cudaFree(s.d_status);
    cudaFree(s.d_lists);
    cudaFree(s.d_counts);
    cudaFreeHost(s.h_stage);
    cudaFreeHost(s.h_pairs);
    if (s.stream) cudaStreamDestroy(s.stream);
    s = Stage();
}

/* Enqueue the alignment of work items 0..n-1 of one batch on stream s: the
 * first tier is launched here; each tier's last CTA launches the next tier
 * on the device, and only when it handed pairs on. */
int run_chain(wfe_ctx* ctx, Stage& st, const Layout& L, uint32_t n, int32_t* dist, int8_t* cigar,
              uint8_t* status, cudaStream_t s)
{
    if (n == 0) return WFE_OK;
    const wfe_config& c = ctx->cfg;
    WFE_CUDA(ctx, cudaMemsetAsync(st.d_counts, 0, sizeof(uint32_t) * 2 * kNumTiers, s));
    const uint32_t B = c.batch_size;
    const int t = ctx->first_tier;
    AlignLaunch a{};
    a.L = L;
    a.work = nullptr;
    a.work_count = nullptr;
    a.n_work = n;
    a.dist = dist;
    a.cigar = cigar;
    a.cigar_stride = c.cigar_stride;
    a.status = status;
    a.max_distance = c.max_distance;
    a.max_len = c.max_seq_len;
    a.retry_count = st.d_counts + t;
    a.passed_total = ctx->d_passed + t;
    a.ops_scratch = ctx->d_ops_scratch;
    a.ops_scratch_bytes = ctx->ops_scratch_bytes;
    a.tier = t;
    /* a distance cap at or below a tier's capacity ends the chain there */
    int last = ctx->last_tier;
    if (c.max_distance > 0)
        for (int u = t; u < kNumTiers; ++u)
            if (c.max_distance <= tier_info(u).dcap) { last = u; break; }
    a.chain.last_tier = last;
    a.retry = t < last ? st.d_lists : nullptr;
    for (int u = 0; u < kNumTiers; ++u) a.chain.shape[u] = ctx->shape[u];
    a.chain.lists[0] = st.d_lists;
    a.chain.lists[1] = st.d_lists + B;
    a.chain.counts = st.d_counts;
    a.chain.cta_done = st.d_counts + kNumTiers;
    a.chain.launched = ctx->d_launched;
    const TierInfo& ti = tier_info(t);
    const uint32_t per_cta = t >= 5 ? 1u : 4u * (32u / (uint32_t)ti.G);
    int grid = (int)std::min<uint64_t>((uint64_t)ctx->grid[t], ((uint64_t)n + per_cta - 1) / per_cta);
    grid = std::max(grid, 1);
    TimedLaunch tl{t, nullptr, nullptr};
    const bool timing = (c.flags & WFE_FLAG_KERNEL_TIMING) != 0;
    if (timing) {
        for (cudaEvent_t* ev : {&tl.start, &tl.stop}) {
            if (!ctx->event_pool.empty()) {
                *ev = ctx->event_pool.back();
                ctx->event_pool.pop_back();
            } else {
                WFE_CUDA(ctx, cudaEventCreate(ev));
            }
        }
        WFE_CUDA(ctx, cudaEventRecord(tl.start, s));
    }
    WFE_CUDA(ctx, launch_tier(t, a, grid, s));
    if (timing) {
        WFE_CUDA(ctx, cudaEventRecord(tl.stop, s));
        ctx->timed.push_back(tl);
    }
    ctx->stats.kernel_launches++;
    ctx->stats.tier_launches[t]++;
    ctx->stats.tier_entered[t] += n;
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

int wfe_create(const wfe_config* cfg, wfe_ctx** out)
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
    ctx->first_tier = default_first_tier(c.max_seq_len);

    auto bail = [&](cudaError_t err) {
        g_last_create_error = (int)err;
        for (auto& s : ctx->st) free_stage(s);
        cudaFree(ctx->d_ops_scratch);
        cudaFree(ctx->d_passed);
        for (auto& sh : ctx->shape) cudaFree(sh.scratch);
        delete ctx;
        return err == cudaErrorMemoryAllocation ? WFE_ERR_OUT_OF_MEMORY : WFE_ERR_CUDA;
    };

    e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, c.device);
    if (e != cudaSuccess) return bail(e);
    size_t scratch = 0;
    ctx->last_tier = c.max_seq_len > (uint32_t)kLongSmemDistance ? 6 : 5;
    for (int t = 0; t < kNumTiers; ++t) {
        ctx->shape[t] = tier_shape(t, c.max_seq_len, c.cigar_stride, ctx->sm_count);
        ctx->grid[t] = ctx->shape[t].grid;
        if (ctx->grid[t] <= 0) { /* sequences too long for this tier's shared memory */
            if (t >= ctx->first_tier && t <= ctx->last_tier) return bail(cudaErrorInvalidValue);
            continue;
        }
        if (t < 5) scratch = std::max(scratch, tier_scratch_bytes(t, ctx->grid[t]));
    }
    /* tiers 5-6: a scratch slab per resident CTA (backtrace store, chain,
     * runs; tier 6 also its wavefront), the grid trimmed to a budget */
    for (int t = 5; t <= ctx->last_tier; ++t) {
        TierShape& sh = ctx->shape[t];
        const uint64_t budget = t == 5 ? (2ull << 30) : (8ull << 30);
        const uint64_t fit = std::max<uint64_t>(1, budget / sh.slab);
        sh.grid = (int)std::min<uint64_t>((uint64_t)sh.grid, fit);
        ctx->grid[t] = sh.grid;
        if ((e = cudaMalloc(&sh.scratch, (size_t)sh.slab * sh.grid)) != cudaSuccess) return bail(e);
    }
    if (scratch) {
        e = cudaMalloc(&ctx->d_ops_scratch, scratch);
        if (e != cudaSuccess) return bail(e);
        ctx->ops_scratch_bytes = scratch;
    }
    if ((e = cudaMalloc(&ctx->d_passed, sizeof(unsigned long long) * 2 * kNumTiers)) != cudaSuccess) return bail(e);
    if ((e = cudaMemset(ctx->d_passed, 0, sizeof(unsigned long long) * 2 * kNumTiers)) != cudaSuccess) return bail(e);
    ctx->d_launched = ctx->d_passed + kNumTiers;
    const size_t B = c.batch_size;
    for (auto& s : ctx->st) {
        s.ascii_cap = B * 2u * (size_t)c.max_seq_len + 64u;
        if ((e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&s.d_ascii, s.ascii_cap)) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&s.d_pairs, B * sizeof(wfe_pair))) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&s.d_plen, B * sizeof(uint32_t))) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&s.d_tlen, B * sizeof(uint32_t))) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&s.d_dist, B * sizeof(int32_t))) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&s.d_cigar, B * (size_t)c.cigar_stride + 16u)) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&s.d_status, B)) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&s.d_lists, 2u * B * sizeof(uint32_t))) != cudaSuccess) return bail(e);
        if ((e = cudaMalloc(&s.d_counts, sizeof(uint32_t) * 2 * kNumTiers)) != cudaSuccess) return bail(e);
    }
    *out = ctx;
    return WFE_OK;
}

void wfe_destroy(wfe_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->cfg.device);
    for (auto& s : ctx->st) {
        if (s.stream) cudaStreamSynchronize(s.stream);
        free_stage(s);
    }
    cudaFree(ctx->d_ops_scratch);
    cudaFree(ctx->d_passed);
    for (auto& sh : ctx->shape) cudaFree(sh.scratch);
    for (auto& t : ctx->timed) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    for (auto ev : ctx->event_pool) cudaEventDestroy(ev);
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
    unsigned long long dev[2 * kNumTiers] = {};
    WFE_CUDA(ctx, cudaMemcpy(dev, ctx->d_passed, sizeof(dev), cudaMemcpyDeviceToHost));
    *out = ctx->stats;
    for (int t = 0; t < kNumTiers; ++t) {
        out->tier_passed[t] = dev[t];
        if (t > ctx->first_tier) out->tier_entered[t] = dev[t - 1];
        out->tier_launches[t] += dev[kNumTiers + t];
        out->kernel_launches += dev[kNumTiers + t];
    }
    return WFE_OK;
}

int wfe_reset_stats(wfe_ctx* ctx)
{
    if (!ctx) return WFE_ERR_INVALID_ARGUMENT;
    wfe_stats tmp;
    const int r = wfe_get_stats(ctx, &tmp); /* drains pending timings */
    if (r != WFE_OK) return r;
    ctx->stats = wfe_stats{};
    WFE_CUDA(ctx, cudaMemset(ctx->d_passed, 0, sizeof(unsigned long long) * 2 * kNumTiers));
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
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->st[0].stream;
    const size_t B = ctx->cfg.batch_size;
    for (size_t b0 = 0; b0 < n; b0 += B) {
        const uint32_t nb = (uint32_t)std::min(B, n - b0);
        Layout L{};
        L.ascii = d_ascii;
        L.pairs = d_pairs + b0;
        L.base_off = 0;
        const int r = run_chain(ctx, ctx->st[0], L, nb, d_dist + b0,
                                d_cigar ? d_cigar + b0 * ctx->cfg.cigar_stride : nullptr,
                                d_status ? d_status + b0 : nullptr, s);
        if (r != WFE_OK) return r;
        ctx->stats.batches++;
        ctx->stats.pairs += nb;
    }
    return WFE_OK;
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

/* Device address of a pinned, device-mapped host buffer (NULL when p is
 * pageable or not host memory). */
void* mapped_address(const void* p)
{
    if (!p) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError(); /* pageable memory of an older driver: not mapped */
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int align_host(wfe_ctx* ctx, const HostJob& job, size_t n, int32_t* dist_out, int8_t* cigar_out,
               uint8_t* status_out)
{
    const wfe_config& c = ctx->cfg;
    WFE_CUDA(ctx, cudaSetDevice(c.device));
    const bool want_cigar = cigar_out && c.cigar_stride;

    /* pinned inputs are read in place, pinned outputs written in place */
    const char* m_ascii = (const char*)mapped_address(job.ascii);
    const wfe_pair* m_pairs = job.pairs ? (const wfe_pair*)mapped_address(job.pairs) : nullptr;
    const uint32_t* m_plen = job.pairs ? nullptr : (const uint32_t*)mapped_address(job.p_len);
    const uint32_t* m_tlen = job.pairs ? nullptr : (const uint32_t*)mapped_address(job.t_len);
    const bool in_place = m_ascii && job.ascii_bytes > 0 && (job.pairs ? m_pairs != nullptr : (m_plen && m_tlen));
    int32_t* m_dist = (int32_t*)mapped_address(dist_out);
    int8_t* m_cigar = want_cigar ? (int8_t*)mapped_address(cigar_out) : nullptr;
    uint8_t* m_status = status_out ? (uint8_t*)mapped_address(status_out) : nullptr;
    const bool out_in_place = m_dist && (!want_cigar || m_cigar) && (!status_out || m_status);

    size_t B = c.batch_size;
    if (!job.pairs && !in_place) {
        /* strided slots may be wider than max_seq_len: fewer pairs per batch */
        const size_t fit = (ctx->st[0].ascii_cap - 32u) / (2u * job.stride);
        if (fit == 0) return WFE_ERR_SEQ_TOO_LONG;
        B = std::min(B, fit);
    }
    const int nstages = (c.flags & WFE_FLAG_NO_PIPELINE) ? 1 : kStages;
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
            const int r = run_chain(ctx, st, L, (uint32_t)nb, m_dist + b0,
                                    want_cigar ? m_cigar + b0 * c.cigar_stride : nullptr,
                                    status_out ? m_status + b0 : nullptr, s);
            if (r != WFE_OK) return r;
        } else {
            const int r = run_chain(ctx, st, L, (uint32_t)nb, st.d_dist, st.d_cigar, st.d_status, s);
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

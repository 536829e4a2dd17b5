/*
 * wfe_server.cu -- continuous batching of alignment requests on one GPU
 * (wfe_server_* / wfe_submit / wfe_poll in wfe.h).
 *
 * The reference aligns one file in fixed batches from a handful of host
 * threads (src/aligner.cu:40-71, src/wavefront.cu:173-208); it has no
 * request path.  Here requests of any size arrive from any thread and a
 * scheduler thread packs whatever is waiting into device batches:
 *
 *   lanes     `lanes` streams, each with its own alignment context (work
 *             lists, tier scratch, slabs of the CTA-per-pair tiers) created
 *             once, so that batches of different lanes overlap on the device
 *             without sharing scratch;
 *   arenas    a device arena holds every batch's descriptors and sequences,
 *             a page-locked, device-mapped host arena its rebased
 *             descriptors, gathered sequences, and the distances, statuses
 *             and CIGAR slots that the kernels write in place; a batch takes
 *             one block of each (first fit) and returns them when it ends;
 *   admission a batch is formed when a lane is free: requests are taken in
 *             arrival order while the batch still fits the largest free
 *             block of both arenas and `batch_pairs`; a request that does
 *             not fit whole is split, its remaining pairs leading the next
 *             batch;
 *   results   a host function queued behind each batch wakes one of up to
 *             four finisher threads, which copies every request's share of
 *             the results into the caller's buffers, finishes the requests
 *             that are complete and frees the batch's lane, while the
 *             scheduler goes on admitting.
 *
 * Sequences reach the device as one copy per request share: the share's
 * span of the caller's buffer when its pairs lie close together (pinned
 * memory is read by DMA), else gathered pair by pair into the host arena.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <iterator>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "wfe.h"
#include "wfe_internal.h"

namespace {

constexpr uint64_t kAlign = 256;
constexpr uint64_t kSeqPad = 32; /* readable bytes after a batch's last sequence */

inline uint64_t up(uint64_t x, uint64_t a) { return (x + a - 1) / a * a; }

uint64_t now_ns()
{
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

/* First-fit allocator over [0, size): free blocks by offset, coalesced on
 * release.  Offsets and sizes are multiples of kAlign. */
class Arena {
  public:
    void reset(uint64_t size)
    {
        free_.clear();
        size_ = size;
        if (size) free_[0] = size;
    }
    uint64_t largest() const
    {
        uint64_t m = 0;
        for (const auto& f : free_) m = std::max(m, f.second);
        return m;
    }
    uint64_t held() const
    {
        uint64_t f = 0;
        for (const auto& b : free_) f += b.second;
        return size_ - f;
    }
    bool alloc(uint64_t bytes, uint64_t* off)
    {
        bytes = up(std::max<uint64_t>(bytes, 1), kAlign);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            *off = it->first;
            const uint64_t rest = it->second - bytes, at = it->first + bytes;
            free_.erase(it);
            if (rest) free_[at] = rest;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t bytes)
    {
        bytes = up(std::max<uint64_t>(bytes, 1), kAlign);
        auto next = free_.lower_bound(off);
        if (next != free_.end() && off + bytes == next->first) {
            bytes += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += bytes;
                return;
            }
        }
        free_[off] = bytes;
    }

  private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t size_ = 0;
};

struct Request {
    uint64_t id = 0;
    const char* ascii = nullptr;
    size_t ascii_bytes = 0;
    const wfe_pair* pairs = nullptr;
    size_t n = 0;
    int32_t* dist = nullptr;
    int8_t* cigar = nullptr;
    uint8_t* status = nullptr;
    bool span_mode = false;  /* shares are copied as spans of the caller's buffer */
    size_t next = 0;         /* pairs handed to batches */
    size_t finished = 0;     /* pairs whose results are in the caller's buffers */
    uint32_t batches = 0;
    int rc = WFE_OK;
    bool done = false;
    uint64_t submit_ns = 0, start_ns = 0, done_ns = 0;
};

/* A request's share of a batch. */
struct Share {
    Request* r;
    size_t first, count;  /* the request's pairs [first, first + count) */
    uint32_t slot;        /* their first slot in the batch */
    uint64_t lo, hi;      /* span mode: bytes [lo, hi) of the caller's buffer */
    uint64_t dev_at;      /* where the share's sequences start in the batch's device block */
    uint64_t host_at;     /* gather mode: where they are gathered in the host block */
    uint64_t bytes;       /* sequence bytes copied */
};

struct Batch {
    wfe_server* srv = nullptr;
    int lane = -1;
    uint64_t dev_off = 0, dev_bytes = 0, host_off = 0, host_bytes = 0;
    uint32_t n = 0;
    uint64_t seq_dev = 0;   /* device bytes of sequences */
    uint64_t seq_host = 0;  /* host bytes of gathered sequences */
    std::vector<Share> shares;
    int rc = WFE_OK;
};

struct Lane {
    wfe_ctx* ctx = nullptr;
    cudaStream_t stream = nullptr;
    bool busy = false;
};

}  // namespace

struct wfe_server {
    wfe_server_config cfg{};
    uint32_t stride = 0;
    std::vector<Lane> lanes;
    char* d_arena = nullptr;
    char* h_arena = nullptr;     /* page-locked, device-mapped */
    char* h_arena_dev = nullptr; /* its device address */
    uint64_t host_arena_bytes = 0;
    Arena dev, host;
    std::mutex mu;
    std::condition_variable cv_work;   /* scheduler: requests arrived or a lane came free */
    std::condition_variable cv_finish; /* finishers: a batch's host function ran */
    std::condition_variable cv_done;   /* pollers: requests finished */
    std::deque<Request*> pending;
    std::unordered_map<uint64_t, Request*> tickets;
    std::deque<Batch*> finished;       /* batches whose host function ran, oldest first */
    uint64_t next_id = 1;
    uint32_t in_flight = 0;
    bool stopping = false;
    bool finishers_stop = false;
    wfe_server_stats stats{};
    std::thread scheduler;
    /* Copying a batch's results into the callers' buffers takes several times
     * as long as admitting one, so it runs on these threads, not on the
     * scheduler's: the next batch is admitted while the last one's results
     * are copied out. */
    std::vector<std::thread> finishers;
};

namespace {

/* Bytes of a batch of n pairs and `seq` device sequence bytes in the device
 * arena: descriptors, then sequences. */
uint64_t dev_block(uint64_t n, uint64_t seq) { return up(n * sizeof(wfe_pair), kAlign) + up(seq + kSeqPad, kAlign); }

/* ... and in the host arena: rebased descriptors, gathered sequences,
 * distances, statuses, CIGAR slots. */
uint64_t host_block(uint64_t n, uint64_t gathered, uint32_t stride)
{
    return up(n * sizeof(wfe_pair), kAlign) + up(gathered, kAlign) + up(n * 4u, kAlign) + up(n, kAlign) +
           up(n * (uint64_t)stride, kAlign);
}

struct HostLayout {
    wfe_pair* pairs;
    char* seq;
    int32_t* dist;
    uint8_t* status;
    int8_t* cigar;
};

HostLayout host_layout(char* base, uint64_t n, uint64_t gathered)
{
    HostLayout h{};
    uint64_t at = 0;
    h.pairs = reinterpret_cast<wfe_pair*>(base + at);
    at += up(n * sizeof(wfe_pair), kAlign);
    h.seq = base + at;
    at += up(gathered, kAlign);
    h.dist = reinterpret_cast<int32_t*>(base + at);
    at += up(n * 4u, kAlign);
    h.status = reinterpret_cast<uint8_t*>(base + at);
    at += up(n, kAlign);
    h.cigar = reinterpret_cast<int8_t*>(base + at);
    return h;
}

void CUDART_CB batch_done(void* arg)
{
    Batch* b = static_cast<Batch*>(arg);
    wfe_server* s = b->srv;
    std::lock_guard<std::mutex> lk(s->mu);
    s->finished.push_back(b);
    s->cv_finish.notify_one();
}

/* Take waiting requests into a batch for a free lane (called with the lock
 * held).  nullptr when nothing waits, no lane is free, or not one more pair
 * fits the free memory. */
Batch* form_batch(wfe_server* s)
{
    int lane = -1;
    for (size_t i = 0; i < s->lanes.size(); ++i)
        if (!s->lanes[i].busy) { lane = (int)i; break; }
    if (lane < 0 || s->pending.empty()) return nullptr;
    const uint64_t dev_free = s->dev.largest(), host_free = s->host.largest();
    const uint64_t cap = s->cfg.batch_pairs;
    std::vector<Share> shares;
    uint64_t n = 0, seq_dev = 0, seq_host = 0;
    bool full = false;
    for (size_t qi = 0; qi < s->pending.size() && !full && n < cap; ++qi) {
        Request* r = s->pending[qi];
        Share sh{r, r->next, 0, (uint32_t)n, 0, 0, seq_dev, seq_host, 0};
        uint64_t lo = UINT64_MAX, hi = 0;
        for (size_t i = r->next; i < r->n; ++i) {
            if (n + sh.count >= cap) { full = true; break; }
            const wfe_pair& q = r->pairs[i];
            uint64_t nlo = lo, nhi = hi, bytes, add_dev, add_host;
            if (r->span_mode) {
                nlo = std::min(lo, std::min(q.p_off, q.t_off));
                nhi = std::max(hi, std::max(q.p_off + q.p_len, q.t_off + q.t_len));
                bytes = nhi - nlo;
                add_host = 0;
            } else {
                bytes = sh.bytes + q.p_len + q.t_len;
                add_host = bytes;
            }
            add_dev = up(bytes, 16) + kSeqPad;
            const uint64_t m = n + sh.count + 1;
            if (dev_block(m, seq_dev + add_dev) > dev_free ||
                host_block(m, seq_host + add_host, s->stride) > host_free) {
                full = true;
                break;
            }
            lo = nlo;
            hi = nhi;
            sh.bytes = bytes;
            ++sh.count;
        }
        if (sh.count == 0) break;
        sh.lo = lo;
        sh.hi = hi;
        seq_dev += up(sh.bytes, 16) + kSeqPad;
        if (!r->span_mode) seq_host += sh.bytes;
        n += sh.count;
        shares.push_back(sh);
        if (r->next + sh.count < r->n) full = true; /* the rest of it leads the next batch */
    }
    if (n == 0) return nullptr;
    Batch* b = new (std::nothrow) Batch();
    if (!b) return nullptr;
    b->srv = s;
    b->lane = lane;
    b->n = (uint32_t)n;
    b->seq_dev = seq_dev;
    b->seq_host = seq_host;
    b->dev_bytes = dev_block(n, seq_dev);
    b->host_bytes = host_block(n, seq_host, s->stride);
    /* both fit: each was checked against the largest free block */
    if (!s->dev.alloc(b->dev_bytes, &b->dev_off)) {
        delete b;
        return nullptr;
    }
    if (!s->host.alloc(b->host_bytes, &b->host_off)) {
        s->dev.release(b->dev_off, b->dev_bytes);
        delete b;
        return nullptr;
    }
    const uint64_t t = now_ns();
    for (Share& sh : shares) {
        Request* r = sh.r;
        r->next += sh.count;
        if (r->batches++ == 0) r->start_ns = t;
    }
    while (!s->pending.empty() && s->pending.front()->next == s->pending.front()->n) s->pending.pop_front();
    b->shares = std::move(shares);
    s->lanes[lane].busy = true;
    s->in_flight++;
    s->stats.max_in_flight = std::max(s->stats.max_in_flight, s->in_flight);
    s->stats.peak_memory = std::max(s->stats.peak_memory, s->dev.held());
    s->stats.batches++;
    return b;
}

/* Copy a batch's inputs to the device and enqueue its alignment (without
 * the lock: only the scheduler touches the batch and its shares' pairs). */
int launch_batch(wfe_server* s, Batch* b)
{
    Lane& L = s->lanes[b->lane];
    char* dblk = s->d_arena + b->dev_off;
    wfe_pair* d_pairs = reinterpret_cast<wfe_pair*>(dblk);
    char* d_seq = dblk + up((uint64_t)b->n * sizeof(wfe_pair), kAlign);
    HostLayout h = host_layout(s->h_arena + b->host_off, b->n, b->seq_host);
    HostLayout hd = host_layout(s->h_arena_dev + b->host_off, b->n, b->seq_host);
    for (const Share& sh : b->shares) {
        const Request* r = sh.r;
        wfe_pair* out = h.pairs + sh.slot;
        if (r->span_mode) {
            for (size_t i = 0; i < sh.count; ++i) {
                wfe_pair q = r->pairs[sh.first + i];
                q.p_off = q.p_off - sh.lo + sh.dev_at;
                q.t_off = q.t_off - sh.lo + sh.dev_at;
                out[i] = q;
            }
        } else {
            char* g = h.seq + sh.host_at;
            uint64_t pos = 0;
            for (size_t i = 0; i < sh.count; ++i) {
                wfe_pair q = r->pairs[sh.first + i];
                std::memcpy(g + pos, r->ascii + q.p_off, q.p_len);
                q.p_off = sh.dev_at + pos;
                pos += q.p_len;
                std::memcpy(g + pos, r->ascii + q.t_off, q.t_len);
                q.t_off = sh.dev_at + pos;
                pos += q.t_len;
                out[i] = q;
            }
        }
    }
    cudaError_t e = cudaMemcpyAsync(d_pairs, h.pairs, (size_t)b->n * sizeof(wfe_pair), cudaMemcpyHostToDevice,
                                    L.stream);
    for (const Share& sh : b->shares) {
        if (e != cudaSuccess) break;
        if (sh.bytes == 0) continue;
        const char* src = sh.r->span_mode ? sh.r->ascii + sh.lo : h.seq + sh.host_at;
        e = cudaMemcpyAsync(d_seq + sh.dev_at, src, sh.bytes, cudaMemcpyHostToDevice, L.stream);
    }
    if (e != cudaSuccess) return WFE_ERR_CUDA;
    int rc = wfe_align_device(L.ctx, d_seq, d_pairs, b->n, s->cfg.max_seq_len, hd.dist, hd.cigar, hd.status,
                              L.stream);
    if (rc != WFE_OK) return rc;
    if (cudaLaunchHostFunc(L.stream, batch_done, b) != cudaSuccess) return WFE_ERR_CUDA;
    return WFE_OK;
}

/* Copy a finished batch's results into the callers' buffers (without the
 * lock). */
void scatter(wfe_server* s, Batch* b)
{
    if (b->rc != WFE_OK) return;
    HostLayout h = host_layout(s->h_arena + b->host_off, b->n, b->seq_host);
    const uint32_t stride = s->stride;
    for (const Share& sh : b->shares) {
        Request* r = sh.r;
        std::memcpy(r->dist + sh.first, h.dist + sh.slot, sh.count * sizeof(int32_t));
        if (r->status) std::memcpy(r->status + sh.first, h.status + sh.slot, sh.count);
        if (r->cigar && stride) {
            for (size_t i = 0; i < sh.count; ++i) {
                const int8_t* src = h.cigar + (size_t)(sh.slot + i) * stride;
                int8_t* dst = r->cigar + (sh.first + i) * (size_t)stride;
                const void* z = std::memchr(src, 0, stride);
                const size_t len = z ? (size_t)(static_cast<const int8_t*>(z) - src) + 1 : stride;
                std::memcpy(dst, src, len);
            }
        }
    }
}

/* A batch whose host function ran: check it, copy its results out (without
 * the lock: only this thread touches the batch, and its shares' rows of the
 * callers' buffers belong to no other batch), then finish its requests and
 * free its lane and arena blocks. */
void finish_batch(wfe_server* s, Batch* b)
{
    Lane& L = s->lanes[b->lane];
    if (b->rc == WFE_OK) {
        /* the lane is busy until this batch is finished: no other thread
         * uses its context now */
        const cudaError_t q = cudaStreamQuery(L.stream);
        if (q != cudaSuccess && q != cudaErrorNotReady) b->rc = WFE_ERR_CUDA;
        else b->rc = wfe::take_launch_error(L.ctx);
    }
    const uint64_t t0 = now_ns();
    scatter(s, b);
    const uint64_t t = now_ns();
    std::lock_guard<std::mutex> lk(s->mu);
    s->stats.finish_ns += t - t0;
    for (const Share& sh : b->shares) {
        Request* r = sh.r;
        if (b->rc != WFE_OK) r->rc = b->rc;
        r->finished += sh.count;
        if (r->finished == r->n) {
            r->done = true;
            r->done_ns = t;
            s->stats.requests++;
            s->stats.pairs += r->n;
            if (r->batches > 1) s->stats.split_requests++;
        }
    }
    s->dev.release(b->dev_off, b->dev_bytes);
    s->host.release(b->host_off, b->host_bytes);
    L.busy = false;
    s->in_flight--;
    delete b;
    s->cv_done.notify_all();
    s->cv_work.notify_one();
}

void run_finisher(wfe_server* s)
{
    cudaSetDevice(s->cfg.device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv_finish.wait(lk, [s] { return !s->finished.empty() || s->finishers_stop; });
        if (s->finished.empty()) break; /* stopping, and nothing left */
        Batch* b = s->finished.front();
        s->finished.pop_front();
        lk.unlock();
        finish_batch(s, b);
        lk.lock();
    }
}

void run_scheduler(wfe_server* s)
{
    cudaSetDevice(s->cfg.device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        bool launched = false;
        for (;;) {
            const uint64_t t0 = now_ns();
            Batch* b = form_batch(s);
            if (!b) break;
            lk.unlock();
            b->rc = launch_batch(s, b);
            const uint64_t t1 = now_ns();
            if (b->rc != WFE_OK) {
                /* finishes as failed, without results, once what was queued is done */
                cudaStreamSynchronize(s->lanes[b->lane].stream);
                batch_done(b);
            }
            lk.lock();
            s->stats.admit_ns += t1 - t0;
            launched = true;
        }
        if (s->stopping && s->pending.empty() && s->in_flight == 0) break;
        if (!launched) s->cv_work.wait(lk);
    }
}

/* Stop the finishers (after the scheduler: every batch has been finished). */
void stop_finishers(wfe_server* s)
{
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->finishers_stop = true;
        s->cv_finish.notify_all();
    }
    for (auto& t : s->finishers)
        if (t.joinable()) t.join();
    s->finishers.clear();
}

void free_server(wfe_server* s)
{
    for (Lane& L : s->lanes) {
        if (L.stream) cudaStreamSynchronize(L.stream);
        wfe_destroy(L.ctx);
        if (L.stream) cudaStreamDestroy(L.stream);
    }
    cudaFree(s->d_arena);
    cudaFreeHost(s->h_arena);
    for (auto& t : s->tickets) delete t.second;
    delete s;
}

}  // namespace

extern "C" {

int wfe_server_create(const wfe_server_config* cfg, wfe_server** out)
{
    if (!cfg || !out || cfg->max_seq_len == 0 || cfg->max_distance < 0 || cfg->nbuckets > WFE_MAX_BUCKETS)
        return WFE_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    wfe_server* s = new (std::nothrow) wfe_server();
    if (!s) return WFE_ERR_OUT_OF_MEMORY;
    s->cfg = *cfg;
    wfe_server_config& c = s->cfg;
    if (c.lanes == 0) c.lanes = 4;
    if (c.batch_pairs == 0) c.batch_pairs = 65536;
    if (c.memory_bytes == 0) c.memory_bytes = 2ull << 30;
    c.memory_bytes = up(c.memory_bytes, kAlign);
    s->stride = c.cigar_stride ? c.cigar_stride : c.max_seq_len + (4u - c.max_seq_len % 4u);
    c.cigar_stride = s->stride;
    /* the host arena also holds the CIGAR slots: as many slots as the device
     * arena holds pairs of the longest sequences */
    const uint64_t longest_pair = 2ull * c.max_seq_len + 2 * kSeqPad;
    s->host_arena_bytes = up(c.memory_bytes + (c.memory_bytes / longest_pair + 1) * ((uint64_t)s->stride + 64u),
                             kAlign);
    /* one pair of the longest sequences must fit an empty arena */
    if (dev_block(1, longest_pair) > c.memory_bytes) {
        delete s;
        return WFE_ERR_INVALID_ARGUMENT;
    }
    cudaError_t e = cudaSetDevice(c.device);
    if (e != cudaSuccess) {
        delete s;
        return WFE_ERR_NO_DEVICE;
    }
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || free_b < c.memory_bytes) {
        delete s;
        return WFE_ERR_BUSY;
    }
    wfe_config lc{};
    lc.device = c.device;
    lc.max_seq_len = c.max_seq_len;
    lc.batch_size = c.batch_pairs;
    lc.max_distance = c.max_distance;
    lc.cigar_stride = s->stride;
    lc.flags = WFE_FLAG_DEVICE_ONLY;
    s->lanes.resize(c.lanes);
    for (Lane& L : s->lanes) {
        /* smaller slabs than a standalone context: lanes run side by side */
        int rc = wfe::create_context(&lc, 512ull << 20, 1ull << 30, &L.ctx);
        if (rc == WFE_OK && c.nbuckets > 0)
            rc = wfe_set_policy(L.ctx, c.nbuckets, c.bucket_max_len, c.first_tier, c.policy_flags);
        if (rc == WFE_OK && cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess)
            rc = WFE_ERR_CUDA;
        if (rc != WFE_OK) {
            free_server(s);
            return rc;
        }
    }
    if (cudaMalloc(&s->d_arena, c.memory_bytes) != cudaSuccess ||
        cudaHostAlloc(&s->h_arena, s->host_arena_bytes, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(&s->h_arena_dev, s->h_arena, 0) != cudaSuccess) {
        cudaGetLastError();
        free_server(s);
        return WFE_ERR_BUSY;
    }
    s->dev.reset(c.memory_bytes);
    s->host.reset(s->host_arena_bytes);
    s->stats.lanes = c.lanes;
    s->stats.memory_bytes = c.memory_bytes;
    try {
        const uint32_t nf = std::min<uint32_t>(c.lanes, 4u);
        for (uint32_t i = 0; i < nf; ++i) s->finishers.emplace_back(run_finisher, s);
        s->scheduler = std::thread(run_scheduler, s);
    } catch (...) {
        stop_finishers(s);
        free_server(s);
        return WFE_ERR_INTERNAL;
    }
    *out = s;
    return WFE_OK;
}

void wfe_server_destroy(wfe_server* s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->cv_work.notify_one();
    }
    if (s->scheduler.joinable()) s->scheduler.join();
    stop_finishers(s);
    cudaSetDevice(s->cfg.device);
    free_server(s);
}

int wfe_submit(wfe_server* s, const char* ascii, size_t ascii_bytes, const wfe_pair* pairs, size_t n,
               int32_t* dist_out, int8_t* cigar_out, uint8_t* status_out, uint64_t* ticket)
{
    if (!s || !ticket || (n && (!ascii || !pairs || !dist_out))) return WFE_ERR_INVALID_ARGUMENT;
    uint64_t lo = UINT64_MAX, hi = 0, seq = 0;
    for (size_t i = 0; i < n; ++i) {
        const wfe_pair& q = pairs[i];
        const uint64_t pe = q.p_off + q.p_len, te = q.t_off + q.t_len;
        if (pe < q.p_off || te < q.t_off || pe > ascii_bytes || te > ascii_bytes) return WFE_ERR_INVALID_ARGUMENT;
        if (q.p_len > s->cfg.max_seq_len || q.t_len > s->cfg.max_seq_len) return WFE_ERR_SEQ_TOO_LONG;
        lo = std::min(lo, std::min(q.p_off, q.t_off));
        hi = std::max(hi, std::max(pe, te));
        seq += (uint64_t)q.p_len + q.t_len;
    }
    Request* r = new (std::nothrow) Request();
    if (!r) return WFE_ERR_OUT_OF_MEMORY;
    r->ascii = ascii;
    r->ascii_bytes = ascii_bytes;
    r->pairs = pairs;
    r->n = n;
    r->dist = dist_out;
    r->cigar = cigar_out;
    r->status = status_out;
    /* copy spans when the pairs lie close together and any share's span
     * fits a quarter of the arena */
    r->span_mode = n > 0 && hi - lo <= 2 * seq + 4096 && hi - lo <= s->cfg.memory_bytes / 4;
    r->submit_ns = now_ns();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) {
        delete r;
        return WFE_ERR_INVALID_ARGUMENT;
    }
    r->id = s->next_id++;
    try { /* no C++ exception crosses the C ABI */
        s->tickets[r->id] = r;
        if (n > 0) s->pending.push_back(r);
    } catch (const std::bad_alloc&) {
        s->tickets.erase(r->id);
        delete r;
        return WFE_ERR_OUT_OF_MEMORY;
    }
    *ticket = r->id;
    if (n == 0) {
        r->done = true;
        r->start_ns = r->done_ns = r->submit_ns;
        s->stats.requests++;
        s->cv_done.notify_all();
        return WFE_OK;
    }
    s->cv_work.notify_one();
    return WFE_OK;
}

int wfe_poll(wfe_server* s, uint64_t ticket, int64_t timeout_us, wfe_request_info* info)
{
    if (!s) return WFE_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return WFE_ERR_NOT_FOUND;
    Request* r = it->second;
    if (!r->done && timeout_us != 0) {
        auto ready = [&] { return r->done; };
        if (timeout_us < 0) s->cv_done.wait(lk, ready);
        else s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), ready);
    }
    if (!r->done) return WFE_ERR_TIMEOUT;
    if (info) {
        info->submit_ns = r->submit_ns;
        info->start_ns = r->start_ns;
        info->done_ns = r->done_ns;
        info->pairs = (uint32_t)r->n;
        info->batches = r->batches;
    }
    const int rc = r->rc;
    s->tickets.erase(it);
    delete r;
    return rc;
}

int wfe_server_get_stats(wfe_server* s, wfe_server_stats* out)
{
    if (!s || !out) return WFE_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    return WFE_OK;
}

}  // extern "C"

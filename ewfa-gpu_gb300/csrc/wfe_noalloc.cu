/*
 * wfe_noalloc.cu -- an alignment entry point that allocates no memory.
 *
 * Some callers cannot call cudaMalloc where they align: a plugin living
 * inside a host application that owns every device allocation through its
 * own pool, a real-time loop that forbids allocation after start-up, code
 * that must run while an allocator is locked or on a memory budget that an
 * outside framework accounts for.  wfe_create allocates the context's
 * buffers, so those callers use wfe_align_device_noalloc instead.  They pass
 * device inputs and outputs; the only scratch the kernel needs, the 2-bit
 * backtrace store of the pairs in flight, lives in the fixed array below,
 * which every GPU that loads this library holds until the process exits.
 *
 * The pairs go through two of the tiers, in rounds of up to 2^20 pairs:
 * tier 0 (4 lanes per pair, distances up to 21, backtrace store in shared
 * memory, so it needs none of the array) aligns every pair, and hands the
 * ones past distance 21 on, through a list at the start of the array, to
 * the tier-3 kernel (32 lanes per pair, distances up to 271, backtrace store
 * in global memory), pointed at the rest of the array.  A pair's store there
 * takes 20,544 bytes (a triangle of 271 rows), so the rest holds the stores
 * of 612 pairs in flight, 153 CTAs of 4 pairs; that grid is sized so that
 * every resident group has its own slot (about one CTA per SM on a GB300,
 * below the kernel's occupancy: the price of the fixed size, paid only by
 * the pairs past distance 21).  With a max_distance of 21 or less tier 0
 * does all of it.
 */
#include <algorithm>
#include <mutex>

#include <cuda.h>

#include "wfe.h"
#include "wfe_kernels.cuh"

namespace {

constexpr size_t kNoallocScratchBytes = (size_t)WFE_NOALLOC_SCRATCH_BYTES;
constexpr int kFirstTier = 0;
constexpr int kNoallocTier = 3;
/* the array: the hand-on list of one round, its count, the tier-3 stores */
constexpr uint32_t kRoundPairs = 1u << 20;
constexpr size_t kListBytes = (size_t)kRoundPairs * sizeof(uint32_t);
constexpr size_t kStoresAt = kListBytes + 256u;

/* The scratch of every call on this device.  Host code must not use the
 * symbol itself as a pointer: on the host it names a stand-in, not the
 * device array; the device address comes from cudaGetSymbolAddress. */
static __device__ __align__(256) unsigned char g_noalloc_ops[kNoallocScratchBytes];

/* The array's device address belongs to one CUDA context: the primary
 * context of a device, or a context the host application created and made
 * current.  After cudaDeviceReset, or in another context of the same
 * device, the module is loaded again and the array can lie elsewhere.  So
 * the address is looked up once per context -- with that context current --
 * and kept under the context's unique ID (cuCtxGetId; IDs are never reused
 * within a process, unlike context handles).  The driver calls are reached
 * through the runtime's entry-point query, so the library does not link the
 * driver library. */
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

struct ScratchEntry {
    unsigned long long ctx_id;
    void* addr;
};

constexpr int kCacheEntries = 64;
std::mutex g_setup_mutex;
ScratchEntry g_cache[kCacheEntries];
int g_cache_used = 0, g_cache_next = 0;
bool g_entry_points_done = false;
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

/* ID of the context current on this thread; false when there is none yet
 * or the driver cannot say. */
bool current_context_id(unsigned long long* id)
{
    if (!g_ctx_get_current || !g_ctx_get_id) return false;
    CUcontext c = nullptr;
    if (g_ctx_get_current(&c) != CUDA_SUCCESS || !c) return false;
    return g_ctx_get_id(c, id) == CUDA_SUCCESS;
}

/* Set-up, once per context, with that context current: look up the array's
 * device address.  The first call in a context may load the module there,
 * so it must happen outside any stream capture.  Without the driver's
 * context IDs the address is looked up on every call. */
cudaError_t scratch_address(void** out)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_entry_points_done) {
        g_entry_points_done = true;
        cudaDriverEntryPointQueryResult q1{}, q2{};
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
        cudaGetLastError(); /* a missing entry point is not the caller's error */
    }
    unsigned long long id = 0;
    const bool have_id = current_context_id(&id);
    if (have_id)
        for (int i = 0; i < g_cache_used; ++i)
            if (g_cache[i].ctx_id == id) {
                *out = g_cache[i].addr;
                return cudaSuccess;
            }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_ops);
    if (e != cudaSuccess) return e;
    /* the lookup makes the device's primary context current when no context
     * was: take the ID now */
    if (have_id || current_context_id(&id)) {
        int k = g_cache_next; /* the oldest entry once all are used */
        if (g_cache_used < kCacheEntries)
            k = g_cache_used++;
        else
            g_cache_next = (g_cache_next + 1) % kCacheEntries;
        g_cache[k].ctx_id = id;
        g_cache[k].addr = p;
    }
    *out = p;
    return cudaSuccess;
}

}  // namespace

extern "C" int wfe_align_device_noalloc(const char* d_ascii, const wfe_pair* d_pairs, size_t n,
                                        uint32_t max_len, int32_t max_distance, int32_t* d_dist,
                                        int8_t* d_cigar, uint32_t cigar_stride, uint8_t* d_status,
                                        void* stream)
{
    if (max_distance < 1 || max_distance > WFE_NOALLOC_MAX_DISTANCE) return WFE_ERR_INVALID_ARGUMENT;
    if (n > 0x7fffffffu) return WFE_ERR_INVALID_ARGUMENT;
    if (n == 0) return WFE_OK;
    if (!d_ascii || !d_pairs || !d_dist || (cigar_stride && !d_cigar) || max_len == 0)
        return WFE_ERR_INVALID_ARGUMENT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return WFE_ERR_NO_DEVICE;
    }
    void* scratch = nullptr;
    if (scratch_address(&scratch) != cudaSuccess) {
        cudaGetLastError();
        return WFE_ERR_CUDA;
    }
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return WFE_ERR_CUDA;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);

    /* tier 0: its occupancy (its store is in shared memory).  Its 32 pairs
     * per CTA each stage a CIGAR in shared memory: for long sequences with
     * wide CIGAR slots it does not fit, and tier 3 aligns every pair. */
    const wfe::TierShape sh0 = wfe::tier_shape(kFirstTier, max_len, cigar_stride, sms);
    const bool first = sh0.grid > 0;
    const bool deep = !first || max_distance > wfe::tier_info(kFirstTier).dcap;
    const bool listed = first && deep; /* tier 3 over the pairs tier 0 handed on */

    /* tier 3: occupancy, capped by the op-store slots of the array; every
     * group's store holds all rows of the tier (distances up to 271) */
    wfe::TierShape sh = wfe::tier_shape(kNoallocTier, max_len, cigar_stride, sms);
    if (deep && sh.grid <= 0) return WFE_ERR_SEQ_TOO_LONG; /* sequences + CIGAR slot exceed shared memory */
    const size_t stores_at = listed ? kStoresAt : 0u;
    const uint32_t full_rows = (uint32_t)WFE_NOALLOC_MAX_DISTANCE;
    const size_t per_cta = wfe::tier_scratch_bytes(kNoallocTier, 1, full_rows);
    const int slots = (int)((kNoallocScratchBytes - stores_at) / per_cta);
    sh.ops_group_bytes = (uint32_t)(per_cta / 4u); /* 4 groups (one per warp) per CTA */
    sh.ops_rows = (int)full_rows;

    unsigned char* base = static_cast<unsigned char*>(scratch);
    uint32_t* list = reinterpret_cast<uint32_t*>(base);
    uint32_t* count = reinterpret_cast<uint32_t*>(base + kListBytes);
    for (size_t b0 = 0; b0 < n; b0 += kRoundPairs) {
        const uint32_t nb = (uint32_t)std::min<size_t>(kRoundPairs, n - b0);
        wfe::AlignLaunch a{};
        a.L.ascii = d_ascii;
        a.L.pairs = d_pairs + b0;
        a.n_work = nb;
        a.dist = d_dist + b0;
        a.cigar = cigar_stride ? d_cigar + b0 * (size_t)cigar_stride : nullptr;
        a.cigar_stride = cigar_stride;
        a.status = d_status ? d_status + b0 : nullptr;
        a.max_distance = max_distance;
        a.max_len = max_len;
        a.passed_total = nullptr; /* a.chain.cta_done stays NULL: the host starts each tier */
        if (first) {
            /* tier 0 over the round, the pairs past its reach to the list */
            if (listed && cudaMemsetAsync(count, 0, sizeof(uint32_t), s) != cudaSuccess) return WFE_ERR_CUDA;
            a.tier = kFirstTier;
            a.retry = listed ? list : nullptr;
            a.retry_count = listed ? count : nullptr;
            a.chain.shape[kFirstTier] = sh0;
            const uint32_t per_cta0 = 4u * (32u / (uint32_t)wfe::tier_info(kFirstTier).G);
            const int grid0 = (int)std::min<uint64_t>((uint64_t)sh0.grid, ((uint64_t)nb + per_cta0 - 1) / per_cta0);
            if (wfe::launch_tier(kFirstTier, a, std::max(grid0, 1), s) != cudaSuccess) return WFE_ERR_CUDA;
        }
        if (!deep) continue;
        /* tier 3 over the list (its count is read on the device), or over
         * every pair of the round */
        a.tier = kNoallocTier;
        a.work = listed ? list : nullptr;
        a.work_count = listed ? count : nullptr;
        a.retry = nullptr; /* max_distance <= the tier's capacity: no pair is handed on */
        a.retry_count = nullptr;
        a.ops_scratch = base + stores_at;
        a.ops_scratch_bytes = kNoallocScratchBytes - stores_at;
        a.chain.shape[kNoallocTier] = sh;
        const int want = (int)(((uint64_t)nb + 3u) / 4u);
        const int grid3 = std::max(1, std::min(std::min(sh.grid, slots), listed ? slots : want));
        if (wfe::launch_tier(kNoallocTier, a, grid3, s) != cudaSuccess) return WFE_ERR_CUDA;
    }
    return WFE_OK;
}

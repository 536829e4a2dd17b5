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
 * The kernel is the tier-3 alignment kernel (32 lanes per pair, distances up
 * to 271, backtrace store in global memory), here pointed at that array.
 * A pair's store takes 20,544 bytes (a triangle of 271 rows), so the array
 * holds the stores of 816 pairs in flight, 204 CTAs of 4 pairs; the grid is
 * sized so that every resident group has its own slot.  On a GB300 (152
 * SMs) that is about 1.3 CTAs per SM, below the kernel's occupancy: the
 * price of the fixed size.
 */
#include <algorithm>
#include <mutex>

#include <cuda.h>

#include "wfe.h"
#include "wfe_kernels.cuh"

namespace {

constexpr size_t kNoallocScratchBytes = (size_t)WFE_NOALLOC_SCRATCH_BYTES;
constexpr int kNoallocTier = 3;

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

    /* resident CTAs: occupancy, capped by the op-store slots of the array;
     * every group's store holds all rows of the tier (distances up to 271) */
    wfe::TierShape sh = wfe::tier_shape(kNoallocTier, max_len, cigar_stride, sms);
    const int occ = sh.grid;
    if (occ <= 0) return WFE_ERR_SEQ_TOO_LONG; /* sequences + CIGAR slot exceed shared memory */
    const uint32_t full_rows = (uint32_t)WFE_NOALLOC_MAX_DISTANCE;
    const size_t per_cta = wfe::tier_scratch_bytes(kNoallocTier, 1, full_rows);
    const int slots = (int)(kNoallocScratchBytes / per_cta);
    sh.ops_group_bytes = (uint32_t)(per_cta / 4u); /* 4 groups (one per warp) per CTA */
    sh.ops_rows = (int)full_rows;
    const uint32_t pairs_per_cta = 4u;
    const int want = (int)std::min<size_t>((n + pairs_per_cta - 1) / pairs_per_cta, (size_t)1 << 30);
    const int grid = std::min(std::min(occ, slots), want);

    wfe::AlignLaunch a{};
    a.L.ascii = d_ascii;
    a.L.pairs = d_pairs;
    a.work = nullptr;
    a.work_count = nullptr;
    a.n_work = (uint32_t)n;
    a.dist = d_dist;
    a.cigar = d_cigar;
    a.cigar_stride = cigar_stride;
    a.status = d_status;
    a.max_distance = max_distance;
    a.max_len = max_len;
    a.retry = nullptr;         /* max_distance <= the tier's capacity: no pair is handed on */
    a.retry_count = nullptr;
    a.passed_total = nullptr;
    a.ops_scratch = static_cast<unsigned char*>(scratch);
    a.ops_scratch_bytes = kNoallocScratchBytes;
    a.tier = kNoallocTier; /* a.chain.cta_done stays NULL: no tier follows */
    a.chain.shape[kNoallocTier] = sh;
    const cudaError_t e = wfe::launch_tier(kNoallocTier, a, grid, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? WFE_OK : WFE_ERR_CUDA;
}

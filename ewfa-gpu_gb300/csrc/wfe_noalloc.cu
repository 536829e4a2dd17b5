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
 * The array holds the stores of kNoallocScratchBytes / 36,864 pairs in
 * flight; the grid is sized so that every resident group has its own slot.
 */
#include <algorithm>
#include <mutex>

#include "wfe.h"
#include "wfe_kernels.cuh"

namespace {

constexpr size_t kNoallocScratchBytes = (size_t)WFE_NOALLOC_SCRATCH_BYTES;
constexpr int kNoallocTier = 3;
constexpr int kMaxDevices = 64;

/* The scratch of every call on this device.  Host code must not use the
 * symbol itself as a pointer: on the host it names a stand-in, not the
 * device array; the device address comes from cudaGetSymbolAddress. */
static __device__ __align__(256) unsigned char g_noalloc_ops[kNoallocScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

/* Once per device, with that device current: look up the array's device
 * address.  The first call may load the module on the device, so it must
 * happen outside any stream capture. */
cudaError_t scratch_address(int dev, void** out)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_ops);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
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
    if (cudaGetDevice(&dev) != cudaSuccess) return WFE_ERR_NO_DEVICE;
    if (dev < 0 || dev >= kMaxDevices) return WFE_ERR_INVALID_ARGUMENT;
    void* scratch = nullptr;
    if (scratch_address(dev, &scratch) != cudaSuccess) return WFE_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return WFE_ERR_CUDA;

    /* resident CTAs: occupancy, capped by the op-store slots of the array */
    const int occ = wfe::tier_grid(kNoallocTier, max_len, cigar_stride, sms);
    if (occ <= 0) return WFE_ERR_SEQ_TOO_LONG; /* sequences + CIGAR slot exceed shared memory */
    const size_t per_cta = wfe::tier_scratch_bytes(kNoallocTier, 1);
    const int slots = (int)(kNoallocScratchBytes / per_cta);
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
    const cudaError_t e = wfe::launch_tier(kNoallocTier, a, grid, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? WFE_OK : WFE_ERR_CUDA;
}

/*
 * int_peak.cu -- the 32-bit integer issue peak of a device, measured: the
 * denominator of the integer-op roofline that bench.py reports beside the
 * HBM one (the alignment kernels are bound by their integer pipes).
 *
 * Every thread keeps two banks of 8 values; one trip updates each x with a
 * three-input add of three live values (one IADD3) and each y with a
 * three-input logic op of three live values (one LOP3): 16 integer
 * operations per thread per trip, with no operand the compiler could hoist
 * out of the loop; the trip loop is unrolled 8 times, so its own counter and branch
 * add under 3% of the instructions.  The grid fills every SM with 2048
 * threads.  The best of several timed launches (CUDA events on one stream)
 * gives operations per second.
 *
 *   int wfe_int32_peak(int device, int iters, int reps, double* ops_per_s,
 *                      double* best_ms)
 */
#include <cstdint>
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;
constexpr int kBlocksPerSm = 8;

__global__ void __launch_bounds__(kThreads) int_peak_kernel(uint32_t* out, uint32_t seed, int iters)
{
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t x[kChains], y[kChains];
#pragma unroll
    for (int u = 0; u < kChains; ++u) {
        x[u] = seed ^ (tid * 2654435761u + (uint32_t)u);
        y[u] = seed + (tid ^ (0x9e3779b9u * (uint32_t)(u + 1)));
    }
#pragma unroll 8
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < kChains; ++u) {
            x[u] = x[u] + y[u] + y[(u + 1) % kChains];
            y[u] = (y[u] & x[u]) ^ x[(u + 1) % kChains];
        }
    }
    uint32_t r = 0;
#pragma unroll
    for (int u = 0; u < kChains; ++u) r ^= x[u] ^ y[u];
    out[tid] = r;
}

}  // namespace

extern "C" int wfe_int32_peak(int device, int iters, int reps, double* ops_per_s, double* best_ms)
{
    if (iters <= 0 || reps <= 0 || !ops_per_s) return 1;
    if (cudaSetDevice(device) != cudaSuccess) return 2;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 2;
    const int grid = sms * kBlocksPerSm;
    const size_t threads = (size_t)grid * kThreads;
    uint32_t* out = nullptr;
    if (cudaMalloc(&out, threads * sizeof(uint32_t)) != cudaSuccess) return 3;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = 0;
    float best = 1e30f;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = 4;
    } else {
        int_peak_kernel<<<grid, kThreads, 0, s>>>(out, 1u, iters); /* warm-up */
        for (int r = 0; r < reps && rc == 0; ++r) {
            cudaEventRecord(e0, s);
            int_peak_kernel<<<grid, kThreads, 0, s>>>(out, (uint32_t)r + 2u, iters);
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = 5;
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) best = ms;
        }
        if (cudaGetLastError() != cudaSuccess) rc = 5;
    }
    if (rc == 0) {
        const double ops = (double)threads * (double)iters * (2.0 * kChains);
        *ops_per_s = ops / (best * 1e-3);
        if (best_ms) *best_ms = best;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(out);
    return rc;
}

/*
 * wfe_kernels.cuh -- launch interface of the libwfe kernels (host side).
 */
#ifndef WFE_KERNELS_CUH
#define WFE_KERNELS_CUH

#include <stdint.h>
#include <cuda_runtime.h>

#include "wfe_device.cuh"

namespace wfe {

/* Register tiers of the alignment kernel: G lanes per alignment, 2J+1
 * register chunks of G diagonals per lane, largest distance G*J + G/2 - 1. */
struct TierInfo {
    int G, J, dcap;
    bool ops_in_smem;
};

/* Tiers 0-4 are register tiers (one pair per group of G lanes); tiers 5
 * and 6 give each pair a whole CTA with the wavefront in shared (5) or
 * global (6) memory and have no distance limit of their own. */
constexpr int kNumTiers = 7;
constexpr int kLongThreads = 256;
constexpr int kLongSmemDistance = 2047; /* largest distance with the wavefront in shared memory */
const TierInfo& tier_info(int t);

/* Launch shape of one tier, for launches made on the device. */
struct TierShape {
    int grid;           /* persistent grid (resident CTAs) */
    uint32_t smem;      /* dynamic shared memory per CTA */
    uint32_t seq_words; /* 16-base words per sequence in shared memory */
    uint32_t gbytes;    /* shared memory per group */
    int dlim;           /* tiers 5-6: largest distance the tier computes */
    uint64_t slab;      /* tiers 5-6: bytes of global scratch per CTA */
    unsigned char* scratch; /* tiers 5-6: grid * slab bytes */
};

/* Global scratch of one CTA of tiers 5-6 for distances up to dlim: 2-bit
 * backtrace store (rows 1..dlim, a 64-bit entry per 32 diagonals),
 * operation chain, runs, and for tier 6 the two wavefront buffers. */
uint64_t long_slab_bytes(int dlim, bool global_wavefront);

/* The tier chain of one batch.  Each tier kernel's last CTA launches the
 * next tier as a tail launch when it handed any pair on, so no launch is
 * made for a tier that has no work. */
struct Chain {
    int last_tier;                   /* last tier of the chain */
    TierShape shape[kNumTiers];
    uint32_t* lists[2];              /* work lists, used alternately by the tiers */
    uint32_t* counts;                /* counts[t]: pairs tier t handed on */
    uint32_t* cta_done;              /* cta_done[t]: CTAs of tier t that finished */
    unsigned long long* launched;    /* launched[t]: launches of tier t (stats) */
};

/* Arguments of one alignment launch over a work list. */
struct AlignLaunch {
    Layout L;
    const uint32_t* work;        /* pair indices; NULL = 0..n_work-1 */
    const uint32_t* work_count;  /* device count of `work`; NULL = n_work */
    uint32_t n_work;             /* bound on the work list */
    int32_t* dist;
    int8_t* cigar;
    uint32_t cigar_stride;
    uint8_t* status;
    int32_t max_distance;        /* 0 = unlimited */
    uint32_t max_len;            /* every sequence of the launch is <= max_len */
    uint32_t* retry;             /* pairs above the tier's distance capacity;
                                    NULL = last tier: they get WFE_PAIR_TOO_LONG */
    uint32_t* retry_count;
    unsigned long long* passed_total; /* running count of pairs handed on (stats) */
    unsigned char* ops_scratch;  /* global op store for tiers that keep it there */
    size_t ops_scratch_bytes;
    int tier;                    /* this launch's tier */
    Chain chain;                 /* chain.cta_done == NULL: no device-side chaining */
};

/* Launch shape of tier t for sequences up to max_len and CIGAR slots of
 * cigar_stride: persistent grid sized by occupancy (grid 0: does not fit). */
TierShape tier_shape(int tier, uint32_t max_len, uint32_t cigar_stride, int sm_count);

/* Bytes of global op-store scratch tier t needs for `grid` CTAs. */
size_t tier_scratch_bytes(int tier, int grid);
/* Persistent grid of tier t for sequences up to max_len, cigar slots of
 * cigar_stride (occupancy-limited, at least 1). */
int tier_grid(int tier, uint32_t max_len, uint32_t cigar_stride, int sm_count);
cudaError_t launch_tier(int tier, const AlignLaunch& a, int grid, cudaStream_t s);

cudaError_t launch_pack(const Layout& L, uint32_t n, uint32_t* words,
                        uint32_t words_per_seq, cudaStream_t s);

cudaError_t launch_cigar_from_history(const Layout& L, uint32_t n, uint32_t max_len,
                                      const int32_t* dist, const uint64_t* hist,
                                      int8_t* cigar, uint32_t cigar_stride,
                                      uint8_t* status, cudaStream_t s);

}  // namespace wfe

#endif

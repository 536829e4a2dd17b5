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
    uint32_t ops_group_bytes; /* tiers 2-4: bytes of one group's backtrace store in the global scratch */
    int ops_rows;       /* tiers 2-4: score steps that store holds (a distance never exceeds the
                           longest sequence, so rows past max_len are never written) */
};

/* Global scratch of one CTA of tiers 5-6 for distances up to dlim: 2-bit
 * backtrace store (rows 1..dlim, a 64-bit entry per 32 diagonals),
 * operation chain, runs, and for tier 6 the two wavefront buffers. */
uint64_t long_slab_bytes(int dlim, bool global_wavefront);

/* The tier chain of one batch (of one length bucket).  Tier t works on the
 * pairs of its list: those routed to it up front and those that tier t-1
 * handed on.  Each tier kernel's last CTA launches, as a tail launch, the
 * next tier whose list is not empty, so no launch is made for a tier that
 * has no work. */
struct Chain {
    int last_tier;                   /* last tier of the chain */
    TierShape shape[kNumTiers];
    uint32_t* list[kNumTiers];       /* list[t]: work of tier t */
    uint32_t* counts;                /* counts[t]: pairs in list[t] */
    uint32_t* cta_done;              /* cta_done[t]: CTAs of tier t that finished */
    uint32_t* work_next;             /* work_next[t]: next work item of tier t (work stealing) */
    unsigned long long* launched;    /* launched[t]: launches of tier t (stats) */
    unsigned long long* passed;      /* passed[t]: pairs tier t handed on (stats) */
    uint8_t* launch_error;           /* byte t set: a device-side launch of tier t failed (host memory
                                        the device writes in place) */
};

/* Length buckets of the classify kernel, and for each the tiers a pair may
 * be routed to by its predicted distance. */
constexpr int kMaxBuckets = 8;
constexpr int kPredictPrefix = 128; /* bases of each sequence the distance prediction aligns */
struct Buckets {
    int n;
    uint32_t max_len[kMaxBuckets];   /* ascending; a pair goes to the first bucket that holds it */
    int first_tier[kMaxBuckets];
    int last_tier[kMaxBuckets];
    int dcap[kNumTiers];             /* largest distance of each tier */
    const uint16_t* pred;            /* predicted prefix distances, or NULL (route to first_tier) */
    uint32_t* lists;                 /* list of bucket b, tier t at lists + (b*kNumTiers + t)*stride */
    uint32_t stride;
    uint32_t* counts;                /* counts of bucket b at counts + b*count_stride */
    uint32_t count_stride;
    unsigned long long* totals;      /* pairs classified into each bucket (stats) */
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
    uint16_t* pred;              /* prediction launch: prefix distance of every pair */
    unsigned char* ops_scratch;  /* global op store for tiers that keep it there */
    size_t ops_scratch_bytes;
    int tier;                    /* this launch's tier */
    Chain chain;                 /* chain.cta_done == NULL: no device-side chaining */
};

/* Launch shape of tier t for sequences up to max_len and CIGAR slots of
 * cigar_stride: persistent grid sized by occupancy (grid 0: does not fit). */
TierShape tier_shape(int tier, uint32_t max_len, uint32_t cigar_stride, int sm_count);

/* Bytes of global op-store scratch tier t needs for `grid` CTAs, each
 * group's store holding the rows of distances up to max_len (capped at the
 * tier's own limit). */
size_t tier_scratch_bytes(int tier, int grid, uint32_t max_len);
/* Persistent grid of tier t for sequences up to max_len, cigar slots of
 * cigar_stride (occupancy-limited, at least 1). */
int tier_grid(int tier, uint32_t max_len, uint32_t cigar_stride, int sm_count);
cudaError_t launch_tier(int tier, const AlignLaunch& a, int grid, cudaStream_t s);

/* Sort pairs 0..n-1 into length buckets by max(p_len, t_len) and, within a
 * bucket, into the tier of their predicted distance (see Buckets). */
cudaError_t launch_classify(const Layout& L, uint32_t n, const Buckets& B, cudaStream_t s);

/* Distance of the first kPredictPrefix bases of every pair (capped at
 * tier 0's limit + 1), for routing: pred[i] for pair i. */
cudaError_t launch_predict(const Layout& L, uint32_t n, uint32_t max_len, uint16_t* pred, int grid,
                           cudaStream_t s);

cudaError_t launch_pack(const Layout& L, uint32_t n, uint32_t* words,
                        uint32_t words_per_seq, cudaStream_t s);

cudaError_t launch_cigar_from_history(const Layout& L, uint32_t n, uint32_t max_len,
                                      const int32_t* dist, const uint64_t* hist,
                                      int8_t* cigar, uint32_t cigar_stride,
                                      uint8_t* status, cudaStream_t s);

}  // namespace wfe

#endif

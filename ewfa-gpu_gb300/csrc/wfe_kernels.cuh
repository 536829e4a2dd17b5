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
    int threads;        /* tiers 5-6 and the bound pass: threads per CTA */
};

/* Distance classes of tier 5.  The bound pass (bound_kernel) sends each pair
 * of tier 5 to the first class whose limit covers its distance bound, and
 * every class is a launch of its own with wavefront buffers (shared memory)
 * and backtrace slabs sized to its limit: a class of short distances keeps
 * two to three times the pairs in flight per SM of one launch sized for
 * distance 2047.  Limits 255, 511 and 1023, each kept only while below half
 * of tier 5's own limit, then tier 5's own limit (min(max_len, 2047)).
 * Class 255 runs CTAs of one warp, classes up to distance 1024 CTAs of 128
 * threads, the last one (when larger) 256: a pair of short distance has few
 * cells per step to share, and fewer warps per pair spend fewer instructions
 * on each step's bookkeeping and barrier. */
constexpr int kLongClasses = 4;
constexpr int kLongClassLimit[kLongClasses - 1] = {255, 511, 1023};
constexpr int kLongTinyThreads = 32;
constexpr int kLongTinyDistance = 255;   /* classes up to this limit use kLongTinyThreads */
constexpr int kLongSmallThreads = 128;
constexpr int kLongSmallDistance = 1024; /* classes up to this limit use kLongSmallThreads */
/* Work lists of one length bucket: one per tier, then one per class. */
constexpr int kListsPerBucket = kNumTiers + kLongClasses;

struct LongClasses {
    int n;                           /* classes (0: tier 5 runs as one launch over its list) */
    TierShape shape[kLongClasses];   /* grid, smem, seq_words, dlim, slab, scratch, threads */
    /* List c holds the pairs of the upper half of the class's distances from
     * its front (counts[c] of them) and the others from its back
     * (low_counts[c], at cap-1, cap-2, ...): a class launch takes its longer
     * pairs first, so that its last CTAs are not left with them. */
    uint32_t* list[kLongClasses];
    uint32_t cap;                    /* entries of each list */
    uint32_t* counts;                /* counts[c]: pairs at the front of list[c] */
    uint32_t* low_counts;            /* low_counts[c]: pairs at its back */
    uint32_t* cta_done;              /* cta_done[c]: CTAs of class c that finished */
    uint32_t* work_next;             /* work_next[c] */
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
    LongClasses cls;                 /* tier 5's distance classes */
    TierShape bound_shape;           /* the bound pass: grid, smem, seq_words, threads */
    /* A chain cut short at the last tier that needs no global scratch (the
     * context has not allocated the scratch of the deeper tiers yet): the
     * pairs that tier hands on go to defer as defer_base + their index (up
     * to defer_cap of them; defer_count counts them all), and byte
     * kDeferByte of launch_error is set, for the host to align them once the
     * scratch exists.  NULL: the chain is whole. */
    uint32_t* defer;
    uint32_t* defer_count;
    uint32_t defer_cap;
    uint32_t defer_base;
};
/* launch_error byte that says pairs were deferred (bytes 0..kNumTiers-1 are
 * the tiers' launch failures) */
constexpr int kDeferByte = kNumTiers;

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
    uint32_t* lists;                 /* list of bucket b, tier t at lists + (b*kListsPerBucket + t)*stride */
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
    int32_t* bound;              /* tiers 5-6: an upper bound on each pair's distance (by pair
                                    index; -1 = none), written by the bound pass; NULL = none */
    int cls;                     /* tier 5: the distance class of this launch; -1 = the bound pass
                                    (which routes tier 5's list into the classes) or, without
                                    classes, tier 5 as one launch */
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

/* Upper bounds on the distances of the pairs of a CTA-per-pair tier's work
 * list (a.work / a.work_count / a.n_work, sequences up to a.max_len) into
 * a.bound, one warp per pair; see bound_kernel.  With a.tier == 5 and
 * classes (a.chain.cls.n > 0) the pass also routes every pair to its class
 * and its last CTA starts the first class that has work (tier 5 as a chain
 * of class launches).  bound_shape: its launch shape (grid 0: its shared
 * memory does not fit, and no bound can be computed). */
TierShape bound_shape(uint32_t max_len, int sm_count);
cudaError_t launch_bound(const AlignLaunch& a, cudaStream_t s);

/* Tier 5's distance classes for sequences up to max_len, their slabs carved
 * from a tier-5 scratch of scratch_bytes (0 classes: none fits). */
LongClasses long_classes(uint32_t max_len, int sm_count, uint64_t scratch_bytes);

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

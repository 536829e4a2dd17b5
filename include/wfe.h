/*
 * wfe.h -- C ABI of libwfe, a GB300 (sm_103a) wavefront edit-distance
 * aligner with full CIGAR output.
 *
 * It replaces the host/device boundary of quim0/eWFA-GPU: the class
 * Sequences (src/wavefront.cuh:435-505, src/wavefront.cu:29-330) and the
 * kernel ABI (src/kernels.cuh:32-54).  Results are bit-exact with the
 * reference's algorithm: same edit distance and the same CIGAR bytes under
 * its tie order (deletion > mismatch > insertion), encoded as the reference
 * encodes them (src/kernels.cu:397-498): M runs as negative signed-char
 * chunks of at most 127, then 'X', 'I', 'D' as ASCII, zero terminated when
 * shorter than the slot (the bytes of a slot after its terminator are not
 * specified).  'D' consumes a pattern base, 'I' a text base.
 *
 * Conventions: every call returns a wfe_status (never exits); the caller owns
 * every buffer passed in, the context owns all device memory it allocates.
 * A context is used by one host thread at a time; different contexts may be
 * used concurrently.  No call takes torch or CUDA C++ types: streams are
 * passed as void* (a cudaStream_t).
 */
#ifndef WFE_H
#define WFE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WFE_ABI_VERSION 3 /* 2: wfe_server_stats gained admit_ns and finish_ns; 3: wfe_stats gained
                             deferred_pairs and deep_scratch_bytes */

/* Call status.  The reference exits the process on any CUDA error
 * (utils/cuda_helpers.cuh:24-31) or fatal condition (utils/logger.h:66-68). */
typedef enum wfe_status {
    WFE_OK = 0,
    WFE_ERR_INVALID_ARGUMENT = 1,
    WFE_ERR_OUT_OF_MEMORY = 2,
    WFE_ERR_SEQ_TOO_LONG = 3,    /* a sequence exceeds the context's max_seq_len */
    WFE_ERR_CUDA = 4,            /* a CUDA runtime call failed (see wfe_last_cuda_error) */
    WFE_ERR_NO_DEVICE = 5,
    WFE_ERR_TIMEOUT = 6,         /* a bounded wait ran out */
    WFE_ERR_BUSY = 7,            /* admission refused: not enough free device memory */
    WFE_ERR_INTERNAL = 8,        /* a device-side consistency check failed */
    WFE_ERR_NOT_FOUND = 9        /* unknown ticket */
} wfe_status;

/* Per-pair status written to status_out. */
enum {
    WFE_PAIR_OK = 0,
    WFE_PAIR_OVER_MAX_DISTANCE = 1, /* distance > max_distance: distance_out =
                                       max_distance + 1 (the reference writes 64
                                       for its cap, src/kernels.cu:259,290), CIGAR
                                       empty */
    WFE_PAIR_CIGAR_TRUNCATED = 2,   /* CIGAR longer than the slot: the first
                                       cigar_stride bytes are written, no
                                       terminator (the reference overflows into
                                       the next slot instead) */
    WFE_PAIR_TOO_LONG = 3,          /* sequence longer than the launch's capacity */
    WFE_PAIR_BAD_HISTORY = 4,       /* history holds a code that is not an
                                       operation: the CIGAR stops there (the
                                       reference's "Incorrect backtrace" exit,
                                       src/kernels.cu:471-478) */
    WFE_PAIR_OUT_OF_RANGE = 5       /* the pair's bytes lie outside the ASCII
                                       buffer (host calls that read it in place);
                                       the pair is not aligned */
};

/* One pattern/text pair inside a caller buffer of ASCII bases.  Any byte is a
 * base: its 2-bit code is (byte & 6) >> 1, so A C T G = 0 1 2 3 and N, a, c,
 * t, g alias to them (src/wavefront_structures.h:73-83). */
typedef struct wfe_pair {
    uint64_t p_off;  /* pattern: bytes [p_off, p_off + p_len) */
    uint64_t t_off;  /* text:    bytes [t_off, t_off + t_len) */
    uint32_t p_len;
    uint32_t t_len;
} wfe_pair;

typedef struct wfe_config {
    int32_t device;        /* CUDA device ordinal (the reference uses 0, src/aligner.cu:147) */
    uint32_t max_seq_len;  /* longest pattern or text accepted, in bases */
    uint32_t batch_size;   /* pairs per device batch (-b, src/aligner.cu:149-159);
                              0 = 100000 */
    int32_t max_distance;  /* largest distance searched, 0 = no limit.  63
                              reproduces the reference's search range
                              (src/wavefront.cuh:462-466) */
    uint32_t cigar_stride; /* bytes per CIGAR slot; 0 = the reference's
                              cigar_max_len for max_seq_len, l + (4 - l % 4)
                              (src/wavefront.cuh:48-50) */
    uint32_t flags;        /* WFE_FLAG_* */
} wfe_config;

#define WFE_FLAG_NO_PIPELINE 1u   /* one batch in flight: no copy/compute overlap in host
                                     calls, no second stream in device calls */
#define WFE_FLAG_KERNEL_TIMING 2u /* time every kernel launch with CUDA events on its
                                     stream; read back by wfe_get_stats */
#define WFE_FLAG_DEVICE_ONLY 4u   /* no staging buffers for host calls: the context
                                     serves wfe_align_device only (wfe_align and
                                     wfe_align_strided return WFE_ERR_INVALID_ARGUMENT) */
#define WFE_FLAG_PAGEABLE_IN_PLACE 8u /* host calls on a device that reads pageable
                                     memory through the CPU's page tables (ATS over
                                     NVLink-C2C on GB300): pageable buffers are used
                                     in place like pinned ones (see wfe_align);
                                     ignored on other devices */

typedef struct wfe_ctx wfe_ctx;

/* Counters of one context since creation (or the last reset). */
typedef struct wfe_stats {
    uint64_t pairs;            /* pairs aligned */
    uint64_t batches;          /* device batches run */
    uint64_t kernel_launches;  /* kernels launched by this context */
    uint64_t h2d_bytes;        /* host-to-device bytes copied */
    uint64_t d2h_bytes;        /* device-to-host bytes copied */
    uint64_t tier_entered[8];  /* pairs that entered each distance tier */
    uint64_t tier_passed[8];   /* pairs each tier handed on to the next (above
                                  its distance capacity) */
    uint64_t tier_launches[8]; /* launches of each tier's kernel */
    double tier_ms[8];         /* GPU milliseconds of the chains started at each
                                  tier (only with WFE_FLAG_KERNEL_TIMING) */
    uint64_t mapped_batches;   /* host-call batches whose inputs the kernels
                                  read in place (pinned, or pageable with
                                  WFE_FLAG_PAGEABLE_IN_PLACE) */
    uint64_t deferred_pairs;   /* pairs a host call deferred past tier 1 and
                                  aligned again once tiers 2-6 had scratch
                                  (see wfe_create) */
    uint64_t deep_scratch_bytes; /* device bytes of tiers 2-6's scratch, both
                                  stages (0 until a call needs it; not reset) */
} wfe_stats;

/* ---- lifecycle -------------------------------------------------------- */

/* Create a context on cfg->device: streams, the work lists of one batch in
 * each pipeline stage, and the scratch of the tiers.  Replaces the Sequences
 * constructor and GPU_memory_init (src/wavefront.cuh:458-485,
 * src/wavefront.cu:29-108).  The device buffers that stage a batch of host
 * inputs and results are allocated by the first host call that stages
 * (buffers used in place never need them); that call returns
 * WFE_ERR_OUT_OF_MEMORY if they do not fit.
 * The global scratch of tiers 2-6 (distances past 79; tens to hundreds of
 * MB, for both pipeline stages) is allocated here only for contexts with
 * WFE_FLAG_DEVICE_ONLY or whose first tier is past 1 (max_seq_len above
 * 1,200).  Otherwise the first call that needs it allocates it: the first
 * device call, the first wfe_set_policy or wfe_autotune that starts a chain
 * past tier 1 or routes by prediction, or the first host call in which a
 * pair's distance passes 79.  Such a host call aligns those pairs again
 * once the scratch exists (from their index in the call; when more than
 * batch_size were deferred, the whole call runs again), with the same
 * results.  A short-read context that never needs it holds ~10 MB of device
 * memory instead of ~200 MB, and frees it sooner.
 * Threading: a context is used by one thread at a time; different contexts
 * may be used from different threads at once.  Every call on a context makes
 * its device the calling thread's current device (as the reference's
 * cudaSetDevice does, src/aligner.cu:147). */
int wfe_create(const wfe_config* cfg, wfe_ctx** out);

/* wfe_create with a bound on the device memory of the CTA-per-pair tiers'
 * slabs: one slab per resident CTA holds a pair's backtrace store, operation
 * chain and runs (tier 6: also its wavefront).  tier5_bytes and tier6_bytes
 * bound tiers 5 and 6; 0 keeps wfe_create's 2 GiB and 8 GiB.  A smaller
 * bound lowers only how many pairs those tiers align at once (never fewer
 * than one); the results are the same.  No reference counterpart: the
 * reference has neither tier (its distance search stops at 63). */
int wfe_create_with_scratch(const wfe_config* cfg, uint64_t tier5_bytes, uint64_t tier6_bytes,
                            wfe_ctx** out);

/* Release everything the context owns.  Replaces GPU_memory_free
 * (src/wavefront.cu:110-125). */
void wfe_destroy(wfe_ctx* ctx);

const char* wfe_strerror(int status);

/* Last CUDA runtime error code seen by ctx (0 if none); ctx may be NULL for
 * the thread's last wfe_create failure. */
int wfe_last_cuda_error(const wfe_ctx* ctx);

/* Counters of ctx; waits for the context's outstanding device work first
 * (the per-tier counters and timings live on the device until then). */
int wfe_get_stats(wfe_ctx* ctx, wfe_stats* out);
int wfe_reset_stats(wfe_ctx* ctx);

/* ---- scheduling policy (mixed lengths) ------------------------------------ */

#define WFE_MAX_BUCKETS 8

/* Length buckets: a pair goes to the first bucket whose bucket_max_len is at
 * least max(p_len, t_len) (the last bucket always ends at max_seq_len).
 * With more than one bucket, every batch is first sorted into buckets on the
 * device and each bucket is aligned with launch shapes sized to its longest
 * sequence -- shared memory per pair, resident CTAs -- starting at its own
 * first tier:
 *   tier 0: 4 lanes per pair, backtrace store in shared memory, distance <= 21
 *   tier 1: 32 lanes per pair, shared-memory store, <= 79
 *   tier 2: 32 lanes, shared-memory store, <= 143
 *   tier 3: 32 lanes, store spilled to global memory, <= 271
 *   tier 4: 32 lanes, global store, <= 527
 *   tier 5: a CTA per pair, wavefront in shared memory, <= 2047
 *   tier 6: a CTA per pair, wavefront in global memory, no limit
 * (a pair above its tier's limit is handed to the next tier on the device).
 * first_tier[b] = -1 picks by length; first_tier may be NULL.  With
 * WFE_POLICY_PREDICT, a first pass aligns the first 128 bases of every pair
 * (distance only) and each pair starts at the lowest tier of its bucket, not
 * below first_tier[b], whose limit covers its distance extrapolated to its
 * length: pairs of one length but very different error rates no longer all
 * start at the same tier (and restart in every tier they outgrow).  Results
 * do not depend on the policy.  The default is one bucket, no prediction.
 * A chain that starts at tier 5 or 6 first bounds the distance of each of its
 * pairs with a narrow band of the wavefront (one warp per pair); the
 * CTA-per-pair tiers then compute only the cells the target cell depends on
 * (about half of them), and a pair whose bound lies past tier 5's limit
 * goes straight to tier 6.  WFE_POLICY_NO_BOUND turns that pass off (for
 * comparison: results are the same).
 * Replaces nothing in the reference, which has one fixed launch shape
 * (src/wavefront.cu:173-208); see also wfe_autotune. */
#define WFE_POLICY_PREDICT 1u  /* route every pair to the tier of its predicted distance */
#define WFE_POLICY_NO_BOUND 2u /* no distance bounds before the CTA-per-pair tiers */
int wfe_set_policy(wfe_ctx* ctx, uint32_t nbuckets, const uint32_t* bucket_max_len,
                   const int32_t* first_tier, uint32_t flags);
int wfe_get_policy(const wfe_ctx* ctx, uint32_t* nbuckets, uint32_t* bucket_max_len,
                   int32_t* first_tier, uint32_t* flags);

/* Choose every bucket's first tier by measurement and install the policy:
 * for each bucket, up to 4096 of the given DEVICE pairs that fall in it are
 * aligned starting at every usable tier (the tier fixes the lanes per pair,
 * whether the backtrace store stays in shared memory or spills to global
 * memory, and whether the wavefront stays in shared memory), through the
 * same routing as a real batch (flags as in wfe_set_policy), and the
 * fastest wins.  With cache_path set, a matching earlier result (same GPU,
 * max_seq_len, slot size, flags and buckets) is reused instead, and new
 * results are appended to that file.  first_tier_out (may be NULL) receives
 * the choice. */
int wfe_autotune(wfe_ctx* ctx, const char* d_ascii, const wfe_pair* d_pairs, size_t n,
                 uint32_t nbuckets, const uint32_t* bucket_max_len, uint32_t flags,
                 const char* cache_path, int32_t* first_tier_out);

/* ---- host-buffer alignment (the reference's batch loop) --------------- */

/* Align n pairs held in HOST memory; results to HOST memory.  Replaces the
 * loop GPU_launch_wavefront_distance / prepare_next_batch
 * (src/aligner.cu:63-65, src/wavefront.cu:173-330), in batches of
 * batch_size pairs.  dist_out[n], cigar_out[n * cigar_stride], status_out[n]
 * (may be NULL).  Synchronous: returns when every result is in host memory.
 *
 * Pinned (page-locked, device-mapped) buffers are used in place: when the
 * ASCII buffer and the descriptors are pinned, the kernels read them directly
 * over the CPU-GPU link (NVLink-C2C on GB300) with no staging copy, checking
 * every descriptor against ascii_bytes (pairs outside get
 * WFE_PAIR_OUT_OF_RANGE) and every length against max_seq_len
 * (WFE_PAIR_TOO_LONG); when the outputs are pinned, the kernels write them
 * directly.  Pageable buffers are staged: each batch's span of ASCII and its
 * descriptors are copied in (the call then returns WFE_ERR_SEQ_TOO_LONG or
 * WFE_ERR_INVALID_ARGUMENT for bad pairs before aligning anything), results
 * copied out, with the copies of one batch overlapping the kernels of the
 * other.  With WFE_FLAG_PAGEABLE_IN_PLACE on a device that reads the CPU's
 * page tables, pageable buffers are used in place as pinned ones are (bad
 * pairs reported per pair); every page is touched on the host first, by up
 * to eight threads, so that none is first faulted in by the GPU.  A range
 * that is not wholly mapped is staged. */
int wfe_align(wfe_ctx* ctx, const char* ascii, size_t ascii_bytes,
              const wfe_pair* pairs, size_t n, int32_t* dist_out,
              int8_t* cigar_out, uint8_t* status_out);

/* Same, with the reference reader's layout: pattern of pair i at
 * ascii + 2*i*stride, text at ascii + (2*i+1)*stride, lengths in p_len[] and
 * t_len[] (utils/sequence_reader.cu:148-189; WF_element,
 * src/wavefront_structures.h:44-50). */
int wfe_align_strided(wfe_ctx* ctx, const char* ascii, size_t stride,
                      const uint32_t* p_len, const uint32_t* t_len, size_t n,
                      int32_t* dist_out, int8_t* cigar_out,
                      uint8_t* status_out);

/* ---- device-buffer alignment ------------------------------------------ */

/* Align n pairs whose ASCII and descriptors are already in DEVICE memory;
 * results to DEVICE memory; enqueued on `stream` (a cudaStream_t; NULL = the
 * context's stream), asynchronous.  max_len: an upper bound on every p_len
 * and t_len of the call (pairs above it get WFE_PAIR_TOO_LONG).  The ASCII
 * buffer must stay readable up to the next 16-byte boundary after every
 * sequence (sequences are read in aligned 16-byte blocks).  A tier that a
 * kernel failed to launch on the device (its pairs are left unaligned) is
 * reported as WFE_ERR_CUDA by the next call on the context; wfe_align and
 * wfe_align_strided report it themselves.  The device calls of a context
 * share its work lists and scratch: enqueue them on one stream (or order
 * them), and synchronise that stream before a host call on the context.
 * A call of more than batch_size pairs runs its batches on two streams --
 * `stream` and one of the context's -- so that consecutive batches overlap
 * on the device; the context's stream waits for the work already on
 * `stream`, and `stream` waits for it at the end, so the call stays ordered
 * on `stream`.  The first device call allocates the scratch of tiers 2-6
 * if the context has none yet (see wfe_create); on a context with
 * WFE_FLAG_DEVICE_ONLY the first call of more than batch_size pairs
 * allocates the second stream's copy of it (without it the batches run one
 * after another; WFE_FLAG_NO_PIPELINE keeps them on `stream` alone).
 * Replaces the kernel chain WF_edit_distance -> generate_cigars
 * (src/wavefront.cu:203-260). */
int wfe_align_device(wfe_ctx* ctx, const char* d_ascii,
                     const wfe_pair* d_pairs, size_t n, uint32_t max_len,
                     int32_t* d_dist, int8_t* d_cigar, uint8_t* d_status,
                     void* stream);

/* Pack 2n sequences into 2-bit words on the device, the layout of the
 * reference's compact_sequences (src/kernels.cu:313-394): 16 bases per
 * 32-bit word, base i of a sequence at bits 31-2(i%16)..30-2(i%16) of word
 * i/16, bases past the end 0.  Pair i: pattern words at
 * d_words + 2*i*words_per_seq, text words at d_words + (2*i+1)*words_per_seq;
 * words_per_seq >= ceil(max length / 16). */
int wfe_pack_device(const char* d_ascii, const wfe_pair* d_pairs, size_t n,
                    uint32_t* d_words, uint32_t words_per_seq, void* stream);

/* Encoded CIGARs from the reference's backtrace records on the device:
 * per pair a distance (< 64) and the 128-bit history words[2] of
 * WF_backtrace_result_t (src/wavefront_structures.h:57-60), op d in bits
 * 2(d%32)..2(d%32)+1 of words[d/32].  Replaces generate_cigars /
 * generate_cigars_sh_mem (src/kernels.cu:397-625). */
int wfe_cigar_from_history_device(const char* d_ascii, const wfe_pair* d_pairs,
                                  size_t n, uint32_t max_len,
                                  const int32_t* d_dist,
                                  const uint64_t* d_history, int8_t* d_cigar,
                                  uint32_t cigar_stride, uint8_t* d_status,
                                  void* stream);

/* ---- allocation-free alignment ------------------------------------------ */

/* Largest max_distance wfe_align_device_noalloc accepts, and the size of the
 * fixed device array that holds its scratch. */
#define WFE_NOALLOC_MAX_DISTANCE 271
#define WFE_NOALLOC_SCRATCH_BYTES (16u << 20)

/* Align n pairs whose ASCII and descriptors are in DEVICE memory, results to
 * DEVICE memory, without allocating anything: no cudaMalloc, no cudaFree, no
 * context.  No counterpart in the reference.  It is for callers that cannot
 * allocate device memory where they align: a plugin whose host application
 * owns every device allocation through its own pool, a real-time loop that
 * forbids allocation after start-up, code on a memory budget that another
 * framework accounts for.
 *
 * Runs on the current device, enqueued on `stream` (a cudaStream_t, NULL =
 * the legacy default stream).  Arguments as wfe_align_device; max_distance
 * must be 1..WFE_NOALLOC_MAX_DISTANCE (the search is bounded because its
 * backtrace store is a fixed array): pairs farther apart get
 * WFE_PAIR_OVER_MAX_DISTANCE and distance max_distance + 1, exactly as
 * wfe_align_device does with the same max_distance.  Results are identical
 * to wfe_align_device's.  Returns WFE_ERR_INVALID_ARGUMENT for a
 * max_distance out of range, WFE_ERR_SEQ_TOO_LONG when max_len and
 * cigar_stride do not fit the kernel's shared memory.
 *
 * Scratch: a WFE_NOALLOC_SCRATCH_BYTES array in the library's device image,
 * held by every GPU that loads the library until the process exits.  Its
 * device address belongs to the CUDA context current at call time (the
 * device's primary context, or one the application made current); the first
 * call in each context looks that address up (set-up, once per context),
 * so make that first call outside any stream capture.  The pairs are aligned
 * in rounds of up to 2^20: the 4-lane tier (distances up to 21, backtrace in
 * shared memory) takes every pair of a round and hands the ones past
 * distance 21, through a list at the start of the array, to the 32-lane
 * tier 3, whose backtrace stores fill the rest: 612 pairs in flight, 153
 * CTAs of 4 (about one per SM on a 152-SM GB300, below that kernel's
 * occupancy).  Sequences and CIGAR slots too wide for the 4-lane tier's
 * shared memory go to tier 3 alone (816 pairs in flight).  On short reads a
 * call runs at ~80% of wfe_align_device's speed.
 * Every call shares the array and it keeps the last call's contents
 * (nothing in it has to start at zero: the list's count is set by a
 * cudaMemsetAsync on `stream` each round, and every other entry is written
 * before it is read).  Calls that overlap on the GPU -- on
 * two streams, or from two host threads -- race on the array and corrupt
 * each other's results: issue them on one stream. */
int wfe_align_device_noalloc(const char* d_ascii, const wfe_pair* d_pairs, size_t n,
                             uint32_t max_len, int32_t max_distance, int32_t* d_dist,
                             int8_t* d_cigar, uint32_t cigar_stride, uint8_t* d_status,
                             void* stream);

/* ---- serving: continuous batching of requests ------------------------- */

/* A request server on one GPU.  Requests of any size (1 pair and up) are
 * submitted from any thread and answered asynchronously.  A scheduler thread
 * admits waiting requests into a new device batch whenever one of `lanes`
 * streams is free and the batch's bytes (sequences, descriptors, distances,
 * statuses, CIGAR slots) fit in the free part of a device-memory arena of
 * `memory_bytes`: a request that arrives while other batches run joins the
 * next batch and its work overlaps theirs on the device; a request larger
 * than what is free is split over several batches.  Each lane keeps its
 * wavefront and backtrace scratch resident for the server's life.  Results
 * do not depend on which requests share a batch.  The reference has no
 * serving mode: its driver aligns one file in fixed batches
 * (src/aligner.cu:40-71, src/wavefront.cu:173-208). */
typedef struct wfe_server wfe_server;

typedef struct wfe_server_config {
    int32_t device;
    uint32_t max_seq_len;       /* longest pattern or text of any request */
    uint32_t cigar_stride;      /* bytes per CIGAR slot; 0 = as wfe_config */
    int32_t max_distance;       /* 0 = no limit */
    uint32_t lanes;             /* batches in flight at once, one stream each; 0 = 4 */
    uint32_t batch_pairs;       /* pairs per batch at most; 0 = 65536 */
    uint64_t memory_bytes;      /* device arena for batches in flight (and as much
                                   page-locked host memory for their results);
                                   0 = 2 GiB */
    uint32_t nbuckets;          /* length buckets of every batch, as in
                                   wfe_set_policy; 0 = one */
    uint32_t bucket_max_len[WFE_MAX_BUCKETS];
    int32_t first_tier[WFE_MAX_BUCKETS];
    uint32_t policy_flags;      /* WFE_POLICY_* */
} wfe_server_config;

/* Times (steady clock, nanoseconds) and shape of one finished request. */
typedef struct wfe_request_info {
    uint64_t submit_ns;  /* wfe_submit was called */
    uint64_t start_ns;   /* its first batch was enqueued */
    uint64_t done_ns;    /* its last result was written to the caller's buffers */
    uint32_t pairs;
    uint32_t batches;    /* batches its pairs were spread over */
} wfe_request_info;

typedef struct wfe_server_stats {
    uint64_t requests;        /* finished */
    uint64_t pairs;           /* aligned */
    uint64_t batches;         /* device batches run */
    uint64_t split_requests;  /* requests spread over more than one batch */
    uint32_t max_in_flight;   /* most batches on the device at once */
    uint32_t lanes;
    uint64_t memory_bytes;    /* arena size */
    uint64_t peak_memory;     /* most arena bytes held at once */
    uint64_t admit_ns;        /* host time the scheduler spent forming batches and
                                 enqueueing their copies and kernels */
    uint64_t finish_ns;       /* host time the finisher threads spent copying
                                 results out and finishing requests (summed
                                 over the threads) */
} wfe_server_stats;

/* Create a server (one context per lane, created with WFE_FLAG_DEVICE_ONLY,
 * the arena, the scheduler thread and up to four finisher threads that copy
 * finished batches' results into the callers' buffers).  WFE_ERR_BUSY when the device has
 * less free memory than the arena asks for. */
int wfe_server_create(const wfe_server_config* cfg, wfe_server** out);

/* Finish every submitted request, then release everything.  No other call
 * on the server (a wfe_poll waiting in another thread included) may be in
 * progress or follow. */
void wfe_server_destroy(wfe_server* srv);

/* Queue n pairs of ascii (ascii_bytes long; descriptors as in wfe_align) for
 * alignment; outputs as in wfe_align.  Returns at once with *ticket.  The
 * inputs and outputs must stay valid until wfe_poll reports the ticket
 * finished.  Checked here: every pair lies inside ascii
 * (WFE_ERR_INVALID_ARGUMENT) and is at most max_seq_len long
 * (WFE_ERR_SEQ_TOO_LONG); nothing is queued then. */
int wfe_submit(wfe_server* srv, const char* ascii, size_t ascii_bytes, const wfe_pair* pairs,
               size_t n, int32_t* dist_out, int8_t* cigar_out, uint8_t* status_out,
               uint64_t* ticket);

/* Wait up to timeout_us microseconds (0: do not wait, < 0: no limit) for a
 * request.  WFE_OK: finished and its results written; the ticket is retired
 * and info (may be NULL) filled.  WFE_ERR_TIMEOUT: not finished yet.
 * WFE_ERR_NOT_FOUND: unknown or already retired ticket.  A request whose
 * batch failed returns that error (WFE_ERR_CUDA) and is retired too. */
int wfe_poll(wfe_server* srv, uint64_t ticket, int64_t timeout_us, wfe_request_info* info);

int wfe_server_get_stats(wfe_server* srv, wfe_server_stats* out);

/* ---- host helpers --------------------------------------------------------- */

/* Number of CUDA devices (0 when there is none or no driver).  Replaces
 * cudaGetDeviceCount in src/aligner.cu:140-145. */
int wfe_device_count(int* count);

/* Name and compute capability of a device, for the CLI's banner
 * (src/aligner.cu:147-151). */
int wfe_device_name(int device, char* name, size_t cap, int* cc_major, int* cc_minor);

/* Page-locked, device-mapped host memory: buffers in it are read and written
 * by the kernels in place (see wfe_align).  Replaces the reader's
 * cudaMallocHost (utils/sequence_reader.cu:77-86). */
int wfe_host_alloc(void** p, size_t bytes);
void wfe_host_free(void* p);

/* ---- pair files ------------------------------------------------------------ */

/* A pair file read into memory: the file's bytes and one descriptor per pair
 * pointing into them (no sequence byte copied). */
typedef struct wfe_pair_file {
    char* ascii;        /* the file's bytes (+64 zero bytes) */
    size_t ascii_bytes; /* file size */
    wfe_pair* pairs;    /* n descriptors into ascii */
    size_t n;           /* pairs read */
    uint32_t longest;   /* longest pattern or text */
    int pinned;         /* ascii and pairs are page-locked (read in place by wfe_align) */
} wfe_pair_file;

/* Read up to max_pairs pairs of a ">pattern" / "<text" file (one sequence
 * per line, '\n' or "\r\n" endings) with nthreads threads; pin = 1 asks for
 * page-locked buffers.  Replaces SequenceReader::read_n_alignments
 * (utils/sequence_reader.cu:108-201), which copies every sequence into a
 * 2*l+pad slot and drops the last base of a final line without '\n'.
 * On a format error returns WFE_ERR_INVALID_ARGUMENT and writes the message
 * into err (err_cap bytes). */
int wfe_read_pair_file(const char* path, size_t max_pairs, int nthreads, int pin,
                       wfe_pair_file* out, char* err, size_t err_cap);
void wfe_free_pair_file(wfe_pair_file* f);

/* ---- host CIGAR utilities ---------------------------------------------- */

/* Text of one encoded CIGAR.  compat = 0: run-length form, e.g.
 * "20M1X129M1D3M".  compat = 1: the reference's -p printer byte for byte,
 * defects included (src/wavefront.cuh:146-184).  Returns the text length
 * (excluding the terminator); out may be NULL to size it. */
size_t wfe_format_cigar(const int8_t* cigar, size_t cigar_stride, char* out,
                        size_t out_cap, int compat);

/* Replay an encoded CIGAR against its pair on the host: M must match, X must
 * mismatch, the walk must end at (p_len, t_len).  Returns 1 if valid and
 * stores the number of X/I/D in *score.  Replaces Cigars::check_cigar
 * (src/wavefront.cuh:297-419), the reference's DEBUG-mode validator. */
int wfe_check_cigar(const char* pattern, uint32_t p_len, const char* text,
                    uint32_t t_len, const int8_t* cigar, size_t cigar_stride,
                    int32_t* score);

#ifdef __cplusplus
}
#endif

#endif /* WFE_H */

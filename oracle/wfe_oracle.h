/*
 * wfe_oracle.h -- CPU restatement of the eWFA-GPU alignment path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls
 * this code; only the test-suite, the smoke check and the CPU-baseline leg of
 * bench.py load it, and only as the oracle the GPU results are compared with,
 * or as the CPU baseline.
 *
 * Every function restates one piece of the reference (quim0/eWFA-GPU) and
 * cites the file:line it follows.  The restatement is pinned against the
 * reference's own kernels compiled for the CPU (oracle/_ref, built by
 * oracle/build_ref.sh) and against committed golden vectors produced from
 * them (tests/golden/).
 *
 * Semantics kept from the reference:
 *   - base code (c & 6) >> 1, so A=0 C=1 T=2 G=3 and N aliases G
 *     (src/wavefront_structures.h:73-83, src/kernels.cu:358);
 *   - offsets are text positions h, diagonal k = h - v
 *     (src/wavefront.cuh:35-38); target diagonal tlen - plen, target
 *     offset tlen;
 *   - every diagonal outside the previous wavefront reads -1, offsets are
 *     never clamped to the sequence bounds (src/kernels.cu:205-219,136-152);
 *   - piggy-back maximum with the tie order DEL > SUB > INS
 *     (src/kernels.cu:141-152);
 *   - termination only on the target diagonal, after the whole wavefront has
 *     been computed and extended, on exact equality (src/kernels.cu:258,268);
 *   - forward CIGAR replay with M runs stored as negative signed-char chunks
 *     of at most 127 (src/kernels.cu:397-498).
 * The distance cap of the reference (64, src/wavefront.cuh:462-466) is a
 * parameter here: max_distance = 63 reproduces the reference search range,
 * max_distance = 0 searches without limit.
 */
#ifndef WFE_ORACLE_H
#define WFE_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Operation codes of the backtrace (src/wavefront_structures.h:66-71). */
enum { WFO_OP_NOOP = 0, WFO_OP_INS = 1, WFO_OP_SUB = 2, WFO_OP_DEL = 3 };

/* Pair status codes, identical to the product's WFE_PAIR_* values. */
enum {
    WFO_PAIR_OK = 0,
    WFO_PAIR_OVER_MAX_DISTANCE = 1,
    WFO_PAIR_CIGAR_TRUNCATED = 2,
};

typedef struct wfo_counts {
    uint64_t cells;        /* wavefront cells computed (sum over d>=1 of 2d+1) */
    uint64_t extend_words; /* 16-base window compares of the reference extend */
} wfo_counts;

/* 2-bit code of one ASCII byte, (c & 6) >> 1. */
static inline uint8_t wfo_code(uint8_t c) { return (uint8_t)((c & 6u) >> 1); }

/* Pack len ASCII bases into nwords 32-bit words, 16 bases per word, base i
 * of the sequence at bits 31-2(i%16)..30-2(i%16) of word i/16; bases past len
 * (and words past the sequence) are code 0.  src/kernels.cu:313-394. */
void wfo_pack(const char* seq, uint32_t len, uint32_t* words, uint32_t nwords);

/* Extend along diagonal k from offset off: longest common prefix of the
 * pattern from v = off - k and the text from h = off, bounded by both
 * lengths.  Returns the new offset.  src/kernels.cu:27-109 (16-base windows,
 * XOR, __clz, masking past the ends).  words (may be NULL) accumulates the
 * number of 16-base windows the reference loop compares. */
int32_t wfo_extend(const uint8_t* pcodes, int32_t plen, const uint8_t* tcodes,
                   int32_t tlen, int32_t k, int32_t off, uint64_t* words);

/* Wavefront edit distance of one pair (src/kernels.cu:111-310).
 * max_distance: largest distance searched (0 = no limit; 63 = reference).
 * On success *distance = D and ops[0..D-1] holds the backtrace chain:
 * ops[d-1] is the operation chosen at score d on the path to the target,
 * i.e. the 2-bit field d-1 of the reference's WF_backtrace_result_t words.
 * ops_cap must be >= D (or ops may be NULL to skip the chain).
 * Returns WFO_PAIR_OK or WFO_PAIR_OVER_MAX_DISTANCE (then *distance =
 * max_distance + 1), or -1 on allocation failure / ops_cap too small. */
int wfo_align(const char* pattern, uint32_t plen, const char* text,
              uint32_t tlen, int32_t max_distance, int32_t* distance,
              uint8_t* ops, size_t ops_cap, wfo_counts* counts);

/* Encoded CIGAR from the backtrace chain by forward replay
 * (src/kernels.cu:397-498).  Writes at most cigar_cap bytes; if the CIGAR
 * is shorter than cigar_cap it is followed by a zero byte.  Returns
 * WFO_PAIR_OK or WFO_PAIR_CIGAR_TRUNCATED; *cigar_len = bytes of the full
 * CIGAR (also when truncated). */
int wfo_cigar(const char* pattern, uint32_t plen, const char* text,
              uint32_t tlen, int32_t distance, const uint8_t* ops,
              int8_t* cigar, size_t cigar_cap, size_t* cigar_len,
              uint64_t* words);

/* Replay an encoded CIGAR against its pair: M must match, X must mismatch,
 * and the walk must end at (plen, tlen).  src/wavefront.cuh:297-419.
 * Returns 1 if valid, 0 if not.  *score = number of X/I/D operations. */
int wfo_check_cigar(const char* pattern, uint32_t plen, const char* text,
                    uint32_t tlen, const int8_t* cigar, size_t cigar_cap,
                    int32_t* score);

/* Plain run-length text of an encoded CIGAR, e.g. "20M1X129M1D3M".
 * Returns the string length (excluding the terminator), or the length that
 * would have been needed if out_cap is too small. */
size_t wfo_format_cigar(const int8_t* cigar, size_t cigar_cap, char* out,
                        size_t out_cap);

/* The reference's -p printer, byte for byte, including its defects (the
 * character code of the following operation is printed as the M count and
 * the final M run is dropped).  src/wavefront.cuh:146-184. */
size_t wfo_format_cigar_compat(const int8_t* cigar, size_t cigar_cap,
                               char* out, size_t out_cap);

/* Levenshtein distance on the 2-bit codes by the textbook O(plen*tlen) DP;
 * independent of the wavefront code above. */
int32_t wfo_levenshtein(const char* pattern, uint32_t plen, const char* text,
                        uint32_t tlen);

/* Align n pairs with nthreads host threads (pthreads), every output as in
 * wfo_align + wfo_cigar.  Pair i: pattern at ascii + p_off[i], text at
 * ascii + t_off[i].  cigar slot i at cigar + i*cigar_stride.  Returns 0. */
int wfo_align_batch(const char* ascii, const uint64_t* p_off,
                    const uint32_t* p_len, const uint64_t* t_off,
                    const uint32_t* t_len, size_t n, int32_t max_distance,
                    int32_t* dist, int8_t* cigar, size_t cigar_stride,
                    uint8_t* status, int nthreads, wfo_counts* counts);

#ifdef __cplusplus
}
#endif

#endif /* WFE_ORACLE_H */

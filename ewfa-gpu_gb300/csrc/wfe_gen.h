/*
 * wfe_gen.h -- deterministic synthetic pair generator for the benchmark
 * workloads (pattern/text pairs in the reference's ">pattern" / "<text" file
 * format).  Workload tooling: not part of the alignment path.
 *
 * Pair i of a workload with seed s is generated from its own splitmix64
 * stream, so any range of pairs can be generated independently and in
 * parallel.  Text: i.i.d. uniform over ACGT.  Pattern: walk the text; at each
 * position, with probability p, apply an edit chosen uniformly among
 *   mismatch  (a uniformly chosen other base),
 *   insertion (a uniform base inserted before the position's base),
 *   deletion  (the position's base is dropped);
 * otherwise copy the base.  Length L is fixed when len_min == len_max, else
 * drawn log-uniformly in [len_min, len_max]; p is fixed when p_min == p_max,
 * else drawn uniformly in [p_min, p_max].
 */
#ifndef WFE_GEN_H
#define WFE_GEN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wfe_gen_config {
    uint64_t seed;
    uint32_t len_min, len_max;
    double p_min, p_max;
} wfe_gen_config;

/* Worst-case bytes of one pair (pattern can grow to 2L, text is L). */
size_t wfe_gen_pair_cap(const wfe_gen_config* cfg);

/* Generate pair `index` into pat (capacity 2*len_max) and txt (len_max). */
void wfe_gen_pair(const wfe_gen_config* cfg, uint64_t index, char* pat,
                  uint32_t* plen, char* txt, uint32_t* tlen);

/* Generate pairs [first, first+n) into one contiguous buffer, pattern then
 * text for each pair, back to back.  Returns total bytes written, or
 * (size_t)-1 if ascii_cap is too small.  Offsets are from `ascii`. */
size_t wfe_gen_batch(const wfe_gen_config* cfg, uint64_t first, size_t n,
                     char* ascii, size_t ascii_cap, uint64_t* p_off,
                     uint32_t* p_len, uint64_t* t_off, uint32_t* t_len,
                     int nthreads);

/* Write pairs [first, first+n) as a ">pattern\n<text\n" file.  Returns 0. */
int wfe_gen_file(const wfe_gen_config* cfg, uint64_t first, size_t n,
                 const char* path);

#ifdef __cplusplus
}
#endif

#endif

/*
 * ref_harness.cpp -- runs the reference's own kernels (src/kernels.cu of
 * quim0/eWFA-GPU, compiled unmodified as host C++ against ref_shim/) on the
 * CPU, one thread block at a time.  TEST INFRASTRUCTURE ONLY: it is built by
 * oracle/build_ref.sh into oracle/_ref/libwfe_ref.so when the reference
 * sources are present, and only the tests and the fixture generator load it.
 *
 * Each entry point mirrors one host step of src/wavefront.cu:
 *   ref_compact  -> compact_sequences launches   (src/wavefront.cu:76-89)
 *   ref_align    -> WF_edit_distance + generate_cigars
 *                                               (src/wavefront.cu:173-260)
 * plus the host helpers of class Cigars (src/wavefront.cuh:146-419).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <algorithm>

#include "cuda.h" /* ref_shim */

/* Cigars keeps its buffers private; the harness points them at host memory. */
#define private public
#include "wavefront.cuh"
#include "kernels.cuh"
#undef private

wfe_shim_dim3 threadIdx, blockIdx, blockDim;

/* Dynamic shared memory of the three kernels that declare it extern. */
static const size_t kShared = (size_t)1 << 24;
uint8_t shared_mem_chunk[kShared];
uint8_t sequences_sh[kShared];
edit_cigar_t cigars_ascii_sh[kShared];

static void set_dims(unsigned bx, unsigned tx, unsigned ty)
{
    blockIdx.x = bx; blockIdx.y = 0; blockIdx.z = 0;
    threadIdx.x = tx; threadIdx.y = ty; threadIdx.z = 0;
    blockDim.x = 1; blockDim.y = 1; blockDim.z = 1;
}

static Cigars make_cigars(int n, size_t cigar_max_len, WF_backtrace_result_t* data,
                          edit_cigar_t* ascii)
{
    Cigars c(n, 64, cigar_max_len, true); /* shim allocators leave NULLs */
    c.cigar_max_len = cigar_max_len;      /* exact stride requested by the caller */
    c.data = data;
    c.cigars_ascii = ascii;
    return c;
}

extern "C" {

/* Padding rules of SequenceReader (utils/sequence_reader.h:65-72). */
size_t ref_max_seq_len_unpacked(size_t seq_len)
{
    size_t u = seq_len * 2;
    return u + (4 - (u % 4));
}

size_t ref_max_seq_len_packed(size_t seq_len)
{
    size_t p = ref_max_seq_len_unpacked(seq_len) / 4;
    return p + (4 - (p % 4));
}

/* compact_sequences over n pairs.  ascii: reader layout, pattern i at
 * 2*i*unp, text at (2*i+1)*unp, zero padded.  packed: 2*packed_len bytes per
 * pair, zeroed here first as src/wavefront.cu:47,144-147 does. */
int ref_compact(const char* ascii, size_t unp, size_t packed_len, size_t n,
                char* packed)
{
    if (2 * unp > kShared) return -1;
    memset(packed, 0, 2 * packed_len * n);
    for (size_t b = 0; b < n; ++b) {
        for (unsigned y = 0; y < 2; ++y) {
            set_dims((unsigned)b, 0, y);
            compact_sequences(ascii, packed, unp, packed_len);
        }
    }
    return 0;
}

/* WF_edit_distance (max_distance 64) then generate_cigars, for n pairs packed
 * by ref_compact.  Pairs with |tlen - plen| > 63 are not run (the reference
 * would index its 129-entry history arrays out of bounds): dist = -1.
 * words: 2 per pair (the 128-bit history), cigars: cigar_max_len per pair. */
int ref_align(const char* packed, size_t packed_len, const uint32_t* plen,
              const uint32_t* tlen, size_t n, int32_t* dist, uint64_t* words,
              int8_t* cigars, size_t cigar_max_len)
{
    if (2 * packed_len + 2 * (WF_ELEMENTS(64) + 2) * 4 > kShared) return -1;
    WF_element* el = (WF_element*)calloc(n ? n : 1, sizeof(WF_element));
    WF_backtrace_result_t* res =
        (WF_backtrace_result_t*)calloc(n ? n : 1, sizeof(WF_backtrace_result_t));
    if (!el || !res) { free(el); free(res); return -2; }
    memset(cigars, 0, n * cigar_max_len);
    for (size_t i = 0; i < n; ++i) {
        el[i].alignment_idx = (int)i;
        el[i].plen = plen[i];
        el[i].tlen = tlen[i];
    }
    Cigars cg = make_cigars((int)n, cigar_max_len, res, (edit_cigar_t*)cigars);
    for (size_t b = 0; b < n; ++b) {
        long kt = (long)tlen[b] - (long)plen[b];
        if (kt > 63 || kt < -63) { res[b].distance = -1; continue; }
        set_dims((unsigned)b, 0, 0);
        WF_edit_distance(el, (SEQ_TYPE*)packed, 64, packed_len, cg);
    }
    for (size_t i = 0; i < n; ++i) {
        if (res[i].distance < 0) continue;
        /* one thread per alignment: tid = blockIdx.x * blockDim.x + threadIdx.x */
        set_dims((unsigned)i, 0, 0);
        generate_cigars(packed, el, packed_len, cg, (int)n);
    }
    for (size_t i = 0; i < n; ++i) {
        dist[i] = res[i].distance;
        words[2 * i] = res[i].words[0];
        words[2 * i + 1] = res[i].words[1];
    }
    free(el); free(res);
    return 0;
}

/* Cigars::check_cigar (src/wavefront.cuh:297-419) on one pair in reader
 * layout; returns 1 for a valid CIGAR. */
int ref_check_cigar(const char* ascii, size_t unp, int idx, uint32_t plen,
                    uint32_t tlen, const int8_t* cigar, size_t cigar_max_len)
{
    Cigars cg = make_cigars(1, cigar_max_len, NULL, NULL);
    WF_element e;
    e.alignment_idx = idx;
    e.plen = plen;
    e.tlen = tlen;
    return cg.check_cigar(0, e, ascii, unp, (const edit_cigar_t*)cigar) ? 1 : 0;
}

/* Cigars::generate_ascii_cigar (src/wavefront.cuh:146-184): the -p printer. */
size_t ref_ascii_cigar(const int8_t* cigar, size_t cigar_max_len, char* out,
                       size_t out_cap)
{
    Cigars cg = make_cigars(1, cigar_max_len, NULL, (edit_cigar_t*)cigar);
    edit_cigar_t* s = cg.generate_ascii_cigar(0);
    if (!s) return 0;
    size_t len = strnlen((char*)s, cigar_max_len * 2);
    size_t c = len < out_cap ? len : (out_cap ? out_cap - 1 : 0);
    if (out_cap) { memcpy(out, s, c); out[c] = 0; }
    free(s);
    return len;
}

/* Cigars::generate_ascii_sequence (src/wavefront.cuh:261-295): packed words
 * back to ACTG text. */
size_t ref_ascii_sequence(const char* packed, size_t len, char* out)
{
    Cigars cg = make_cigars(1, 4, NULL, NULL);
    SEQ_TYPE* s = cg.generate_ascii_sequence(packed, len);
    memcpy(out, s, len);
    free(s);
    return len;
}

/* Cigars::generate_ascii_cigar_from_bt_vector (src/wavefront.cuh:186-259):
 * expands a 128-bit history into one letter per column (M/X/I/D). */
size_t ref_cigar_from_bt(const char* pattern, int plen, const char* text,
                         int tlen, int32_t distance, const uint64_t* words,
                         char* out, size_t out_cap)
{
    WF_backtrace_result_t r;
    r.words[0] = words[0];
    r.words[1] = words[1];
    r.distance = distance;
    memset(out, 0, out_cap);
    Cigars cg = make_cigars(1, out_cap, &r, (edit_cigar_t*)out);
    cg.generate_ascii_cigar_from_bt_vector(0, text, tlen, pattern, plen);
    return strnlen(out, out_cap);
}

} /* extern "C" */

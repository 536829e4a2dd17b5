/*
 * wfe_host.cpp -- host utilities of the C ABI: CIGAR text and CIGAR
 * validation (the reference's class Cigars host methods,
 * src/wavefront.cuh:146-184 and 297-419).
 */
#include <cstdio>
#include <cstring>

#include "wfe.h"

namespace {

struct Text {
    char* out;
    size_t cap;
    size_t pos = 0;
    void put(char c)
    {
        if (pos + 1 < cap) out[pos] = c;
        ++pos;
    }
    void num(long v)
    {
        char buf[24];
        const int n = std::snprintf(buf, sizeof buf, "%ld", v);
        for (int i = 0; i < n; ++i) put(buf[i]);
    }
    size_t finish()
    {
        if (cap) out[pos < cap ? pos : cap - 1] = 0;
        return pos;
    }
};

size_t cigar_len(const int8_t* cigar, size_t stride)
{
    size_t n = 0;
    while (n < stride && cigar[n] != 0) ++n;
    return n;
}

}  // namespace

extern "C" {

size_t wfe_format_cigar(const int8_t* cigar, size_t cigar_stride, char* out, size_t out_cap, int compat)
{
    Text t{out, out ? out_cap : 0};
    const size_t n = cigar_len(cigar, cigar_stride);
    if (compat) {
        /* src/wavefront.cuh:161-181: on the first operation after M bases the
         * reference prints that operation's character code, then 'M', then the
         * operation; the last M run is never printed. */
        long pending = 0;
        for (size_t i = 0; i < n; ++i) {
            const int8_t c = cigar[i];
            if (c < 0) {
                pending += -c;
                continue;
            }
            if (pending > 0) {
                t.num(c);
                t.put('M');
                pending = 0;
            }
            t.put((char)c);
        }
        return t.finish();
    }
    long m = 0, run = 0;
    char op = 0;
    for (size_t i = 0; i < n; ++i) {
        const int8_t c = cigar[i];
        if (c < 0) {
            if (run) { t.num(run); t.put(op); run = 0; }
            m += -c;
            continue;
        }
        if (m) { t.num(m); t.put('M'); m = 0; }
        if (run && c != op) { t.num(run); t.put(op); run = 0; }
        op = (char)c;
        ++run;
    }
    if (m) { t.num(m); t.put('M'); }
    if (run) { t.num(run); t.put(op); }
    return t.finish();
}

int wfe_check_cigar(const char* pattern, uint32_t p_len, const char* text, uint32_t t_len,
                    const int8_t* cigar, size_t cigar_stride, int32_t* score)
{
    /* src/wavefront.cuh:329-409: M bases must be equal bytes, X bases unequal,
     * I consumes text, D consumes pattern, the walk ends at both ends. */
    const size_t n = cigar_len(cigar, cigar_stride);
    uint32_t pp = 0, tp = 0;
    int32_t edits = 0;
    for (size_t i = 0; i < n; ++i) {
        const int8_t c = cigar[i];
        if (c < 0) {
            for (int j = 0; j > c; --j) {
                if (pp >= p_len || tp >= t_len || pattern[pp] != text[tp]) return 0;
                ++pp;
                ++tp;
            }
        } else if (c == 'I') {
            ++tp;
            ++edits;
        } else if (c == 'D') {
            ++pp;
            ++edits;
        } else if (c == 'X') {
            if (pp >= p_len || tp >= t_len || pattern[pp] == text[tp]) return 0;
            ++pp;
            ++tp;
            ++edits;
        } else {
            return 0;
        }
    }
    if (pp != p_len || tp != t_len) return 0;
    if (score) *score = edits;
    return 1;
}

}  // extern "C"

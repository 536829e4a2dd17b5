/*
 * wfe_oracle.c -- CPU restatement of the eWFA-GPU alignment path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle of the parity tests and the CPU
 * baseline); the product library never links it.  See wfe_oracle.h for the
 * reference semantics kept and the file:line each function follows.
 */
#define _GNU_SOURCE
#include "wfe_oracle.h"

#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Packing: src/kernels.cu:313-394.  Four ASCII bytes become one byte with the
 * first base in bits 7:6; the bytes of each 32-bit word are stored so that a
 * little-endian load sees 16 bases most-significant first. */
void wfo_pack(const char* seq, uint32_t len, uint32_t* words, uint32_t nwords)
{
    const uint8_t* s = (const uint8_t*)seq;
    for (uint32_t w = 0; w < nwords; ++w) {
        uint32_t word = 0;
        for (uint32_t i = 0; i < 16; ++i) {
            uint64_t pos = (uint64_t)w * 16u + i;
            uint32_t code = pos < len ? wfo_code(s[pos]) : 0u;
            word |= code << (30u - 2u * i);
        }
        words[w] = word;
    }
}

/* ------------------------------------------------------------------------ */
/* Extend: src/kernels.cu:27-109.  The reference compares 16 bases per loop
 * trip and stops at the first trip with fewer than 16 equal bases, masking
 * positions past either end as different; the result is the longest common
 * prefix bounded by both remaining lengths, computed here 8 codes at a time. */
int32_t wfo_extend(const uint8_t* pc, int32_t plen, const uint8_t* tc,
                   int32_t tlen, int32_t k, int32_t off, uint64_t* words)
{
    int32_t v = off - k;
    int32_t h = off;
    if (v < 0 || h < 0) {
        fprintf(stderr, "wfo_extend: negative position v=%d h=%d\n", v, h);
        abort();
    }
    if (v >= plen || h >= tlen) return off;
    int32_t rem = plen - v < tlen - h ? plen - v : tlen - h;
    int32_t n = 0;
    while (n + 8 <= rem) {
        uint64_t a, b;
        memcpy(&a, pc + v + n, 8);
        memcpy(&b, tc + h + n, 8);
        if (a != b) break;
        n += 8;
    }
    while (n < rem && pc[v + n] == tc[h + n]) ++n;
    if (words) {
        /* trips of the reference loop: one per started 16-base window; a
         * window that matched completely and ended exactly at a sequence end
         * starts no further trip. */
        uint64_t trips = (uint64_t)(n / 16) + 1u;
        if (n % 16 == 0 && n > 0 && n == rem &&
            (v + n >= plen || h + n >= tlen))
            trips -= 1u;
        *words += trips;
    }
    return off + n;
}

static uint8_t* codes_of(const char* s, uint32_t len)
{
    uint8_t* c = (uint8_t*)malloc((size_t)len + 16u);
    if (!c) return NULL;
    for (uint32_t i = 0; i < len; ++i) c[i] = wfo_code((uint8_t)s[i]);
    memset(c + len, 0xff, 16); /* never equal to a code: stops the 8-wide loop */
    return c;
}

/* ------------------------------------------------------------------------ */
/* Wavefront recurrence: src/kernels.cu:111-310.
 *   d = 0:  O[0] = extend(0, 0)                         (kernels.cu:249-253)
 *   d >= 1: for k in [-d, d]
 *             del = O[k+1], sub = O[k] + 1, ins = O[k-1] + 1, with O[j] = -1
 *             for |j| > d-1                           (kernels.cu:205-219)
 *             m = max((del<<2)|3, (sub<<2)|2, (ins<<2)|1)   (kernels.cu:141-146)
 *             O'[k] = extend(k, m >> 2), op(d,k) = m & 3    (kernels.cu:149-176)
 *   stop at the first d with |kt| <= d and O'[kt] == tlen   (kernels.cu:258,268)
 * The reference carries a 128-bit forward history per diagonal:
 * hist(d,k) = hist(d-1, k + op - 2) | op << 2(d-1)  (kernels.cu:154-171).
 * Keeping op(d,k) for every cell and walking back from (D, kt) yields the same
 * chain without the 64-step limit of the 128-bit words. */
int wfo_align(const char* pattern, uint32_t plen, const char* text,
              uint32_t tlen, int32_t max_distance, int32_t* distance,
              uint8_t* ops, size_t ops_cap, wfo_counts* counts)
{
    const int32_t P = (int32_t)plen, T = (int32_t)tlen;
    const int32_t kt = T - P;
    const int32_t target = T;
    /* The unclamped recurrence reaches (plen, tlen) exactly at the edit
     * distance, which is at most max(plen, tlen). */
    int32_t limit = (P > T ? P : T) + 1;
    if (max_distance > 0 && max_distance < limit) limit = max_distance;

    uint8_t* pc = codes_of(pattern, plen);
    uint8_t* tc = codes_of(text, tlen);
    const int32_t width = 2 * (limit + 2) + 1;
    const int32_t centre = limit + 2;
    int32_t* cur = (int32_t*)malloc(sizeof(int32_t) * (size_t)width);
    int32_t* nxt = (int32_t*)malloc(sizeof(int32_t) * (size_t)width);
    size_t opcap = 1024;
    uint8_t* opm = (uint8_t*)malloc(opcap);
    int ret = -1;
    if (!pc || !tc || !cur || !nxt || !opm) goto done;
    for (int32_t i = 0; i < width; ++i) cur[i] = nxt[i] = -1;

    uint64_t words = 0, cells = 0;
    cur[centre] = wfo_extend(pc, P, tc, T, 0, 0, &words);
    int32_t d = 0;
    int found = (kt == 0 && cur[centre] == target);
    while (!found && d < limit) {
        ++d;
        size_t need = (size_t)d * (size_t)d + 2u * (size_t)d; /* cells up to d */
        if (need > opcap) {
            while (opcap < need) opcap *= 2;
            uint8_t* g = (uint8_t*)realloc(opm, opcap);
            if (!g) goto done;
            opm = g;
        }
        uint8_t* row = opm + ((size_t)d * d - 1u); /* cell (d, k) at row[k + d] */
        for (int32_t k = -d; k <= d; ++k) {
            const int32_t okp = cur[centre + k + 1];
            const int32_t ok = cur[centre + k];
            const int32_t okm = cur[centre + k - 1];
            const int32_t del_p = (int32_t)((uint32_t)okp << 2) | WFO_OP_DEL;
            const int32_t sub_p = (int32_t)((uint32_t)(ok + 1) << 2) | WFO_OP_SUB;
            const int32_t ins_p = (int32_t)((uint32_t)(okm + 1) << 2) | WFO_OP_INS;
            int32_t m = del_p > sub_p ? del_p : sub_p;
            m = m > ins_p ? m : ins_p;
            row[k + d] = (uint8_t)(m & 3);
            nxt[centre + k] = wfo_extend(pc, P, tc, T, k, m >> 2, &words);
        }
        cells += (uint64_t)(2 * d + 1);
        /* cells outside [-d, d] of the buffer just written still hold -1:
         * the two buffers alternate and the written range grows by one. */
        int32_t* t = cur; cur = nxt; nxt = t;
        if (kt >= -d && kt <= d && cur[centre + kt] == target) found = 1;
    }
    if (counts) { counts->cells += cells; counts->extend_words += words; }
    if (!found) {
        if (max_distance > 0 && d >= max_distance) {
            *distance = max_distance + 1;
            ret = WFO_PAIR_OVER_MAX_DISTANCE;
        } else {
            fprintf(stderr, "wfo_align: no termination (bug)\n");
            abort();
        }
        goto done;
    }
    *distance = d;
    if (ops) {
        if (ops_cap < (size_t)d) goto done;
        int32_t k = kt;
        for (int32_t s = d; s >= 1; --s) {
            const uint8_t op = opm[(size_t)s * s - 1u + (size_t)(k + s)];
            ops[s - 1] = op;
            k += (int32_t)op - 2;
            if (k < -(s - 1) || k > (s - 1)) {
                fprintf(stderr, "wfo_align: backtrace left the wavefront\n");
                abort();
            }
        }
        if (k != 0) { fprintf(stderr, "wfo_align: backtrace end k=%d\n", k); abort(); }
    }
    ret = WFO_PAIR_OK;
done:
    free(pc); free(tc); free(cur); free(nxt); free(opm);
    return ret;
}

/* ------------------------------------------------------------------------ */
/* CIGAR replay: src/kernels.cu:397-498 (generate_cigars). */
static void put(int8_t* cigar, size_t cap, size_t* pos, int8_t b)
{
    if (*pos < cap) cigar[*pos] = b;
    ++*pos;
}

static void put_run(int8_t* cigar, size_t cap, size_t* pos, int32_t run)
{
    for (int32_t j = 0; j < run / 127; ++j) put(cigar, cap, pos, (int8_t)-127);
    if (run % 127) put(cigar, cap, pos, (int8_t)(-(run % 127)));
}

int wfo_cigar(const char* pattern, uint32_t plen, const char* text,
              uint32_t tlen, int32_t distance, const uint8_t* ops,
              int8_t* cigar, size_t cigar_cap, size_t* cigar_len,
              uint64_t* words)
{
    uint8_t* pc = codes_of(pattern, plen);
    uint8_t* tc = codes_of(text, tlen);
    if (!pc || !tc) { free(pc); free(tc); return -1; }
    const int32_t P = (int32_t)plen, T = (int32_t)tlen;
    size_t pos = 0;
    int32_t off = 0, k = 0;
    for (int32_t d = 0; d < distance; ++d) {
        const int32_t prev = off;
        off = wfo_extend(pc, P, tc, T, k, off, words);
        put_run(cigar, cigar_cap, &pos, off - prev);
        switch (ops[d]) {
        case WFO_OP_DEL: put(cigar, cigar_cap, &pos, 'D'); --k; break;
        case WFO_OP_SUB: put(cigar, cigar_cap, &pos, 'X'); ++off; break;
        case WFO_OP_INS: put(cigar, cigar_cap, &pos, 'I'); ++k; ++off; break;
        default:
            fprintf(stderr, "wfo_cigar: bad op %u at %d\n", ops[d], d);
            abort();
        }
    }
    const int32_t prev = off;
    off = wfo_extend(pc, P, tc, T, k, off, words);
    put_run(cigar, cigar_cap, &pos, off - prev);
    if (pos < cigar_cap) cigar[pos] = 0;
    if (cigar_len) *cigar_len = pos;
    free(pc); free(tc);
    return pos > cigar_cap ? WFO_PAIR_CIGAR_TRUNCATED : WFO_PAIR_OK;
}

/* ------------------------------------------------------------------------ */
/* CIGAR validity replay: src/wavefront.cuh:297-419 (check_cigar).  Like the
 * reference it compares the raw bytes of the pair, not the 2-bit codes. */
int wfo_check_cigar(const char* pattern, uint32_t plen, const char* text,
                    uint32_t tlen, const int8_t* cigar, size_t cigar_cap,
                    int32_t* score)
{
    size_t n = 0;
    while (n < cigar_cap && cigar[n] != 0) ++n;
    uint32_t pp = 0, tp = 0;
    int32_t edits = 0;
    for (size_t i = 0; i < n; ++i) {
        const int8_t c = cigar[i];
        if (c < 0) {
            for (int j = 0; j > c; --j) {
                if (pp >= plen || tp >= tlen) return 0;
                if (pattern[pp] != text[tp]) return 0;
                ++pp; ++tp;
            }
        } else if (c == 'I') {
            ++tp; ++edits;
        } else if (c == 'D') {
            ++pp; ++edits;
        } else if (c == 'X') {
            if (pp >= plen || tp >= tlen) return 0;
            if (pattern[pp] == text[tp]) return 0;
            ++pp; ++tp; ++edits;
        } else {
            return 0;
        }
    }
    if (score) *score = edits;
    return pp == plen && tp == tlen;
}

/* ------------------------------------------------------------------------ */
static void out_put(char* out, size_t cap, size_t* pos, char c)
{
    if (*pos + 1 < cap) out[*pos] = c;
    ++*pos;
}

static void out_num(char* out, size_t cap, size_t* pos, long v)
{
    char buf[32];
    int len = snprintf(buf, sizeof buf, "%ld", v);
    for (int i = 0; i < len; ++i) out_put(out, cap, pos, buf[i]);
}

size_t wfo_format_cigar(const int8_t* cigar, size_t cigar_cap, char* out,
                        size_t out_cap)
{
    size_t n = 0;
    while (n < cigar_cap && cigar[n] != 0) ++n;
    size_t pos = 0;
    long mrun = 0;
    char op = 0;
    long oprun = 0;
    for (size_t i = 0; i <= n; ++i) {
        const int8_t c = i < n ? cigar[i] : 0;
        if (i < n && c < 0) {
            if (oprun) { out_num(out, out_cap, &pos, oprun); out_put(out, out_cap, &pos, op); oprun = 0; }
            mrun += -c;
            continue;
        }
        if (mrun) { out_num(out, out_cap, &pos, mrun); out_put(out, out_cap, &pos, 'M'); mrun = 0; }
        if (i == n) break;
        if (oprun && c != op) { out_num(out, out_cap, &pos, oprun); out_put(out, out_cap, &pos, op); oprun = 0; }
        op = (char)c;
        ++oprun;
    }
    if (oprun) { out_num(out, out_cap, &pos, oprun); out_put(out, out_cap, &pos, op); }
    if (out_cap) out[pos < out_cap ? pos : out_cap - 1] = 0;
    return pos;
}

/* src/wavefront.cuh:146-184 (generate_ascii_cigar), defects included. */
size_t wfo_format_cigar_compat(const int8_t* cigar, size_t cigar_cap,
                               char* out, size_t out_cap)
{
    size_t n = 0;
    while (n < cigar_cap && cigar[n] != 0) ++n;
    size_t pos = 0;
    long mpending = 0;
    for (size_t i = 0; i < n; ++i) {
        const int8_t c = cigar[i];
        if (c < 0) { mpending += -c; continue; }
        if (mpending > 0) {
            out_num(out, out_cap, &pos, (long)c);
            out_put(out, out_cap, &pos, 'M');
            mpending = 0;
        }
        out_put(out, out_cap, &pos, (char)c);
    }
    if (out_cap) out[pos < out_cap ? pos : out_cap - 1] = 0;
    return pos;
}

/* ------------------------------------------------------------------------ */
int32_t wfo_levenshtein(const char* pattern, uint32_t plen, const char* text,
                        uint32_t tlen)
{
    int32_t* row = (int32_t*)malloc(sizeof(int32_t) * ((size_t)tlen + 1u));
    if (!row) return -1;
    for (uint32_t j = 0; j <= tlen; ++j) row[j] = (int32_t)j;
    for (uint32_t i = 1; i <= plen; ++i) {
        int32_t diag = row[0];
        row[0] = (int32_t)i;
        const uint8_t a = wfo_code((uint8_t)pattern[i - 1]);
        for (uint32_t j = 1; j <= tlen; ++j) {
            const int32_t up = row[j];
            int32_t best = diag + (a == wfo_code((uint8_t)text[j - 1]) ? 0 : 1);
            if (up + 1 < best) best = up + 1;
            if (row[j - 1] + 1 < best) best = row[j - 1] + 1;
            diag = up;
            row[j] = best;
        }
    }
    const int32_t r = row[tlen];
    free(row);
    return r;
}

/* ------------------------------------------------------------------------ */
typedef struct batch_job {
    const char* ascii;
    const uint64_t* p_off; const uint32_t* p_len;
    const uint64_t* t_off; const uint32_t* t_len;
    size_t begin, end;
    int32_t max_distance;
    int32_t* dist; int8_t* cigar; size_t cigar_stride; uint8_t* status;
    wfo_counts counts;
} batch_job;

static void* batch_worker(void* arg)
{
    batch_job* j = (batch_job*)arg;
    size_t cap = 256;
    uint8_t* ops = (uint8_t*)malloc(cap);
    for (size_t i = j->begin; i < j->end; ++i) {
        const char* p = j->ascii + j->p_off[i];
        const char* t = j->ascii + j->t_off[i];
        const uint32_t pl = j->p_len[i], tl = j->t_len[i];
        size_t need = (size_t)(pl > tl ? pl : tl) + 2u;
        if (need > cap) { cap = need; free(ops); ops = (uint8_t*)malloc(cap); }
        int32_t d = 0;
        int st = wfo_align(p, pl, t, tl, j->max_distance, &d, ops, cap, &j->counts);
        j->dist[i] = d;
        int8_t* cg = j->cigar + i * j->cigar_stride;
        if (st == WFO_PAIR_OK) {
            st = wfo_cigar(p, pl, t, tl, d, ops, cg, j->cigar_stride, NULL,
                           &j->counts.extend_words);
        } else if (j->cigar_stride) {
            cg[0] = 0;
        }
        j->status[i] = (uint8_t)st;
    }
    free(ops);
    return NULL;
}

int wfo_align_batch(const char* ascii, const uint64_t* p_off,
                    const uint32_t* p_len, const uint64_t* t_off,
                    const uint32_t* t_len, size_t n, int32_t max_distance,
                    int32_t* dist, int8_t* cigar, size_t cigar_stride,
                    uint8_t* status, int nthreads, wfo_counts* counts)
{
    if (nthreads < 1) nthreads = 1;
    if ((size_t)nthreads > n && n > 0) nthreads = (int)n;
    batch_job* jobs = (batch_job*)calloc((size_t)nthreads, sizeof(batch_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) { free(jobs); free(th); return -1; }
    for (int t = 0; t < nthreads; ++t) {
        batch_job* j = &jobs[t];
        j->ascii = ascii; j->p_off = p_off; j->p_len = p_len;
        j->t_off = t_off; j->t_len = t_len;
        j->begin = n * (size_t)t / (size_t)nthreads;
        j->end = n * (size_t)(t + 1) / (size_t)nthreads;
        j->max_distance = max_distance;
        j->dist = dist; j->cigar = cigar; j->cigar_stride = cigar_stride;
        j->status = status;
        if (t > 0) pthread_create(&th[t], NULL, batch_worker, j);
    }
    if (nthreads > 0) batch_worker(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    if (counts) {
        for (int t = 0; t < nthreads; ++t) {
            counts->cells += jobs[t].counts.cells;
            counts->extend_words += jobs[t].counts.extend_words;
        }
    }
    free(jobs); free(th);
    return 0;
}

/*
 * wfe_gen.c -- deterministic synthetic pair generator (see wfe_gen.h).
 */
#include "wfe_gen.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static inline uint64_t sm64_next(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* uniform double in [0, 1) from the top 53 bits */
static inline double sm64_unit(uint64_t* s)
{
    return (double)(sm64_next(s) >> 11) * (1.0 / 9007199254740992.0);
}

static const char kBases[4] = {'A', 'C', 'G', 'T'};

size_t wfe_gen_pair_cap(const wfe_gen_config* cfg)
{
    return 3u * (size_t)cfg->len_max;
}

static inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Start of pair `index`'s stream: a hash of (seed, index), so that the
 * streams of neighbouring pairs are unrelated. */
static uint64_t pair_state(const wfe_gen_config* cfg, uint64_t index)
{
    return mix64(mix64(cfg->seed + 0x632BE59BD9B4E019ull) ^ mix64(index * 0xD1B54A32D192ED03ull + 1u));
}

void wfe_gen_pair(const wfe_gen_config* cfg, uint64_t index, char* pat,
                  uint32_t* plen, char* txt, uint32_t* tlen)
{
    uint64_t s = pair_state(cfg, index);
    uint32_t L = cfg->len_min;
    if (cfg->len_max > cfg->len_min) {
        const double lo = log((double)cfg->len_min);
        const double hi = log((double)cfg->len_max + 1.0);
        double x = exp(lo + (hi - lo) * sm64_unit(&s));
        L = (uint32_t)x;
        if (L < cfg->len_min) L = cfg->len_min;
        if (L > cfg->len_max) L = cfg->len_max;
    }
    double p = cfg->p_min;
    if (cfg->p_max > cfg->p_min) p = cfg->p_min + (cfg->p_max - cfg->p_min) * sm64_unit(&s);

    uint64_t bits = 0;
    int nbits = 0;
    for (uint32_t i = 0; i < L; ++i) {
        if (nbits == 0) { bits = sm64_next(&s); nbits = 32; }
        txt[i] = kBases[bits & 3u];
        bits >>= 2;
        --nbits;
    }
    uint32_t o = 0;
    for (uint32_t i = 0; i < L; ++i) {
        if (sm64_unit(&s) < p) {
            const uint64_t r = sm64_next(&s);
            const uint32_t kind = (uint32_t)(r % 3u);
            if (kind == 0) {                   /* mismatch: another base */
                uint32_t b = 0;
                while (kBases[b] != txt[i]) ++b;
                pat[o++] = kBases[(b + 1u + (uint32_t)((r >> 8) % 3u)) & 3u];
            } else if (kind == 1) {            /* insertion before the base */
                pat[o++] = kBases[(r >> 8) & 3u];
                pat[o++] = txt[i];
            }                                  /* kind 2: deletion */
        } else {
            pat[o++] = txt[i];
        }
    }
    *plen = o;
    *tlen = L;
}

typedef struct gen_job {
    const wfe_gen_config* cfg;
    uint64_t first;
    size_t begin, end;
    char* scratch;
    uint32_t* p_len; uint32_t* t_len;
    char* ascii; const uint64_t* base;
    uint64_t* p_off; uint64_t* t_off;
    int pass;
} gen_job;

static void* gen_worker(void* arg)
{
    gen_job* j = (gen_job*)arg;
    const size_t cap = wfe_gen_pair_cap(j->cfg);
    char* pat = j->scratch;
    char* txt = j->scratch + 2u * (size_t)j->cfg->len_max;
    uint64_t pos = j->pass ? j->base[0] : 0;
    (void)cap;
    for (size_t i = j->begin; i < j->end; ++i) {
        uint32_t pl, tl;
        wfe_gen_pair(j->cfg, j->first + i, pat, &pl, txt, &tl);
        if (j->pass == 0) {
            j->p_len[i] = pl;
            j->t_len[i] = tl;
        } else {
            j->p_off[i] = pos;
            memcpy(j->ascii + pos, pat, pl);
            pos += pl;
            j->t_off[i] = pos;
            memcpy(j->ascii + pos, txt, tl);
            pos += tl;
        }
    }
    return NULL;
}

size_t wfe_gen_batch(const wfe_gen_config* cfg, uint64_t first, size_t n,
                     char* ascii, size_t ascii_cap, uint64_t* p_off,
                     uint32_t* p_len, uint64_t* t_off, uint32_t* t_len,
                     int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if ((size_t)nthreads > n && n > 0) nthreads = (int)n;
    gen_job* jobs = (gen_job*)calloc((size_t)nthreads, sizeof(gen_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    uint64_t* starts = (uint64_t*)calloc((size_t)nthreads + 1u, sizeof(uint64_t));
    char* scratch = (char*)malloc((size_t)nthreads * wfe_gen_pair_cap(cfg));
    size_t total = (size_t)-1;
    if (!jobs || !th || !starts || !scratch) goto out;
    for (int pass = 0; pass < 2; ++pass) {
        for (int t = 0; t < nthreads; ++t) {
            gen_job* j = &jobs[t];
            j->cfg = cfg; j->first = first;
            j->begin = n * (size_t)t / (size_t)nthreads;
            j->end = n * (size_t)(t + 1) / (size_t)nthreads;
            j->scratch = scratch + (size_t)t * wfe_gen_pair_cap(cfg);
            j->p_len = p_len; j->t_len = t_len;
            j->ascii = ascii; j->base = &starts[t];
            j->p_off = p_off; j->t_off = t_off;
            j->pass = pass;
            if (t > 0) pthread_create(&th[t], NULL, gen_worker, j);
        }
        gen_worker(&jobs[0]);
        for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
        if (pass == 0) {
            uint64_t acc = 0;
            for (int t = 0; t < nthreads; ++t) {
                starts[t] = acc;
                for (size_t i = jobs[t].begin; i < jobs[t].end; ++i)
                    acc += (uint64_t)p_len[i] + t_len[i];
            }
            starts[nthreads] = acc;
            if (acc > ascii_cap) goto out;
        }
    }
    total = (size_t)starts[nthreads];
out:
    free(jobs); free(th); free(starts); free(scratch);
    return total;
}

int wfe_gen_file(const wfe_gen_config* cfg, uint64_t first, size_t n,
                 const char* path)
{
    FILE* f = fopen(path, "w");
    if (!f) return -1;
    char* pat = (char*)malloc(2u * (size_t)cfg->len_max + 1u);
    char* txt = (char*)malloc((size_t)cfg->len_max + 1u);
    if (!pat || !txt) { free(pat); free(txt); fclose(f); return -1; }
    for (size_t i = 0; i < n; ++i) {
        uint32_t pl, tl;
        wfe_gen_pair(cfg, first + i, pat, &pl, txt, &tl);
        fputc('>', f); fwrite(pat, 1, pl, f); fputc('\n', f);
        fputc('<', f); fwrite(txt, 1, tl, f); fputc('\n', f);
    }
    free(pat); free(txt);
    return fclose(f) == 0 ? 0 : -1;
}

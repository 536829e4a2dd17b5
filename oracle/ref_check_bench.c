/* ref_check_bench -- times the reference's own host check path
 * (Cigars::check_cigar, src/wavefront.cuh:297-419, in oracle/_ref/libwfe_ref.so
 * built from the reference sources) over every pair, on the reference
 * reader's layout (304-byte slots, utils/sequence_reader.cu:148-189), split
 * over T pthreads in contiguous shares as src/aligner.cu:45-48 splits its
 * pairs.  A CPU baseline only (validity replay, not an aligner); the input
 * file is written by oracle/ref_check_baseline.py.
 *
 *   ref_check_bench FILE N THREADS   -> one JSON line (best of 3)
 */
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "wfe_oracle.h"
int ref_check_cigar(const char* ascii, size_t unp, int idx, uint32_t plen, uint32_t tlen, const int8_t* cigar,
                    size_t cigar_max_len);
typedef struct { const char* buf; size_t unp; const uint32_t* pl; const uint32_t* tl; const int8_t* cg; size_t S;
                 size_t lo, hi; size_t good; } job_t;
static void* run(void* a) { job_t* j = a; size_t g = 0;
  for (size_t i = j->lo; i < j->hi; ++i) g += ref_check_cigar(j->buf, j->unp, (int)i, j->pl[i], j->tl[i], j->cg + i * j->S, j->S);
  j->good = g; return NULL; }
static double now(void) { struct timespec t; clock_gettime(CLOCK_MONOTONIC, &t); return t.tv_sec + 1e-9 * t.tv_nsec; }
int main(int argc, char** argv) {
  const char* path = argv[1]; size_t n = strtoull(argv[2], 0, 10); int T = atoi(argv[3]);
  if (T < 1) T = 1;
  if (T > 64) T = 64; /* the thread arrays below */
  /* raw file: n pairs as u32 plen, u32 tlen, then bytes; produced by the Python driver */
  FILE* f = fopen(path, "rb"); size_t unp = 304, S = 152;
  char* buf = calloc(2 * unp * n + 64, 1); uint32_t* pl = malloc(4 * n); uint32_t* tl = malloc(4 * n);
  int8_t* cg = malloc(S * n);
  if (fread(pl, 4, n, f) != n || fread(tl, 4, n, f) != n || fread(buf, 1, 2 * unp * n, f) != 2 * unp * n ||
      fread(cg, 1, S * n, f) != S * n) { printf("short read\n"); return 1; }
  fclose(f);
  double best = 1e9; size_t good = 0;
  for (int rep = 0; rep < 3; ++rep) {
    pthread_t th[64]; job_t jb[64];
    double t0 = now();
    for (int t = 0; t < T; ++t) { jb[t] = (job_t){buf, unp, pl, tl, cg, S, n * t / T, n * (t + 1) / T, 0};
      pthread_create(&th[t], 0, run, &jb[t]); }
    good = 0; for (int t = 0; t < T; ++t) { pthread_join(th[t], 0); good += jb[t].good; }
    double dt = now() - t0; if (dt < best) best = dt;
  }
  printf("{\"pairs\": %zu, \"threads\": %d, \"valid\": %zu, \"best_s\": %.4f, \"pairs_per_s\": %.0f}\n", n, T, good, best, n / best);
  return 0;
}

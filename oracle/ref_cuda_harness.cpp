/*
 * ref_cuda_harness.cpp -- runs the reference's own CUDA kernels on the GPU.
 * TEST AND BASELINE INFRASTRUCTURE ONLY (never part of libwfe).
 *
 * The kernels are the reference's src/kernels.cu, compiled unmodified for
 * sm_100 into oracle/_ref/ref_kernels_sm100.cubin by oracle/Makefile (target
 * ref-cubin, where the reference sources are mounted), exactly as its
 * `make SM=100 COMPUTE=100 all` compiles them.  This program restates the
 * host side that drives them -- src/aligner.cu worker() and the Sequences
 * batch loop of src/wavefront.cu -- call for call, and loads the cubin with
 * the CUDA driver API.  Two deliberate differences:
 *   - the reader's input buffer is filled from the synthetic generator
 *     instead of a file (the reference parses its file before its clock
 *     starts, src/aligner.cu:192-199, so neither is timed);
 *   - d_elements and the backtrace records are allocated 512 entries longer
 *     than the batch: generate_cigars_sh_mem reads one element and one record
 *     per thread of its last block before its bounds check
 *     (src/kernels.cu:508-539), which would otherwise read past the
 *     allocations.
 * The module is loaded before the clock starts.
 *
 *   ref_cuda_harness --cubin F -n N -l L [-b B] [-t T] [--p P] [--seed S]
 *                    [--reps R] [--dump FILE] [--steady] [--pairs-file F]
 * prints one JSON line: wall time of the timed region (src/aligner.cu:198-233)
 * and alignments per second; --dump writes every CIGAR slot (cigar_max_len
 * bytes per pair, pair order) for parity checks.  --steady times the batch
 * loop alone: every thread makes its allocations (the Sequences constructor
 * and the cudaMalloc/cudaMemset of GPU_memory_init) before the clock starts
 * and frees them after it stops; the clock covers the first batch's copy and
 * packing, every batch and the last CIGAR copy.  --pairs-file aligns given
 * pairs instead of generated ones: a u64 pair count n, a u64 slot length l
 * (the reader's -l: every sequence at most 2*l bases), u32 pattern lengths
 * [n], u32 text lengths [n], then each pair's pattern and text bytes; -n and
 * -l come from the file.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <vector>

extern "C" {
#include "wfe_gen.h"
}

namespace {

/* src/wavefront_structures.h:44-60 */
struct WF_element {
    int alignment_idx;
    size_t tlen;
    size_t plen;
};
struct WF_backtrace_result_t {
    uint64_t words[2];
    int distance;
};
/* class Cigars (src/wavefront.cuh:43-433), passed to the kernels by value:
 * public size_t cigar_max_len, then max_distance, num_cigars, data,
 * cigars_ascii. */
struct CigarsParam {
    size_t cigar_max_len;
    size_t max_distance;
    int num_cigars;
    WF_backtrace_result_t* data;
    signed char* cigars_ascii;
};

CUfunction f_compact, f_wf, f_cigars, f_cigars_sh;

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            exit(2);                                                                  \
        }                                                                             \
    } while (0)
#define CKD(call)                                                                     \
    do {                                                                              \
        CUresult r_ = (call);                                                         \
        if (r_ != CUDA_SUCCESS) {                                                     \
            const char* s_ = nullptr;                                                 \
            cuGetErrorString(r_, &s_);                                                \
            fprintf(stderr, "CUDA driver error %s at %s:%d\n", s_ ? s_ : "?", __FILE__, __LINE__); \
            exit(2);                                                                  \
        }                                                                             \
    } while (0)

struct Reader {                    /* SequenceReader (utils/sequence_reader.h) */
    size_t seq_len, max_seq_len, max_seq_len_unpacked, num_alignments;
    char* sequences_mem_unpacked;  /* pinned */
    WF_element* sequences;
};

struct Params {                    /* src/aligner.cu:29-38 */
    size_t seq_len, num_alignments, batch_size;
    unsigned tid, total_threads;
    const Reader* reader;
    signed char* dump;
    pthread_barrier_t* steady;     /* --steady: threads meet after allocating and before freeing */
    double* t_start;               /* --steady: the clock, read by thread 0 at the meetings */
    double* t_stop;
};

double now_s();

void launch(CUfunction f, unsigned gx, unsigned bx, unsigned by, unsigned smem, CUstream s, void** args)
{
    CKD(cuLaunchKernel(f, gx, 1, 1, bx, by, 1, smem, s, args, nullptr));
}

/* src/wavefront.cuh:458-505 + src/wavefront.cu, one object per thread */
struct Sequences {
    WF_element* elements;
    WF_element* d_elements = nullptr;
    size_t num_elements, max_distance = 64, batch_size;
    int batch_idx = 0, initial_alignment;
    const Reader* r;
    CigarsParam d_cigars, h_cigars;
    cudaStream_t HtD_stream;
    char* seq_dev = nullptr;
    char* seq_dev_unpacked = nullptr;
    signed char* dump;
    size_t pad;

    Sequences(WF_element* e, size_t n, size_t seq_len, size_t batch, const Reader* reader, int first,
              signed char* dump_)
        : elements(e), num_elements(n), batch_size(batch), initial_alignment(first), r(reader), dump(dump_)
    {
        pad = (batch + 511) / 512 * 512 + 512;
        const size_t cml = seq_len + (4 - seq_len % 4); /* Cigars ctor, src/wavefront.cuh:45-78 */
        d_cigars = {cml, 64, (int)batch, nullptr, nullptr};
        CK(cudaMalloc((void**)&d_cigars.data, pad * sizeof(WF_backtrace_result_t)));
        CK(cudaMemset(d_cigars.data, 0, pad * sizeof(WF_backtrace_result_t)));
        CK(cudaMalloc((void**)&d_cigars.cigars_ascii, batch * cml));
        CK(cudaMemset(d_cigars.cigars_ascii, 0, batch * cml));
        h_cigars = {cml, 64, (int)batch, nullptr, nullptr};
        CK(cudaMallocHost((void**)&h_cigars.data, batch * sizeof(WF_backtrace_result_t)));
        CK(cudaMallocHost((void**)&h_cigars.cigars_ascii, batch * cml));
        CK(cudaStreamCreate(&HtD_stream));
    }

    void GPU_memory_init() /* src/wavefront.cu:29-108 */
    {
        GPU_memory_alloc();
        GPU_memory_first_batch();
    }

    void GPU_memory_alloc() /* src/wavefront.cu:29-70: the allocations */
    {
        CK(cudaMalloc((void**)&d_elements, pad * sizeof(WF_element)));
        CK(cudaMemset(d_elements, 0, pad * sizeof(WF_element)));
        const size_t packed = r->max_seq_len;
        CK(cudaMalloc((void**)&seq_dev, packed * 2 * batch_size));
        CK(cudaMemset(seq_dev, 0, packed * 2 * batch_size));
        const size_t unp = r->max_seq_len_unpacked;
        CK(cudaMalloc((void**)&seq_dev_unpacked, unp * 2 * batch_size));
    }

    void GPU_memory_first_batch() /* src/wavefront.cu:71-108: first copy, packing, elements */
    {
        const size_t unp = r->max_seq_len_unpacked;
        const char* first = r->sequences_mem_unpacked + unp * 2 * initial_alignment;
        CK(cudaMemcpy(seq_dev_unpacked, first, unp * 2 * batch_size, cudaMemcpyHostToDevice));
        const unsigned bx = (unsigned)std::min<size_t>(r->seq_len / 4, 256);
        void* a[] = {&seq_dev_unpacked, &seq_dev, (void*)&r->max_seq_len_unpacked, (void*)&r->max_seq_len};
        launch(f_compact, (unsigned)batch_size, bx, 2, (unsigned)(unp * 2), CU_STREAM_PER_THREAD, a);
        CK(cudaMemcpyAsync(d_elements, &elements[initial_alignment], batch_size * sizeof(WF_element),
                           cudaMemcpyHostToDevice, cudaStreamPerThread));
        CK(cudaStreamSynchronize(cudaStreamPerThread));
    }

    void GPU_launch_wavefront_distance() /* src/wavefront.cu:173-208 */
    {
        const size_t remaining = num_elements - batch_size * batch_idx;
        const unsigned blocks = (unsigned)std::min(remaining, batch_size);
        const unsigned shared = (unsigned)(r->max_seq_len * 2 + 2 * (2 * max_distance + 1 + 2) * sizeof(int32_t));
        CK(cudaStreamSynchronize(HtD_stream));
        void* a[] = {&d_elements, &seq_dev, &max_distance, (void*)&r->max_seq_len, &d_cigars};
        launch(f_wf, blocks, 64, 1, shared, CU_STREAM_PER_THREAD, a);
    }

    bool is_last_iter() const { return (batch_idx + 1) * batch_size >= num_elements; }

    void GPU_prepare_memory_next_batch() /* src/wavefront.cu:127-171 */
    {
        const size_t pos = (batch_idx + 1) * batch_size;
        const size_t cur = std::min(num_elements - pos, batch_size);
        CK(cudaMemsetAsync(seq_dev, 0, r->max_seq_len * 2 * batch_size, HtD_stream));
        const unsigned bx = (unsigned)std::min<size_t>(r->seq_len / 4, 256);
        void* a[] = {&seq_dev_unpacked, &seq_dev, (void*)&r->max_seq_len_unpacked, (void*)&r->max_seq_len};
        launch(f_compact, (unsigned)batch_size, bx, 2, (unsigned)(r->max_seq_len_unpacked * 2),
               (CUstream)HtD_stream, a);
        CK(cudaMemcpyAsync(d_elements, &elements[pos + initial_alignment], cur * sizeof(WF_element),
                           cudaMemcpyHostToDevice, cudaStreamPerThread));
    }

    bool prepare_next_batch() /* src/wavefront.cu:211-330, printing off */
    {
        CK(cudaMemsetAsync(d_cigars.cigars_ascii, 0, d_cigars.num_cigars * d_cigars.cigar_max_len,
                           cudaStreamPerThread));
        const size_t pos = batch_idx * batch_size;
        int cur = (int)std::min(num_elements - pos, batch_size);
        const size_t unp = r->max_seq_len_unpacked;
        int apb;
        bool sh;
        if (unp < 400) { apb = 128; sh = true; }
        else if (unp < 800) { apb = 64; sh = true; }
        else if (unp < 1600) { apb = 32; sh = true; }
        else { apb = 512; sh = false; }
        const unsigned blocks = (unsigned)((cur + apb - 1) / apb);
        const unsigned smem = (unsigned)(apb * h_cigars.cigar_max_len);
        void* a[] = {&seq_dev, &d_elements, (void*)&r->max_seq_len, &d_cigars, &cur};
        launch(sh ? f_cigars_sh : f_cigars, blocks, (unsigned)apb, 1, sh ? smem : 0, CU_STREAM_PER_THREAD, a);
        const bool finished = is_last_iter();
        if (!finished) {
            const size_t next = (batch_idx + 1) * batch_size;
            const size_t next_n = std::min(num_elements - next, batch_size);
            const char* src = r->sequences_mem_unpacked +
                              2 * (size_t)elements[next + initial_alignment].alignment_idx * unp;
            CK(cudaMemcpyAsync(seq_dev_unpacked, src, unp * 2 * next_n, cudaMemcpyHostToDevice, HtD_stream));
        }
        CK(cudaMemcpyAsync(h_cigars.cigars_ascii, d_cigars.cigars_ascii,
                           d_cigars.num_cigars * d_cigars.cigar_max_len, cudaMemcpyDeviceToHost,
                           cudaStreamPerThread));
        CK(cudaStreamSynchronize(cudaStreamPerThread));
        if (dump)
            memcpy(dump + (initial_alignment + pos) * h_cigars.cigar_max_len, h_cigars.cigars_ascii,
                   (size_t)cur * h_cigars.cigar_max_len);
        if (!finished) GPU_prepare_memory_next_batch();
        batch_idx++;
        return !finished;
    }

    void GPU_memory_free() /* src/wavefront.cu:110-125 */
    {
        CK(cudaFree(seq_dev));
        CK(cudaFree(seq_dev_unpacked));
        CK(cudaFree(d_elements));
    }
};

void* worker(void* arg) /* src/aligner.cu:40-71 */
{
    Params* p = (Params*)arg;
    CK(cudaSetDevice(0));
    unsigned n = (unsigned)(p->num_alignments / p->total_threads);
    const unsigned skip = n * p->tid;
    if (p->tid == p->total_threads - 1) n += (unsigned)(p->num_alignments % p->total_threads);
    size_t batch = p->batch_size;
    if (batch > n) batch = n;
    Sequences s(p->reader->sequences, n, p->seq_len, batch, p->reader, (int)skip, p->dump);
    if (p->steady) {
        s.GPU_memory_alloc();
        CK(cudaDeviceSynchronize());
        pthread_barrier_wait(p->steady);
        if (p->tid == 0) *p->t_start = now_s();
        s.GPU_memory_first_batch();
    } else {
        s.GPU_memory_init();
    }
    do {
        s.GPU_launch_wavefront_distance();
    } while (s.prepare_next_batch());
    if (p->steady) {
        pthread_barrier_wait(p->steady);
        if (p->tid == 0) *p->t_stop = now_s();
    }
    s.GPU_memory_free();
    return nullptr;
}

double now_s()
{
    struct timespec t;
    clock_gettime(CLOCK_REALTIME, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

}  // namespace

int main(int argc, char** argv)
{
    const char* cubin = nullptr;
    const char* dump_path = nullptr;
    size_t n = 0, l = 0, b = 0;
    unsigned threads = 1, reps = 1;
    bool steady = false;
    const char* pairs_path = nullptr;
    double prob = 0.05;
    unsigned long long seed = 2;
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        const char* v = i + 1 < argc ? argv[i + 1] : "";
        if (!strcmp(a, "--cubin")) { cubin = v; ++i; }
        else if (!strcmp(a, "-n")) { n = strtoull(v, nullptr, 10); ++i; }
        else if (!strcmp(a, "-l")) { l = strtoull(v, nullptr, 10); ++i; }
        else if (!strcmp(a, "-b")) { b = strtoull(v, nullptr, 10); ++i; }
        else if (!strcmp(a, "-t")) { threads = (unsigned)atoi(v); ++i; }
        else if (!strcmp(a, "--p")) { prob = atof(v); ++i; }
        else if (!strcmp(a, "--seed")) { seed = strtoull(v, nullptr, 10); ++i; }
        else if (!strcmp(a, "--reps")) { reps = (unsigned)atoi(v); ++i; }
        else if (!strcmp(a, "--dump")) { dump_path = v; ++i; }
        else if (!strcmp(a, "--steady")) { steady = true; }
        else if (!strcmp(a, "--pairs-file")) { pairs_path = v; ++i; }
        else { fprintf(stderr, "unknown argument %s\n", a); return 1; }
    }
    FILE* pf = nullptr;
    std::vector<uint32_t> fpl, ftl;
    if (pairs_path) {
        pf = fopen(pairs_path, "rb");
        uint64_t hdr[2];
        if (!pf || fread(hdr, 8, 2, pf) != 2) { fprintf(stderr, "cannot read %s\n", pairs_path); return 1; }
        n = (size_t)hdr[0];
        l = (size_t)hdr[1];
        fpl.resize(n);
        ftl.resize(n);
        if (fread(fpl.data(), 4, n, pf) != n || fread(ftl.data(), 4, n, pf) != n) {
            fprintf(stderr, "short pairs file\n");
            return 1;
        }
    }
    if (!cubin || !n || !l) {
        fprintf(stderr, "usage: %s --cubin F -n N -l L [-b B] [-t T] [--p P] [--seed S] [--reps R] [--dump F]\n", argv[0]);
        return 1;
    }
    if (!b) b = n;
    if (threads < 1 || b > n) return 1;

    /* the reader's layout (utils/sequence_reader.h:65-72, sequence_reader.cu:148-189) */
    Reader r{};
    r.seq_len = l;
    r.max_seq_len_unpacked = l * 2 + (4 - (l * 2) % 4);
    r.max_seq_len = r.max_seq_len_unpacked / 4;
    r.max_seq_len += 4 - r.max_seq_len % 4;
    r.num_alignments = n;
    CK(cudaSetDevice(0));
    CK(cudaMallocHost((void**)&r.sequences_mem_unpacked, n * 2 * r.max_seq_len_unpacked));
    memset(r.sequences_mem_unpacked, 0, n * 2 * r.max_seq_len_unpacked);
    r.sequences = (WF_element*)calloc(n, sizeof(WF_element));
    wfe_gen_config gc{seed, (uint32_t)l, (uint32_t)l, prob, prob};
    std::vector<char> pat(2 * l + 1), txt(l + 1);
    for (size_t i = 0; i < n; ++i) {
        uint32_t pl, tl;
        if (pf) {
            pl = fpl[i];
            tl = ftl[i];
            if (pl > 2 * l || tl > 2 * l) { fprintf(stderr, "pair too long\n"); return 1; }
            if (pat.size() < pl + 1u) pat.resize(pl + 1u);
            if (txt.size() < tl + 1u) txt.resize(tl + 1u);
            if (fread(pat.data(), 1, pl, pf) != pl || fread(txt.data(), 1, tl, pf) != tl) {
                fprintf(stderr, "short pairs file\n");
                return 1;
            }
        } else {
            wfe_gen_pair(&gc, i, pat.data(), &pl, txt.data(), &tl);
        }
        if (pl > r.max_seq_len_unpacked || tl > r.max_seq_len_unpacked) { fprintf(stderr, "pair too long\n"); return 1; }
        memcpy(r.sequences_mem_unpacked + 2 * i * r.max_seq_len_unpacked, pat.data(), pl);
        memcpy(r.sequences_mem_unpacked + (2 * i + 1) * r.max_seq_len_unpacked, txt.data(), tl);
        r.sequences[i].alignment_idx = (int)i;
        r.sequences[i].plen = pl;
        r.sequences[i].tlen = tl;
    }

    if (pf) fclose(pf);
    CK(cudaFree(nullptr)); /* primary context */
    CKD(cuInit(0));
    CUmodule mod;
    CKD(cuModuleLoad(&mod, cubin));
    CKD(cuModuleGetFunction(&f_compact, mod, "_Z17compact_sequencesPKcPcmm"));
    CKD(cuModuleGetFunction(&f_wf, mod, "_Z16WF_edit_distancePK10WF_elementPcmm6Cigars"));
    CKD(cuModuleGetFunction(&f_cigars, mod, "_Z15generate_cigarsPKcPK10WF_elementm6Cigarsi"));
    CKD(cuModuleGetFunction(&f_cigars_sh, mod, "_Z22generate_cigars_sh_memPKcPK10WF_elementm6Cigarsi"));

    const size_t cml = l + (4 - l % 4);
    std::vector<signed char> dump;
    if (dump_path) dump.assign(n * cml, 0);

    double best = 1e30, total = 0;
    for (unsigned rep = 0; rep < reps; ++rep) {
        std::vector<pthread_t> th(threads);
        std::vector<Params> ps(threads);
        pthread_barrier_t bar;
        double ts = 0, te = 0;
        if (steady) pthread_barrier_init(&bar, nullptr, threads);
        const double t0 = now_s(); /* CLOCK_START_NO_DEBUG, src/aligner.cu:198-199 */
        for (unsigned t = 0; t < threads; ++t)
            ps[t] = Params{l, n, b, t, threads, &r, dump_path ? dump.data() : nullptr, steady ? &bar : nullptr,
                           &ts, &te};
        for (unsigned t = 1; t < threads; ++t) pthread_create(&th[t], nullptr, worker, &ps[t]);
        worker(&ps[0]);
        for (unsigned t = 1; t < threads; ++t) pthread_join(th[t], nullptr);
        double dt = now_s() - t0; /* CLOCK_STOP_NO_DEBUG, src/aligner.cu:233 */
        if (steady) {
            dt = te - ts;
            pthread_barrier_destroy(&bar);
        }
        best = std::min(best, dt);
        total += dt;
    }
    CK(cudaDeviceSynchronize());
    if (dump_path) {
        FILE* f = fopen(dump_path, "wb");
        if (!f || fwrite(dump.data(), 1, dump.size(), f) != dump.size()) return 3;
        fclose(f);
    }
    printf("{\"impl\": \"reference-cuda-sm100\", \"n\": %zu, \"l\": %zu, \"b\": %zu, \"t\": %u, \"reps\": %u, "
           "\"steady\": %s, \"best_wall_s\": %.6f, \"mean_wall_s\": %.6f, \"alignments_per_s\": %.1f}\n",
           n, l, b, threads, reps, steady ? "true" : "false", best, total / reps, (double)n / best);
    return 0;
}

/*
 * aligner.cpp -- wfe.aligner, the command line of the reference
 * (src/aligner.cu) on libwfe.
 *
 *   wfe.aligner -f FILE -n N -l L [-b B] [-t T] [-p] [--compat-print]
 *               [--max-distance D] [--check] [--device I]
 *
 * Same flags, file format and output as the reference's wfe.aligner:
 *   -f/--file, -n/--num-alignments, -l/--seq-len (required), -b/--batch-size
 *   (default n), -t/--cpu-threads (default 1; T contiguous shares of the
 *   pairs, one libwfe context each, src/aligner.cu:40-71), -p/--print-cigars
 *   ("<index>: <CIGAR>" lines), and the closing
 *   "Aligned executed. Wall time <s>s" (src/aligner.cu:198-233; the timed
 *   region, like the reference's, starts after the file is read).
 * Differences, on purpose:
 *   - -p prints the run-length CIGAR ("20M1X129M1D3M"); --compat-print
 *     prints the reference's text byte for byte (src/wavefront.cuh:146-184,
 *     which writes the next operation's character code as the M count and
 *     drops the last M run);
 *   - distances have no 63 cap unless --max-distance 63 is given;
 *   - --check replays every CIGAR against its pair (the reference's
 *     DEBUG-mode check_cigar, src/wavefront.cu:302-320) and prints the count;
 *   - a sequence longer than 2*l is an error instead of a buffer overrun, and
 *     a last line without '\n' keeps its last base.
 */
#include <algorithm>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "wfe.h"

namespace {

struct Option {
    Option(const char* n, const char* d, char s, const char* l, bool r, int k)
        : name(n), description(d), short_arg(s), long_arg(l), required(r), kind(k)
    {
    }
    const char* name;
    const char* description;
    char short_arg;
    const char* long_arg;
    bool required;
    int kind; /* 0 int, 1 string, 2 no value */
    bool parsed = false;
    long long ival = 0;
    std::string sval;
};

void print_usage(const std::vector<Option>& opts)
{
    std::fprintf(stderr, "Options:\n");
    for (const Option& o : opts) {
        const char* type = o.kind == 0 ? "int" : "string";
        if (o.kind == 2)
            std::fprintf(stderr, "\t-%c, --%-30s%s%s: %s\n", o.short_arg ? o.short_arg : ' ', o.long_arg,
                         o.required ? "(required) " : "", o.name, o.description);
        else
            std::fprintf(stderr, "\t-%c, --%-30s(%s%s) %s: %s\n", o.short_arg ? o.short_arg : ' ', o.long_arg, type,
                         o.required ? ", required" : "", o.name, o.description);
    }
}

/* -x VALUE or --long VALUE; unknown arguments are skipped; every required
 * option must be present (utils/arg_handler.c:88-138). */
bool parse_args(int argc, char** argv, std::vector<Option>& opts)
{
    Option* cur = nullptr;
    for (int i = 1; i < argc; ++i) {
        const char* a = argv[i];
        if (cur) {
            if (cur->kind == 0) cur->ival = std::atoll(a);
            else cur->sval = a;
            cur->parsed = true;
            cur = nullptr;
            continue;
        }
        if (a[0] != '-') continue;
        Option* hit = nullptr;
        for (Option& o : opts) {
            if (a[1] == '-' ? std::strcmp(a + 2, o.long_arg) == 0 : (o.short_arg && a[1] == o.short_arg))
                hit = &o;
        }
        if (!hit) continue;
        if (hit->kind == 2) hit->parsed = true;
        else cur = hit;
    }
    for (const Option& o : opts)
        if (o.required && !o.parsed) return false;
    return true;
}

double now_s()
{
    timespec t;
    clock_gettime(CLOCK_REALTIME, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

struct Share {
    size_t first = 0, n = 0;
    size_t batch = 0;  /* batch size of its context */
    size_t window = 0; /* pairs per wfe_align call: the results arrays hold that many */
    /* One buffer for the results arrays, page-locked when possible (the
     * kernels then write it in place like any pinned output), else
     * ordinary memory whose pages helper threads make present.  Never
     * initialised: the kernels write every result. */
    char* buf = nullptr;
    bool pinned = false;
    int32_t* dist = nullptr;
    int8_t* cigar = nullptr;
    uint8_t* status = nullptr;
    wfe_ctx* ctx = nullptr;
    int rc = WFE_OK;
    std::string what;
    Share() = default;
    Share(const Share&) = delete;
    Share& operator=(const Share&) = delete;
    ~Share()
    {
        if (pinned) wfe_host_free(buf);
        else delete[] buf;
    }
};

/* Results arrays of at most this many bytes per share, written over and
 * over by the share's wfe_align calls (a whole share when it fits). */
constexpr size_t kWindowBytes = size_t(256) << 20;

}  // namespace

int main(int argc, char** argv)
{
    /* Load the kernels with the CUDA context, which the pinned file read
     * creates before the clock starts, instead of at their first launch
     * inside the timed region (4-5 ms for libwfe's kernels).  A value the
     * user set is kept. */
    setenv("CUDA_MODULE_LOADING", "EAGER", 0);
    std::vector<Option> opts = {
        {"Sequences file", "File containing the sequences to align.", 'f', "file", true, 1},
        {"Number of alignments", "Number of alignments to read from the file.", 'n', "num-alignments", true, 0},
        {"Sequence length", "Maximum sequence length.", 'l', "seq-len", true, 0},
        {"Batch size", "Number of alignments per batch (default=num-alignments).", 'b', "batch-size", false, 0},
        {"Number of CPU threads", "Number of CPU threads, each with its own GPU context and streams. (default=1)",
         't', "cpu-threads", false, 0},
        {"Print CIGARS", "Print CIGARS to stdout", 'p', "print-cigars", false, 2},
        {"Compat print", "Print CIGARs exactly as the reference's -p does", 0, "compat-print", false, 2},
        {"Max distance", "Largest distance searched, 0 = no limit (63 = the reference's range)", 0,
         "max-distance", false, 0},
        {"Check", "Replay every CIGAR against its pair and report how many are valid", 0, "check", false, 2},
        {"Device", "CUDA device (default 0)", 0, "device", false, 0},
    };

    int ndev = 0;
    if (wfe_device_count(&ndev) != WFE_OK || ndev == 0) {
        std::fprintf(stderr, "No available CUDA devices detected.");
        return 1;
    }
    if (!parse_args(argc, argv, opts)) {
        print_usage(opts);
        return 1;
    }
    const int device = opts[9].parsed ? (int)opts[9].ival : 0;
    char name[256] = {0};
    int major = 0, minor = 0;
    if (wfe_device_name(device, name, sizeof name, &major, &minor) != WFE_OK) {
        std::fprintf(stderr, "No CUDA device %d.\n", device);
        return 1;
    }
    std::printf("Using device \"%s\", with compute capability %d.%d\n", name, major, minor);

    const std::string path = opts[0].sval;
    const long long n_req = opts[1].ival;
    const long long seq_len = opts[2].ival;
    long long batch = opts[3].parsed ? opts[3].ival : n_req;
    const long long threads = opts[4].parsed ? opts[4].ival : 1;
    const bool print = opts[5].parsed;
    const bool compat = opts[6].parsed;
    const long long max_distance = opts[7].parsed ? opts[7].ival : 0;
    const bool check = opts[8].parsed;
    if (threads < 1) {
        std::fprintf(stderr, "Minimum needed is 1 thread");
        return 1;
    }
    if (n_req < 0 || seq_len <= 0 || batch <= 0 || max_distance < 0) {
        print_usage(opts);
        return 1;
    }
    if (batch > n_req) {
        std::fprintf(stderr, "batch_size must be <= than the number of alignments.");
        return 1;
    }

    const uint32_t max_len = (uint32_t)(2 * seq_len); /* the reader's slot holds 2*l bases */
    const size_t N = (size_t)n_req;
    const uint32_t stride = (uint32_t)(seq_len + (4 - seq_len % 4)); /* cigar_max_len */
    const bool keep = print || check;

    /* Every share's context and results arrays are set up by a thread of
     * its own while the main thread reads the file: the shares, batch sizes
     * and sequence length are known from the arguments.  The results arrays
     * are made present page by page (the first touch of a page is the slow
     * part of the kernels writing them in place).  The timed region starts
     * after the read, as the reference's does, and includes any part of the
     * set-up still running then. */
    std::vector<Share> shares((size_t)threads);
    auto prepare = [&](size_t t) {
        Share& sh = shares[t];
        const size_t per = N / (size_t)threads;
        sh.first = per * t;
        sh.n = per + (t == (size_t)threads - 1 ? N % (size_t)threads : 0);
        sh.batch = std::min((size_t)batch, sh.n);
        if (sh.n == 0) return;
        /* Results that are printed or checked are kept for the whole
         * share; otherwise a window of up to kWindowBytes is written over
         * and over (the reference keeps one batch, src/wavefront.cu:267-300). */
        const size_t cap = std::max<size_t>(2 * sh.batch, kWindowBytes / ((size_t)stride + 5u));
        sh.window = keep ? sh.n : std::min(sh.n, cap);
        /* dist, then the CIGAR slots (the stride is a multiple of 4), then status */
        const size_t total = sh.window * (sizeof(int32_t) + (size_t)stride + 1u);
        void* pinned = nullptr;
        if (wfe_host_alloc(&pinned, total) == WFE_OK) {
            sh.buf = static_cast<char*>(pinned);
            sh.pinned = true;
        } else {
            sh.buf = new char[total];
        }
        sh.dist = reinterpret_cast<int32_t*>(sh.buf);
        sh.cigar = reinterpret_cast<int8_t*>(sh.buf + sh.window * sizeof(int32_t));
        sh.status = reinterpret_cast<uint8_t*>(sh.buf + sh.window * (sizeof(int32_t) + (size_t)stride));
        std::vector<std::thread> touch;
        if (!sh.pinned) {
            char* base = sh.buf;
            constexpr unsigned kTouchThreads = 4;
            for (unsigned k = 0; k < kTouchThreads; ++k)
                touch.emplace_back([=] {
                    const size_t page = 4096; /* every 4 KiB: covers any page size */
                    const size_t lo = total * k / kTouchThreads, hi = total * (k + 1) / kTouchThreads;
                    for (size_t i = lo; i < hi; i += page) base[i] = 0;
                    if (hi > lo) base[hi - 1] = 0;
                });
        }
        wfe_config cfg{};
        cfg.device = device;
        cfg.max_seq_len = max_len;
        cfg.batch_size = (uint32_t)sh.batch;
        cfg.max_distance = (int32_t)max_distance;
        cfg.cigar_stride = stride;
        cfg.flags = WFE_FLAG_PAGEABLE_IN_PLACE; /* the results go straight to this share's arrays */
        sh.rc = wfe_create(&cfg, &sh.ctx);
        if (sh.rc != WFE_OK) sh.what = "wfe_create";
        for (auto& x : touch) x.join();
    };
    std::vector<std::thread> setup;
    for (size_t t = 0; t < (size_t)threads; ++t) setup.emplace_back(prepare, t);
    struct Teardown {
        std::vector<std::thread>& setup;
        std::vector<Share>& shares;
        ~Teardown()
        {
            for (auto& x : setup)
                if (x.joinable()) x.join();
            for (Share& sh : shares)
                if (sh.ctx) wfe_destroy(sh.ctx);
        }
    } teardown{setup, shares};

    /* read the file before the clock starts, like the reference */
    wfe_pair_file pf{};
    char err[256] = {0};
    if (wfe_read_pair_file(path.c_str(), (size_t)n_req, (int)std::thread::hardware_concurrency(), 1, &pf, err,
                           sizeof err) != WFE_OK) {
        std::fprintf(stderr, "%s\n", err);
        std::fprintf(stderr, "Could not read the sequences from file %s\n", path.c_str());
        return 1;
    }
    struct Release {
        wfe_pair_file* f;
        ~Release() { wfe_free_pair_file(f); }
    } release{&pf};
    if (pf.longest > max_len) {
        std::fprintf(stderr, "A sequence of %u bases is longer than 2*l = %u.\n", pf.longest, max_len);
        return 1;
    }
    /* pairs the file does not have are empty (utils/sequence_reader.cu:30) */
    std::vector<wfe_pair> tail;
    if (pf.n < (size_t)n_req) {
        std::fprintf(stderr, "The file holds %zu pairs; the other %lld are empty.\n", pf.n,
                     n_req - (long long)pf.n);
        tail.assign((size_t)n_req - pf.n, wfe_pair{0, 0, 0, 0});
    }
    auto pair_at = [&](size_t i) -> const wfe_pair* { return i < pf.n ? pf.pairs + i : tail.data() + (i - pf.n); };

    const double t0 = now_s();
    for (auto& x : setup) x.join();
    for (size_t t = 0; t < shares.size(); ++t)
        if (shares[t].n && shares[t].batch < (size_t)batch)
            std::fprintf(stderr, "[Thread %zu] Changing batch size to %zu", t, shares[t].batch);
    auto worker = [&](size_t t) {
        Share& sh = shares[t];
        if (sh.n == 0 || sh.rc != WFE_OK) return;
        wfe_ctx* ctx = sh.ctx;
        const size_t window = sh.window;
        /* the pairs of this share: in the file's pinned descriptors, or the
         * empty tail */
        std::vector<wfe_pair> mine;
        const wfe_pair* src = pf.pairs + sh.first;
        if (sh.first + sh.n > pf.n) {
            mine.resize(sh.n);
            for (size_t i = 0; i < sh.n; ++i) mine[i] = *pair_at(sh.first + i);
            src = mine.data();
        }
        for (size_t c0 = 0; c0 < sh.n && sh.rc == WFE_OK; c0 += window) {
            sh.rc = wfe_align(ctx, pf.ascii, pf.ascii_bytes, src + c0, std::min(window, sh.n - c0), sh.dist,
                              sh.cigar, sh.status);
        }
        if (sh.rc != WFE_OK) sh.what = "wfe_align";
        wfe_destroy(ctx);
        sh.ctx = nullptr;
    };
    {
        std::vector<std::thread> th;
        for (size_t t = 1; t < (size_t)threads; ++t) th.emplace_back(worker, t);
        worker(0);
        for (auto& x : th) x.join();
    }
    for (const Share& sh : shares) {
        if (sh.rc != WFE_OK) {
            std::fprintf(stderr, "%s failed: %s\n", sh.what.c_str(), wfe_strerror(sh.rc));
            return 1;
        }
    }
    if (print) {
        std::vector<char> line(4u * stride + 64u);
        for (const Share& sh : shares)
            for (size_t i = 0; i < sh.n; ++i) {
                wfe_format_cigar(&sh.cigar[i * stride], stride, line.data(), line.size(), compat ? 1 : 0);
                std::printf("%zu: %s\n", sh.first + i, line.data());
            }
    }
    const double secs = now_s() - t0;

    if (check) {
        size_t good = 0, over = 0;
        for (const Share& sh : shares)
            for (size_t i = 0; i < sh.n; ++i) {
                if (sh.status[i] != WFE_PAIR_OK) {
                    ++over;
                    continue;
                }
                const wfe_pair* q = pair_at(sh.first + i);
                int32_t score = -1;
                if (wfe_check_cigar(pf.ascii + q->p_off, q->p_len, pf.ascii + q->t_off, q->t_len,
                                    &sh.cigar[i * stride], stride, &score) && score == sh.dist[i])
                    ++good;
            }
        std::fprintf(stderr, "Correct alignments: %zu/%zu (%zu not aligned: over the distance limit or slot)\n",
                     good, N - over, over);
    }
    std::printf("Aligned executed. Wall time %fs\n", secs);
    return 0;
}

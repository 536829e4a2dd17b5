/*
 * seqfile.cpp -- pair-file reader (see seqfile.h).
 *
 * The reference reads the file line by line with getline and copies every
 * sequence into a slot of 2*l+pad bytes of one pinned buffer
 * (utils/sequence_reader.cu:108-201).  Here the file is read once into one
 * page-locked buffer and the pairs are described in place: threads count
 * the lines of their share of the buffer, a prefix sum numbers them, and a
 * second pass writes one descriptor per pair (line 2i is pattern i, line
 * 2i+1 its text).  No sequence byte is copied.
 */
#include "seqfile.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <thread>

namespace wfe {

namespace {

void* alloc_buf(size_t bytes, bool pin)
{
    if (pin) {
        void* p = nullptr;
        if (wfe_host_alloc(&p, bytes) == WFE_OK) return p;
        return nullptr;
    }
    return std::malloc(bytes ? bytes : 1);
}

void free_buf(void* p, bool pin)
{
    if (!p) return;
    if (pin)
        wfe_host_free(p);
    else
        std::free(p);
}

/* Lines that start in [begin, end) of buf[0..size). */
size_t count_lines(const char* buf, size_t size, size_t begin, size_t end)
{
    size_t n = 0;
    size_t pos = begin;
    while (pos < end && pos < size) {
        ++n;
        const void* nl = std::memchr(buf + pos, '\n', size - pos);
        if (!nl) break;
        pos = (size_t)((const char*)nl - buf) + 1;
    }
    return n;
}

/* first line start at or after `at` */
size_t line_start(const char* buf, size_t size, size_t at)
{
    if (at == 0) return 0;
    if (at >= size) return size;
    const void* nl = std::memchr(buf + at - 1, '\n', size - (at - 1));
    return nl ? (size_t)((const char*)nl - buf) + 1 : size;
}

}  // namespace

PairFile::~PairFile()
{
    free_buf(data, pinned);
    free_buf(pairs, pinned);
}

bool read_pair_file(const std::string& path, size_t max_pairs, int nthreads, bool pin, PairFile& pf)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        pf.error = "Could not open the file " + path;
        return false;
    }
    std::fseek(f, 0, SEEK_END);
    const long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (sz < 0) {
        std::fclose(f);
        pf.error = "Could not size the file " + path;
        return false;
    }
    pf.bytes = (size_t)sz;
    pf.pinned = pin;
    pf.data = (char*)alloc_buf(pf.bytes + 64, pin);
    if (!pf.data && pin) {
        pf.pinned = pin = false;
        pf.data = (char*)alloc_buf(pf.bytes + 64, false);
    }
    if (!pf.data) {
        std::fclose(f);
        pf.error = "Could not allocate memory.";
        return false;
    }
    if (pf.bytes && std::fread(pf.data, 1, pf.bytes, f) != pf.bytes) {
        std::fclose(f);
        pf.error = "Could not read the file " + path;
        return false;
    }
    std::fclose(f);
    std::memset(pf.data + pf.bytes, 0, 64);

    const char* buf = pf.data;
    const size_t size = pf.bytes;
    if (nthreads < 1) nthreads = 1;
    if (size < (size_t)nthreads * 4096u) nthreads = 1;
    std::vector<size_t> lo(nthreads), hi(nthreads), lines(nthreads), first(nthreads + 1);
    for (int t = 0; t < nthreads; ++t) {
        lo[t] = line_start(buf, size, size * (size_t)t / (size_t)nthreads);
        hi[t] = line_start(buf, size, size * (size_t)(t + 1) / (size_t)nthreads);
    }
    {
        std::vector<std::thread> th;
        for (int t = 1; t < nthreads; ++t)
            th.emplace_back([&, t] { lines[t] = count_lines(buf, size, lo[t], hi[t]); });
        lines[0] = count_lines(buf, size, lo[0], hi[0]);
        for (auto& x : th) x.join();
    }
    first[0] = 0;
    for (int t = 0; t < nthreads; ++t) first[t + 1] = first[t] + lines[t];
    const size_t total_lines = first[nthreads];
    pf.n = std::min(max_pairs, (total_lines + 1) / 2);
    pf.pairs = (wfe_pair*)alloc_buf(sizeof(wfe_pair) * (pf.n ? pf.n : 1), pin);
    if (!pf.pairs) {
        pf.error = "Could not allocate memory.";
        return false;
    }
    std::memset(pf.pairs, 0, sizeof(wfe_pair) * (pf.n ? pf.n : 1));

    std::vector<std::string> errs(nthreads);
    std::vector<uint32_t> longest(nthreads, 0);
    auto fill = [&](int t) {
        size_t pos = lo[t];
        size_t li = first[t];
        while (pos < hi[t] && li / 2 < pf.n) {
            const void* nl = std::memchr(buf + pos, '\n', size - pos);
            size_t end = nl ? (size_t)((const char*)nl - buf) : size;
            const size_t next = nl ? end + 1 : size;
            if (end > pos && buf[end - 1] == '\r') --end;
            const bool text = (li & 1) != 0;
            const char want = text ? '<' : '>';
            if (end == pos || buf[pos] != want) {
                char msg[96];
                std::snprintf(msg, sizeof msg, "Invalid sequence format on line %zu.", li);
                errs[t] = msg;
                return;
            }
            const uint64_t off = pos + 1;
            const uint64_t len = end - pos - 1;
            if (len > 0xffffffffu) {
                errs[t] = "sequence too long";
                return;
            }
            wfe_pair& q = pf.pairs[li / 2];
            if (text) {
                q.t_off = off;
                q.t_len = (uint32_t)len;
            } else {
                /* the text fields belong to the text line, which another
                 * thread may be writing; a missing text line leaves them 0 */
                q.p_off = off;
                q.p_len = (uint32_t)len;
            }
            longest[t] = std::max(longest[t], (uint32_t)len);
            ++li;
            pos = next;
        }
    };
    {
        std::vector<std::thread> th;
        for (int t = 1; t < nthreads; ++t) th.emplace_back(fill, t);
        fill(0);
        for (auto& x : th) x.join();
    }
    for (int t = 0; t < nthreads; ++t) {
        if (!errs[t].empty()) {
            pf.error = errs[t];
            return false;
        }
        pf.longest = std::max(pf.longest, longest[t]);
    }
    return true;
}

}  // namespace wfe

extern "C" int wfe_read_pair_file(const char* path, size_t max_pairs, int nthreads, int pin, wfe_pair_file* out,
                                  char* err, size_t err_cap)
{
    if (!path || !out) return WFE_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof *out);
    wfe::PairFile* pf = new (std::nothrow) wfe::PairFile();
    if (!pf) return WFE_ERR_OUT_OF_MEMORY;
    if (!wfe::read_pair_file(path, max_pairs, nthreads, pin != 0, *pf)) {
        if (err && err_cap) {
            std::strncpy(err, pf->error.c_str(), err_cap - 1);
            err[err_cap - 1] = 0;
        }
        const bool oom = pf->error.find("allocate") != std::string::npos;
        delete pf;
        return oom ? WFE_ERR_OUT_OF_MEMORY : WFE_ERR_INVALID_ARGUMENT;
    }
    out->ascii = pf->data;
    out->ascii_bytes = pf->bytes;
    out->pairs = pf->pairs;
    out->n = pf->n;
    out->longest = pf->longest;
    out->pinned = pf->pinned ? 1 : 0;
    pf->data = nullptr; /* ownership moves to *out */
    pf->pairs = nullptr;
    delete pf;
    return WFE_OK;
}

extern "C" void wfe_free_pair_file(wfe_pair_file* f)
{
    if (!f) return;
    if (f->pinned) {
        wfe_host_free(f->ascii);
        wfe_host_free(f->pairs);
    } else {
        std::free(f->ascii);
        std::free(f->pairs);
    }
    std::memset(f, 0, sizeof *f);
}

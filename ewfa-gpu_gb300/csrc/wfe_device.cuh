/*
 * wfe_device.cuh -- device building blocks shared by the libwfe kernels.
 *
 * Packed sequence layout (the reference's, src/kernels.cu:313-394): 16 bases
 * per 32-bit word, base i at bits 31-2(i%16)..30-2(i%16) of word i/16, 2-bit
 * code (c & 6) >> 1 (src/wavefront_structures.h:73-83).
 *
 * In shared memory a sequence is kept as "overlapped pairs": Q[w] = {x:
 * W[w+1], y: W[w]}, so the 16-base window starting at any base v is one
 * 64-bit load and one funnel shift: window(v) = funnelshift_l(Q[v/16].x,
 * Q[v/16].y, 2*(v%16)).
 */
#ifndef WFE_DEVICE_CUH
#define WFE_DEVICE_CUH

#include <stdint.h>
#include <cuda_runtime.h>

#include "wfe.h"

namespace wfe {

constexpr unsigned kFull = 0xffffffffu;

/* Operation codes (src/wavefront_structures.h:66-71). */
constexpr int kOpIns = 1, kOpSub = 2, kOpDel = 3;

/* Four ASCII bytes (first base in the low byte) -> one byte c0c1c2c3 with
 * c0 in bits 7:6.  The multiply gathers the four 2-bit codes, which sit at
 * bits 0, 8, 16, 24, into bits 30, 28, 26, 24 without carries. */
__device__ __forceinline__ uint32_t pack4(uint32_t w)
{
    const uint32_t x = (w & 0x06060606u) >> 1;
    return (x * 0x40100401u) >> 24;
}

/* Sixteen ASCII bytes -> one packed word. */
__device__ __forceinline__ uint32_t pack16(uint4 b)
{
    return (pack4(b.x) << 24) | (pack4(b.y) << 16) | (pack4(b.z) << 8) | pack4(b.w);
}

/* Where the bases of pair i live. */
struct Layout {
    const char* ascii;      /* device ASCII buffer */
    const wfe_pair* pairs;  /* descriptor layout; NULL = strided layout */
    const uint32_t* plen;   /* strided layout lengths */
    const uint32_t* tlen;
    uint64_t stride;        /* strided layout: pattern i at 2*i*stride, text at (2i+1)*stride */
    uint64_t base_off;      /* descriptor offsets are relative to ascii - base_off */
    uint64_t ascii_bytes;   /* descriptor bytes must lie below this offset (0 = unchecked) */
};

struct PairRef {
    const char* p;
    const char* t;
    uint32_t plen, tlen;
    bool in_range;          /* both sequences lie inside the checked buffer */
};

/* Where the bases of a pair of the descriptor layout live, from its
 * descriptor d. */
__device__ __forceinline__ PairRef pair_from_desc(const Layout& L, const wfe_pair& d)
{
    PairRef r;
    r.p = L.ascii + (d.p_off - L.base_off);
    r.t = L.ascii + (d.t_off - L.base_off);
    r.plen = d.p_len;
    r.tlen = d.t_len;
    r.in_range = true;
    if (L.ascii_bytes)
        r.in_range = d.p_off <= L.ascii_bytes && d.p_len <= L.ascii_bytes - d.p_off &&
                     d.t_off <= L.ascii_bytes && d.t_len <= L.ascii_bytes - d.t_off;
    return r;
}

__device__ __forceinline__ PairRef get_pair(const Layout& L, uint32_t i)
{
    PairRef r;
    r.in_range = true;
    if (L.pairs) {
        const wfe_pair d = L.pairs[i];
        r = pair_from_desc(L, d);
    } else {
        r.p = L.ascii + 2ull * i * L.stride;
        r.t = r.p + L.stride;
        r.plen = L.plen[i];
        r.tlen = L.tlen[i];
        if (L.ascii_bytes) r.in_range = r.plen <= L.stride && r.tlen <= L.stride;
    }
    return r;
}

/* Packed word w of a sequence of len bytes at s, produced by a group of G
 * lanes, words w0+g for g in [0, G).  The sequence is read in aligned 16-byte
 * blocks (every block holds at least one base of the sequence); the bytes
 * before s are shifted out and the bases at or past len are cleared.
 * Returns the word for lane g (0 if w0+g >= nw).  All lanes of `mask` call. */
template <int G>
__device__ __forceinline__ uint32_t packed_word(const char* s, uint32_t len,
                                                uint32_t w0, int g, unsigned mask)
{
    const uint32_t nw = (len + 15u) >> 4;
    const uintptr_t a = reinterpret_cast<uintptr_t>(s);
    const uint32_t sh = (uint32_t)(a & 15u);
    const uint4* base = reinterpret_cast<const uint4*>(a - sh);
    const uint32_t nblk = (sh + len + 15u) >> 4;
    const uint32_t w = w0 + (uint32_t)g;
    uint32_t x0 = 0;
    if (w < nw) x0 = pack16(__ldg(base + w));
    const uint32_t nb = __shfl_down_sync(mask, x0, 1, G);
    uint32_t W = x0;
    if (sh != 0) {
        uint32_t x1 = nb;
        if (g == G - 1 || w + 1 >= nw) x1 = (w + 1 < nblk) ? pack16(__ldg(base + w + 1)) : 0u;
        W = __funnelshift_l(x1, x0, 2u * sh);
    }
    if (w < nw) {
        const uint32_t r = len - 16u * w;
        if (r < 16u) W &= ~0u << (2u * (16u - r));
    } else {
        W = 0;
    }
    return W;
}

/* Pack a sequence into overlapped pairs Q[0..nw) (see top of file) by a
 * group of G lanes; Q[nw-1].x = 0.  When the sequence spans at most RMAX*G
 * aligned blocks, every lane issues all of its block loads first (blocks g,
 * g+G, ...) and the neighbour block for the funnel shift comes from one
 * rotating shuffle per word; longer sequences take the word-by-word loop.
 * The caller syncs the group afterwards. */
template <int G, int RMAX>
__device__ __forceinline__ void load_packed(const char* s, uint32_t len, uint2* Q,
                                            int g, unsigned mask)
{
    const uint32_t nw = (len + 15u) >> 4;
    if (nw == 0) return;
    const uintptr_t a = reinterpret_cast<uintptr_t>(s);
    const uint32_t sh = (uint32_t)(a & 15u);
    const uint4* base = reinterpret_cast<const uint4*>(a - sh);
    const uint32_t nblk = (sh + len + 15u) >> 4;
    if (nblk <= (uint32_t)(RMAX * G)) {
        uint32_t x[RMAX + 1];
#pragma unroll
        for (int r = 0; r < RMAX; ++r) {
            const uint32_t b = (uint32_t)(g + r * G);
            x[r] = b < nblk ? pack16(__ldg(base + b)) : 0u;
        }
        x[RMAX] = 0u;
#pragma unroll
        for (int r = 0; r < RMAX; ++r) {
            if ((uint32_t)(r * G) >= nw) break;
            /* block w+1 is lane g+1's block r, or lane 0's block r+1 for the
             * last lane */
            const uint32_t y = (g == 0) ? x[r + 1] : x[r];
            const uint32_t nb = __shfl_sync(mask, y, (g + 1) & (G - 1), G);
            const uint32_t w = (uint32_t)(g + r * G);
            uint32_t W = sh ? __funnelshift_l(nb, x[r], 2u * sh) : x[r];
            if (w < nw) {
                const uint32_t rem = len - 16u * w;
                if (rem < 16u) W &= ~0u << (2u * (16u - rem));
                Q[w].y = W;
                if (w > 0) Q[w - 1].x = W;
            }
        }
    } else {
        for (uint32_t w0 = 0; w0 < nw; w0 += G) {
            const uint32_t W = packed_word<G>(s, len, w0, g, mask);
            const uint32_t w = w0 + (uint32_t)g;
            if (w < nw) {
                Q[w].y = W;
                if (w > 0) Q[w - 1].x = W;
            }
        }
    }
    if (g == 0) Q[nw - 1].x = 0u;
}

/* Coalesced load of the pairs of a warp whose groups each align one pair:
 * when every byte of the warp's patterns and texts lies in one span of at
 * most SPAN aligned 16-byte blocks (pairs stored one after another), the 32
 * lanes read the span in consecutive blocks -- whole 512-byte rows per
 * instruction instead of one short run per group, which the CPU-GPU link
 * serves 20% faster -- pack every block to a 32-bit word and keep the words
 * in `words` (SPAN per warp).  Every aligned block of [lo, hi) is read --
 * lo the warp's lowest base address, hi one past its highest -- including
 * blocks that fall in gaps between the pairs and hold none of their bases.
 * That is safe because the span is at most SPAN * 16 bytes, less than one
 * 4 KiB page: the whole span lies within the page of its first block and
 * the page of its last, and both of those blocks hold a base, so both pages
 * are mapped.  A SPAN above 256 would break that argument (the static
 * assertion below).  Returns the span's first block address (16-aligned), or
 * 0 when the span is too long (then nothing was read).  All 32 lanes call;
 * p/t/lp/lt are the calling lane's group's pair (lengths 0 for a group
 * without one). */
template <int SPAN>
__device__ __forceinline__ uintptr_t load_warp_span(const char* p, uint32_t lp, const char* t, uint32_t lt,
                                                    uint32_t* words, int lane)
{
    static_assert(SPAN * 16 <= 4096, "a span must fit in one 4 KiB page (see above)");
    unsigned long long lo = ~0ull, hi = 0ull;
    if (lp) {
        lo = min(lo, (unsigned long long)(uintptr_t)p);
        hi = max(hi, (unsigned long long)(uintptr_t)p + lp);
    }
    if (lt) {
        lo = min(lo, (unsigned long long)(uintptr_t)t);
        hi = max(hi, (unsigned long long)(uintptr_t)t + lt);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(kFull, lo, o));
        hi = max(hi, __shfl_xor_sync(kFull, hi, o));
    }
    if (hi == 0ull) return 0;
    const unsigned long long a0 = lo & ~15ull;
    const unsigned long long nblk = (hi - a0 + 15ull) >> 4;
    if (nblk > (unsigned long long)SPAN) return 0;
    const uint4* base = reinterpret_cast<const uint4*>((uintptr_t)a0);
    constexpr int R = (SPAN + 31) / 32;
    /* every load of the lane is issued before the first is used: over the
     * CPU-GPU link each round trip costs microseconds */
    uint4 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t b = (uint32_t)(lane + 32 * r);
        v[r] = b < nblk ? __ldg(base + b) : make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint32_t b = (uint32_t)(lane + 32 * r);
        if (b < nblk) words[b] = pack16(v[r]);
    }
    __syncwarp();
    return (uintptr_t)a0;
}

/* Overlapped packed pairs Q[0..nw) of a sequence of len bytes at s (see top
 * of file) from the packed blocks of a warp span starting at a0, by a group
 * of G lanes (words w = g, g+G, ...); Q[nw-1].x = 0.  The same words as
 * load_packed. */
template <int G>
__device__ __forceinline__ void pack_from_span(const uint32_t* words, uintptr_t a0, const char* s, uint32_t len,
                                               uint2* Q, int g)
{
    const uint32_t nw = (len + 15u) >> 4;
    if (nw == 0) return;
    const uintptr_t a = reinterpret_cast<uintptr_t>(s);
    const uint32_t sh = (uint32_t)(a & 15u);
    const uint32_t b0 = (uint32_t)((a - sh - a0) >> 4);
    const uint32_t nblk = (sh + len + 15u) >> 4;
    for (uint32_t w = (uint32_t)g; w < nw; w += G) {
        const uint32_t x0 = words[b0 + w];
        uint32_t W = x0;
        if (sh != 0) {
            const uint32_t x1 = (w + 1 < nblk) ? words[b0 + w + 1] : 0u;
            W = __funnelshift_l(x1, x0, 2u * sh);
        }
        const uint32_t rem = len - 16u * w;
        if (rem < 16u) W &= ~0u << (2u * (16u - rem));
        Q[w].y = W;
        if (w > 0) Q[w - 1].x = W;
    }
    if (g == 0) Q[nw - 1].x = 0u;
}

/* The best of a cell's three candidates, with the operation in the low two
 * bits (src/kernels.cu:136-152): deletion from diagonal k+1 (its offset),
 * mismatch from k (offset + 1), insertion from k-1 (offset + 1); the
 * largest offset wins and equal offsets go to the larger operation code,
 * DEL > SUB > INS.  An offset of -1 (outside the previous wavefront) gives a
 * deletion of -1 and candidates 2 and 1 for the others, as in the
 * reference.  Written as multiply-adds and one three-way maximum. */
__device__ __forceinline__ int piggyback_max(int up, int self, int dn)
{
    const int del_p = (int)((unsigned)up * 4u + (unsigned)kOpDel);
    const int sub_p = (int)((unsigned)self * 4u + (unsigned)(4 + kOpSub));
    const int ins_p = (int)((unsigned)dn * 4u + (unsigned)(4 + kOpIns));
    return __vimax3_s32(del_p, sub_p, ins_p);
}

/* 16-base window of a packed sequence starting at base v. */
__device__ __forceinline__ uint32_t window(const uint2* Q, int v)
{
    const uint2 q = Q[v >> 4];
    return __funnelshift_l(q.x, q.y, (uint32_t)(v & 15) << 1);
}

/* Extend along diagonal k from offset off (src/kernels.cu:27-109): the
 * longest common prefix of pattern[v..] and text[h..], v = off - k, h = off,
 * bounded by both lengths, 16 bases per trip.  Returns the new offset. */
__device__ __forceinline__ int extend_lane(const uint2* QP, const uint2* QT,
                                           int plen, int tlen, int k, int off)
{
    int v = off - k, h = off;
    /* unsigned compares: a negative position (impossible for cells inside
     * the wavefront) can never index the shared-memory sequences */
    while ((unsigned)v < (unsigned)plen && (unsigned)h < (unsigned)tlen) {
        const uint32_t x = window(QP, v) ^ window(QT, h);
        int n = __clz(x) >> 1;
        n = min(n, min(plen - v, tlen - h));
        v += n;
        h += n;
        if (n < 16) break;
    }
    return h;
}

/* The same longest common prefix computed by a group of G lanes at once:
 * lane g compares the window 16*g bases further on, a ballot finds the first
 * window that is not a full match.  Returns the run length.  All lanes of
 * the group call with the same arguments.
 * A warp-wide group (G = 32, one pair per warp) first compares the first
 * window on every lane -- the same shared-memory words, so one broadcast
 * read -- and a run shorter than 16 bases, the common case at high error
 * rates, is then known on every lane without the vote and shuffle. */
template <int G>
__device__ __forceinline__ int group_extend(const uint2* QP, const uint2* QT, int plen,
                                            int tlen, int k, int off, int g, int grp,
                                            unsigned gmask)
{
    const int v0 = off - k, h0 = off;
    int total = 0;
    if constexpr (G == 32) {
        int n = 0;
        if ((unsigned)v0 < (unsigned)plen && (unsigned)h0 < (unsigned)tlen) {
            const uint32_t x = window(QP, v0) ^ window(QT, h0);
            n = min(__clz(x) >> 1, min(plen - v0, tlen - h0));
        }
        if (n < 16) return n;
        total = 16;
    }
    for (;;) {
        const int v = v0 + total + 16 * g, h = h0 + total + 16 * g;
        int n = 0;
        if ((unsigned)v < (unsigned)plen && (unsigned)h < (unsigned)tlen) {
            const uint32_t x = window(QP, v) ^ window(QT, h);
            n = min(__clz(x) >> 1, min(plen - v, tlen - h));
        }
        const unsigned sb = __ballot_sync(gmask, n < 16);
        const unsigned rel = (G == 32) ? sb : ((sb >> (grp * G)) & ((1u << (G & 31)) - 1u));
        if (rel) {
            const int first = __ffs((int)rel) - 1;
            const int nf = __shfl_sync(gmask, n, first, G);
            return total + 16 * first + nf;
        }
        total += 16 * G;
    }
}

__device__ __forceinline__ int8_t op_letter(int op)
{
    return op == kOpDel ? (int8_t)'D' : (op == kOpSub ? (int8_t)'X' : (int8_t)'I');
}

/* Encoded CIGAR bytes of steps 0..last of a replayed chain
 * (src/kernels.cu:397-498), by a group of G lanes: runs[d] is the run of M
 * bases before operation d (chain[d], the operation of score d+1).  Lane g
 * takes steps g, g+G, ...: each step's bytes are its run as chunks of at
 * most 127 (-127, ..., -(run % 127)) and then its operation letter (none for
 * step D and for a step at bad_at); an inclusive shuffle scan over the group
 * gives the step's first byte, and every lane writes its own bytes into buf
 * (cap bytes; positions past cap are counted but not written).  Returns the
 * full length on every lane. */
template <int G>
__device__ __forceinline__ int encode_runs(const int* runs, const uint8_t* chain, int D, int last, int bad_at,
                                           int8_t* buf, uint32_t cap, int g, unsigned gmask)
{
    int total = 0;
    for (int base = 0; base <= last; base += G) {
        const int d = base + g;
        int r = 0, letter = 0, nb = 0;
        if (d <= last) {
            r = runs[d];
            letter = (d < D && d != bad_at) ? (int)op_letter(chain[d]) : 0;
            nb = r / 127 + (r % 127 != 0) + (letter != 0);
        }
        int x = nb;
#pragma unroll
        for (int sft = 1; sft < G; sft <<= 1) {
            const int y = __shfl_up_sync(gmask, x, sft, G);
            if (g >= sft) x += y;
        }
        uint32_t pos = (uint32_t)(total + x - nb);
        if (d <= last) {
            for (int j = 0; j < r / 127; ++j) {
                if (pos < cap) buf[pos] = (int8_t)-127;
                ++pos;
            }
            if (r % 127) {
                if (pos < cap) buf[pos] = (int8_t)(-(r % 127));
                ++pos;
            }
            if (letter) {
                if (pos < cap) buf[pos] = (int8_t)letter;
                ++pos;
            }
        }
        total += __shfl_sync(gmask, x, G - 1, G);
    }
    return total;
}

/* Forward replay of an operation chain into an encoded CIGAR
 * (src/kernels.cu:397-498) by a group of G lanes.  chain[d] is the operation
 * of score d+1.
 *   1. In order of d, the run of M bases before operation d comes from a
 *      group-parallel extend from (k, off), starting at (0, 0); runs[d]
 *      keeps it (lane 0 writes).
 *   2. encode_runs writes the bytes.
 * Returns the full CIGAR length on every lane, or -1 - length if the chain
 * holds a code other than INS/SUB/DEL: the CIGAR then stops after that
 * step's run, like the reference's "Incorrect backtrace" exit
 * (src/kernels.cu:471-478). */
template <int G>
__device__ __forceinline__ int replay_chain(const uint2* QP, const uint2* QT, int plen, int tlen,
                                            const uint8_t* chain, int D, int* runs, int8_t* buf,
                                            uint32_t cap, int g, int grp, unsigned gmask)
{
    int k = 0, off = 0, bad_at = -1;
    for (int d = 0; d <= D; ++d) {
        const int run = group_extend<G>(QP, QT, plen, tlen, k, off, g, grp, gmask);
        if (g == 0) runs[d] = run;
        off += run;
        if (d == D) break;
        const int op = chain[d];
        if (op == kOpDel) {
            --k;
        } else if (op == kOpSub) {
            ++off;
        } else if (op == kOpIns) {
            ++k;
            ++off;
        } else {
            bad_at = d;
            break;
        }
    }
    const int last = bad_at >= 0 ? bad_at : D;
    __syncwarp(gmask);
    const int total = encode_runs<G>(runs, chain, D, last, bad_at, buf, cap, g, gmask);
    return bad_at >= 0 ? -1 - total : total;
}

/* Copy a staged CIGAR of `len` bytes (plus terminator when it fits) from
 * shared to global memory by a group; pads to whole 32-bit words with zeros
 * inside the slot when the slot size allows word stores. */
template <int G>
__device__ __forceinline__ void store_cigar(int8_t* stage, uint32_t len, uint32_t cap,
                                            int8_t* dst, int g, unsigned gmask)
{
    uint32_t nbytes = len < cap ? len + 1u : cap;
    if (g == 0 && len < cap) stage[len] = 0;
    if ((cap & 3u) == 0u && (reinterpret_cast<uintptr_t>(dst) & 3u) == 0u) {
        const uint32_t nwords = (nbytes + 3u) >> 2;
        if (g == 0)
            for (uint32_t b = nbytes; b < nwords * 4u; ++b) stage[b] = 0;
        __syncwarp(gmask);
        const uint32_t* s32 = reinterpret_cast<const uint32_t*>(stage);
        uint32_t* d32 = reinterpret_cast<uint32_t*>(dst);
        for (uint32_t i = (uint32_t)g; i < nwords; i += G) d32[i] = s32[i];
    } else {
        __syncwarp(gmask);
        for (uint32_t i = (uint32_t)g; i < nbytes; i += G) dst[i] = stage[i];
    }
}

}  // namespace wfe

#endif

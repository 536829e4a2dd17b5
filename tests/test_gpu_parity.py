"""GPU parity: libwfe's CUDA path against the reference's golden vectors and
against the CPU oracle, through the C ABI.  Integer work: every comparison is
bit-exact (distance, status and the bytes of each CIGAR up to and including
its terminator)."""
import os

import numpy as np
import pytest

import oracle as O
import wfe

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_vectors.npz")


def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN)
    a = z["ascii"].tobytes()
    seqs = [(a[o[0]:o[0] + o[1]], a[o[2]:o[2] + o[3]]) for o in z["offsets"]]
    ascii, pairs = wfe.pairs_from_list(seqs)
    return z, seqs, ascii, pairs


def cigar_bytes(row):
    """Encoded CIGAR up to and including its terminator (or the full slot)."""
    row = np.asarray(row, dtype=np.int8)
    nz = np.flatnonzero(row == 0)
    return row[: nz[0] + 1].tobytes() if len(nz) else row.tobytes()


def assert_same_cigars(got, want, idx=None):
    idx = range(len(got)) if idx is None else idx
    for i in idx:
        assert cigar_bytes(got[i]) == cigar_bytes(want[i]), f"pair {i}"


def oracle_run(ascii, pairs, stride, max_distance=0):
    return O.align_batch(ascii, pairs["p_off"], pairs["p_len"], pairs["t_off"], pairs["t_len"], stride,
                         max_distance=max_distance, nthreads=os.cpu_count() or 1)


def compare_with_oracle(ascii, pairs, stride, dist, cg, st, max_distance=0):
    od, ocg, ost, _ = oracle_run(ascii, pairs, stride, max_distance)
    bad = np.flatnonzero((od != dist) | (ost != st))
    assert len(bad) == 0, f"{len(bad)} pairs differ, first {bad[:5]}: gpu {dist[bad[:5]]} oracle {od[bad[:5]]}"
    assert_same_cigars(cg, ocg)


# ---------------------------------------------------------------------------
# golden vectors of the reference itself

def test_golden_host_api(golden):
    """wfe_align (descriptor layout) with the reference's search range."""
    z, seqs, ascii, pairs = golden
    with wfe.Context(max_seq_len=300, max_distance=63, cigar_stride=152) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    ok = z["dist"] < 64
    np.testing.assert_array_equal(dist[ok], z["dist"][ok])
    assert (st[ok] == wfe.PAIR_OK).all()
    assert_same_cigars(cg, z["cigars"], np.flatnonzero(ok))
    # over the reference's cap: the reference's distance 64, no CIGAR
    assert (dist[~ok] == 64).all() and (st[~ok] == wfe.PAIR_OVER_MAX_DISTANCE).all()
    assert (cg[~ok, 0] == 0).all()


def test_golden_strided_reference_layout(golden):
    """wfe_align_strided on the reference reader's buffer (304-byte slots)."""
    z, seqs, _, _ = golden
    unp = 150 * 2 + (4 - (150 * 2) % 4)
    buf = np.zeros(2 * unp * len(seqs), dtype=np.uint8)
    for i, (p, t) in enumerate(seqs):
        buf[2 * i * unp: 2 * i * unp + len(p)] = np.frombuffer(p, np.uint8)
        buf[(2 * i + 1) * unp: (2 * i + 1) * unp + len(t)] = np.frombuffer(t, np.uint8)
    pl = np.array([len(p) for p, _ in seqs], np.uint32)
    tl = np.array([len(t) for _, t in seqs], np.uint32)
    with wfe.Context(max_seq_len=300, max_distance=63, cigar_stride=152, batch_size=128) as ctx:
        dist, cg, st = ctx.align_strided(buf, unp, pl, tl)
    ok = z["dist"] < 64
    np.testing.assert_array_equal(dist[ok], z["dist"][ok])
    assert_same_cigars(cg, z["cigars"], np.flatnonzero(ok))


def test_golden_unlimited_distance(golden):
    """No cap: every pair, the 18 over the reference's cap included, gets
    the oracle's distance and CIGAR."""
    z, seqs, ascii, pairs = golden
    with wfe.Context(max_seq_len=300, cigar_stride=400) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    compare_with_oracle(ascii, pairs, 400, dist, cg, st)
    assert (dist[z["dist"] >= 64] >= 64).all()
    for i, (p, t) in enumerate(seqs):
        assert O.levenshtein(p, t) == dist[i]


def test_golden_device_api_and_pack(golden):
    torch = torch_cuda()
    z, seqs, ascii, pairs = golden
    n = len(seqs)
    d_ascii = torch.from_numpy(ascii).cuda()
    d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
    d_dist = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_cg = torch.zeros(n * 152, dtype=torch.int8, device="cuda")
    d_st = torch.zeros(n, dtype=torch.uint8, device="cuda")
    with wfe.Context(max_seq_len=300, max_distance=63, cigar_stride=152) as ctx:
        ctx.align_device(d_ascii, d_pairs, n, 300, d_dist, d_cg, d_st, torch.cuda.current_stream())
        torch.cuda.synchronize()
    dist = d_dist.cpu().numpy()
    cg = d_cg.cpu().numpy().reshape(n, 152)
    ok = z["dist"] < 64
    np.testing.assert_array_equal(dist[ok], z["dist"][ok])
    assert_same_cigars(cg, z["cigars"], np.flatnonzero(ok))
    # the packing kernel against the reference's compact_sequences words
    wps = z["packed"].shape[2] // 4
    d_words = torch.full((n * 2 * wps,), -1, dtype=torch.int32, device="cuda")
    wfe.pack_device(d_ascii, d_pairs, n, d_words, wps, torch.cuda.current_stream())
    torch.cuda.synchronize()
    words = d_words.cpu().numpy().view(np.uint32).reshape(n, 2, wps)
    np.testing.assert_array_equal(words, z["packed"].view("<u4").reshape(n, 2, wps))


def test_golden_cigar_from_history(golden):
    """The CIGAR kernel fed the reference's own 128-bit histories."""
    torch = torch_cuda()
    z, seqs, ascii, pairs = golden
    n = len(seqs)
    d_ascii = torch.from_numpy(ascii).cuda()
    d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
    d_dist = torch.from_numpy(z["dist"].astype(np.int32)).cuda()
    d_hist = torch.from_numpy(z["words"].view(np.int64).reshape(-1)).cuda()
    d_cg = torch.zeros(n * 152, dtype=torch.int8, device="cuda")
    d_st = torch.zeros(n, dtype=torch.uint8, device="cuda")
    wfe.cigar_from_history_device(d_ascii, d_pairs, n, 300, d_dist, d_hist, d_cg, 152, d_st,
                                  torch.cuda.current_stream())
    torch.cuda.synchronize()
    cg = d_cg.cpu().numpy().reshape(n, 152)
    st = d_st.cpu().numpy()
    ok = z["dist"] < 64
    assert (st[ok] == wfe.PAIR_OK).all()
    assert_same_cigars(cg, z["cigars"], np.flatnonzero(ok))
    assert (st[~ok] == wfe.PAIR_OVER_MAX_DISTANCE).all()


# ---------------------------------------------------------------------------
# synthetic workloads against the oracle

@pytest.mark.parametrize("n,L,p,seed", [
    (10000, 150, 0.02, 1),   # plain method, small
    (100000, 150, 0.05, 2),  # one batch of the short-read throughput workload
])
def test_short_reads(n, L, p, seed):
    ascii, pairs = wfe.generate(n, L, p_min=p, seed=seed)
    with wfe.Context(max_seq_len=2 * L, cigar_stride=wfe.reference_cigar_stride(L)) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    compare_with_oracle(ascii, pairs, wfe.reference_cigar_stride(L), dist, cg, st)


def test_high_error_pairs_cross_every_tier():
    """Distances from 0 to ~330 (lengths 100-600, edit probability up to
    0.9) start in the 8-lane tier and are handed on through every tier."""
    ascii, pairs = wfe.generate(6000, 100, 600, p_min=0.0, p_max=0.9, seed=21)
    with wfe.Context(max_seq_len=1200, cigar_stride=2000) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
        stats = ctx.stats()
    assert dist.max() > 271
    assert all(stats["tier_passed"][t] > 0 for t in range(4)), stats
    compare_with_oracle(ascii, pairs, 2000, dist, cg, st)


def test_long_reads_sample():
    ascii, pairs = wfe.generate(1500, 1000, p_min=0.10, seed=3)
    with wfe.Context(max_seq_len=2000, cigar_stride=1004) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    assert dist.mean() > 64
    compare_with_oracle(ascii, pairs, 1004, dist, cg, st)


def test_mixed_lengths_sample():
    ascii, pairs = wfe.generate(1500, 100, 1500, p_min=0.01, p_max=0.15, seed=4)
    with wfe.Context(max_seq_len=3000, cigar_stride=3004) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    compare_with_oracle(ascii, pairs, 3004, dist, cg, st)


def test_edge_cases():
    seqs = [(b"", b""), (b"A", b""), (b"", b"ACGT"), (b"ACGT", b"ACGT"), (b"A" * 40, b"C" * 40),
            (b"ACGTN", b"ACGTG"), (b"acgt", b"ACGT"), (b"A" * 299, b"A" * 300), (b"T" * 300, b""),
            (b"G" * 16, b"G" * 16), (b"G" * 17, b"G" * 15), (b"ACGT" * 75, b"TGCA" * 75)]
    for L in range(1, 40):
        seqs.append((bytes(b"ACGT"[(i * 7 + L) % 4] for i in range(L)), bytes(b"ACGT"[(i * 5) % 4] for i in range(L))))
    ascii, pairs = wfe.pairs_from_list(seqs)
    with wfe.Context(max_seq_len=300, cigar_stride=604) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    compare_with_oracle(ascii, pairs, 604, dist, cg, st)
    assert dist[0] == 0 and cg[0, 0] == 0
    assert dist[2] == 4 and wfe.format_cigar(cg[2]) == "4I"


def test_unaligned_offsets_and_batches():
    """Sequences at every byte alignment, several batches, both pipeline stages."""
    ascii, pairs = wfe.generate(3000, 150, p_min=0.05, seed=8)
    shifted = np.zeros(len(ascii) + 64, np.uint8)
    shifted[7:7 + len(ascii)] = ascii
    pairs2 = pairs.copy()
    pairs2["p_off"] += 7
    pairs2["t_off"] += 7
    with wfe.Context(max_seq_len=300, batch_size=512) as ctx:
        d1, c1, s1 = ctx.align(ascii, pairs)
        d2, c2, s2 = ctx.align(shifted, pairs2)
        assert ctx.stats()["batches"] == 12
    np.testing.assert_array_equal(d1, d2)
    assert_same_cigars(c1, c2)
    compare_with_oracle(ascii, pairs, 152, d1, c1, s1)


def test_two_stages_in_the_scratch_tiers():
    """Host calls keep two batches in flight on two streams; with small
    batches of pairs whose distances need tiers 3-6, both stages' chains run
    those tiers at the same time, each on its own scratch."""
    torch_cuda()
    ascii, pairs = wfe.generate(3000, 300, 2600, p_min=0.2, p_max=0.45, seed=41)
    with wfe.Context(max_seq_len=2700, batch_size=150, cigar_stride=3000) as ctx:
        ctx.set_policy([2700], [3])  # the register tiers first, so that chains pass through 3-6
        d1, c1, s1 = ctx.align(ascii, pairs)
        st = ctx.stats()
        assert st["batches"] == 20 and st["tier_passed"][3] > 0 and st["tier_passed"][4] > 0, st
        d2, c2, s2 = ctx.align(_pinned(ascii), _pinned(pairs))
    np.testing.assert_array_equal(d1, d2)
    assert_same_cigars(c1, c2)
    compare_with_oracle(ascii, pairs, 3000, d1, c1, s1)


def test_device_call_of_several_batches_on_two_streams():
    """wfe_align_device over more than batch_size pairs alternates its
    batches between the caller's stream and a stream of the context, each
    with its own scratch of tiers 2-6.  Results equal one-stream calls
    (FLAG_NO_PIPELINE) and the oracle's, and work enqueued on the caller's
    stream after the call sees every batch's results."""
    torch = torch_cuda()
    ascii, pairs = wfe.generate(3000, 300, 2600, p_min=0.2, p_max=0.45, seed=43)
    n, stride = len(pairs), 3000
    d_ascii = torch.from_numpy(ascii).cuda()
    d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
    out = {}
    for flags in (0, wfe.FLAG_NO_PIPELINE):
        d_dist = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_cg = torch.zeros(n * stride, dtype=torch.int8, device="cuda")
        d_st = torch.full((n,), 255, dtype=torch.uint8, device="cuda")
        s = torch.cuda.Stream()
        with wfe.Context(max_seq_len=2700, batch_size=150, cigar_stride=stride, flags=flags) as ctx:
            ctx.set_policy([2700], [3])  # chains through the scratch tiers 3-6
            for _ in range(2):
                ctx.align_device(d_ascii, d_pairs, n, 2700, d_dist, d_cg, d_st, s)
                with torch.cuda.stream(s):
                    # runs after the call on the same stream: must see all of it
                    unset = int((d_st == 255).sum().item())
                assert unset == 0
            st = ctx.stats()
        assert st["batches"] == 40 and st["tier_passed"][3] > 0 and st["tier_passed"][4] > 0, st
        out[flags] = (d_dist.cpu().numpy(), d_cg.view(n, stride).cpu().numpy(), d_st.cpu().numpy())
    a, b = out[0], out[wfe.FLAG_NO_PIPELINE]
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[2], b[2])
    assert_same_cigars(a[1], b[1])
    compare_with_oracle(ascii, pairs, stride, *a)


def test_warp_span_layouts():
    """Tier 0 loads a warp's 8 pairs as one coalesced span when they lie
    within 2,560 bytes.  Layouts that exercise it: each warp's 16 sequences
    stored in shuffled order (texts before patterns), random gaps and
    alignments, empty sequences, spans on both sides of the limit, and warps
    with one sequence far away (the per-group load).  Results equal the
    oracle's and the back-to-back layout's, staged and read in place."""
    rng = np.random.default_rng(23)
    ascii, pairs = wfe.generate(4096, 150, p_min=0.05, seed=23)
    seqs = [(ascii[q["p_off"]: q["p_off"] + q["p_len"]].tobytes(), ascii[q["t_off"]: q["t_off"] + q["t_len"]].tobytes())
            for q in pairs]
    for i in rng.choice(len(seqs), 40, replace=False):
        seqs[i] = (b"", seqs[i][1]) if i % 2 else (seqs[i][0], b"")

    def filler(k):
        return rng.choice(np.frombuffer(b"ACGT", np.uint8), size=k).tobytes()

    buf = bytearray(filler(int(rng.integers(0, 16))))
    far = bytearray()
    far_at = {}
    offs = np.zeros((len(seqs), 2), np.uint64)
    for w0 in range(0, len(seqs), 8):
        w = w0 // 8
        pieces = [(i, s) for i in range(w0, w0 + 8) for s in (0, 1)]
        order = rng.permutation(len(pieces))
        start = len(buf)
        for j, o in enumerate(order):
            i, s = pieces[o]
            if w % 16 == 5 and j == len(order) - 1:
                far_at[(i, s)] = len(far)   # placed 10 KB after the main buffer below
                far += seqs[i][s] + filler(7)
                continue
            if w % 7 == 3 and j == len(order) - 1:
                # pad so that the span lands within 40 bytes either side of 2,560
                span = len(buf) - start + len(seqs[i][s])
                buf += filler(max(0, 2540 + int(rng.integers(0, 41)) - span))
            else:
                buf += filler(int(rng.integers(0, 6)))
            offs[i, s] = len(buf)
            buf += seqs[i][s]
    base_far = len(buf) + 10000
    buf += filler(10000) + far + b"\0" * 64
    for (i, s), at in far_at.items():
        offs[i, s] = base_far + at
    big = np.frombuffer(bytes(buf), np.uint8).copy()
    lay = np.zeros(len(seqs), wfe.PAIR_DTYPE)
    lay["p_off"], lay["t_off"] = offs[:, 0], offs[:, 1]
    lay["p_len"] = [len(p) for p, _ in seqs]
    lay["t_len"] = [len(t) for _, t in seqs]
    for i in range(0, len(seqs), 97):   # the layout holds the sequences it claims
        assert big[lay["p_off"][i]: lay["p_off"][i] + lay["p_len"][i]].tobytes() == seqs[i][0]
        assert big[lay["t_off"][i]: lay["t_off"][i] + lay["t_len"][i]].tobytes() == seqs[i][1]

    flat_ascii, flat_pairs = wfe.pairs_from_list(seqs)
    with wfe.Context(max_seq_len=300, batch_size=1000, cigar_stride=152) as ctx:
        want = ctx.align(flat_ascii, flat_pairs)
        staged = ctx.align(big, lay)
        in_place = ctx.align(_pinned(big), _pinned(lay))
        assert ctx.stats()["mapped_batches"] == 5
    for got in (staged, in_place):
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[2], want[2])
        assert_same_cigars(got[1], want[1])
    compare_with_oracle(big, lay, 152, *in_place)


def test_scattered_pairs_gather_path():
    """Pairs that point all over a large buffer go through the pinned gather."""
    ascii, pairs = wfe.generate(2000, 150, p_min=0.05, seed=9)
    perm = np.random.default_rng(0).permutation(len(pairs))
    big = np.zeros(len(ascii) * 300, np.uint8)
    pairs2 = pairs.copy()
    for j, i in enumerate(perm):
        base = j * 150 * 300 // 2
        big[base: base + pairs["p_len"][i]] = ascii[pairs["p_off"][i]: pairs["p_off"][i] + pairs["p_len"][i]]
        big[base + 320: base + 320 + pairs["t_len"][i]] = ascii[pairs["t_off"][i]: pairs["t_off"][i] + pairs["t_len"][i]]
        pairs2[i]["p_off"], pairs2[i]["t_off"] = base, base + 320
    with wfe.Context(max_seq_len=300, batch_size=700) as ctx:
        d1, c1, s1 = ctx.align(ascii, pairs)
        d2, c2, s2 = ctx.align(big, pairs2)
    np.testing.assert_array_equal(d1, d2)
    assert_same_cigars(c1, c2)


def test_cigar_truncation_and_caps():
    ascii, pairs = wfe.generate(500, 150, p_min=0.3, seed=12)
    with wfe.Context(max_seq_len=300, cigar_stride=16) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    compare_with_oracle(ascii, pairs, 16, dist, cg, st)
    assert (st == wfe.PAIR_CIGAR_TRUNCATED).any()
    with wfe.Context(max_seq_len=300, max_distance=20) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    compare_with_oracle(ascii, pairs, 152, dist, cg, st, max_distance=20)
    assert (st == wfe.PAIR_OVER_MAX_DISTANCE).any()


def test_too_long_rejected():
    ascii, pairs = wfe.generate(4, 200, p_min=0.05, seed=1)
    with wfe.Context(max_seq_len=150) as ctx:
        with pytest.raises(wfe.WfeError) as e:
            ctx.align(ascii, pairs)
    assert e.value.code == wfe.ERR_SEQ_TOO_LONG


def test_full_short_read_workload_properties():
    """All 1,000,000 pairs of the short-read workload: every CIGAR replays
    against its pair and scores its distance; a 1-in-50 sample matches the
    oracle byte for byte."""
    ascii, pairs = wfe.generate(1000000, 150, p_min=0.05, seed=2)
    with wfe.Context(max_seq_len=300, batch_size=100000) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    assert (st == 0).all()
    # replay: sum of M/X/D consumes the pattern, M/X/I the text, X+I+D = dist
    # (only the bytes before each terminator count)
    live = np.cumsum(cg == 0, axis=1) == 0
    mruns = np.where(live & (cg < 0), -cg.astype(np.int64), 0).sum(1)
    nx = (live & (cg == ord("X"))).sum(1)
    ni = (live & (cg == ord("I"))).sum(1)
    nd = (live & (cg == ord("D"))).sum(1)
    np.testing.assert_array_equal(nx + ni + nd, dist)
    np.testing.assert_array_equal(mruns + nx + nd, pairs["p_len"])
    np.testing.assert_array_equal(mruns + nx + ni, pairs["t_len"])
    sample = np.arange(0, len(pairs), 50)
    sub_ascii, sub_pairs = ascii, pairs[sample]
    od, ocg, ost, _ = oracle_run(sub_ascii, sub_pairs, 152)
    np.testing.assert_array_equal(dist[sample], od)
    assert_same_cigars(cg[sample], ocg)


def _pinned(a):
    import torch
    t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True).numpy().view(a.dtype).reshape(a.shape)
    t[...] = a
    return t


def test_pinned_buffers_read_and_written_in_place():
    """Pinned inputs are read by the kernels in place (no staging copy) and
    pinned outputs written in place; results equal the staged path's, for
    every combination, with both input layouts."""
    torch_cuda()
    ascii, pairs = wfe.generate(30000, 150, p_min=0.05, seed=13)
    stride = 152
    with wfe.Context(max_seq_len=300, batch_size=7000, cigar_stride=stride) as ctx:
        want = ctx.align(ascii, pairs)
        assert ctx.stats()["mapped_batches"] == 0
        for pin_in in (False, True):
            for pin_out in (False, True):
                a = _pinned(ascii) if pin_in else ascii
                p = _pinned(pairs) if pin_in else pairs
                n = len(pairs)
                out = (np.zeros(n, np.int32), np.zeros((n, stride), np.int8), np.zeros(n, np.uint8))
                if pin_out:
                    out = tuple(_pinned(o) for o in out)
                ctx.reset_stats()
                got = ctx.align(a, p, out=out)
                assert (ctx.stats()["mapped_batches"] > 0) == pin_in
                np.testing.assert_array_equal(got[0], want[0])
                np.testing.assert_array_equal(got[2], want[2])
                assert_same_cigars(got[1], want[1])
    compare_with_oracle(ascii, pairs, stride, *want)


def test_pinned_pairs_in_any_order():
    """Pinned descriptor layout read in place: pairs swapped in from far
    away, and batches whose first pair lies after their last, give the same
    results as the staged path."""
    torch_cuda()
    ascii, pairs = wfe.generate(20000, 150, p_min=0.05, seed=16)
    rng = np.random.default_rng(16)
    order = np.arange(len(pairs))
    a, b = rng.choice(len(pairs), 300, replace=False), rng.choice(len(pairs), 300, replace=False)
    order[a], order[b] = order[b], order[a]
    order[5000:6000] = order[5000:6000][::-1]   # first pair of a batch after its last
    mixed = pairs[order]
    with wfe.Context(max_seq_len=300, batch_size=3000, cigar_stride=152) as ctx:
        want = ctx.align(ascii, mixed)
        got = ctx.align(_pinned(ascii), _pinned(mixed))
        assert ctx.stats()["mapped_batches"] > 0
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[2], want[2])
    assert_same_cigars(got[1], want[1])
    compare_with_oracle(ascii, mixed, 152, *want)


def test_pinned_bad_descriptors_flagged_per_pair():
    """In place, a descriptor outside the buffer or a sequence over
    max_seq_len is reported per pair; nothing outside the buffer is read."""
    torch_cuda()
    ascii, pairs = wfe.generate(200, 150, p_min=0.05, seed=14)
    pairs = pairs.copy()
    pairs[3]["p_off"] = len(ascii) + 1000          # beyond the buffer
    pairs[5]["t_len"] = len(ascii)                 # runs past the end
    pairs[7]["p_off"] = np.uint64(2**63)           # wraps
    a, p = _pinned(ascii), _pinned(pairs)
    with wfe.Context(max_seq_len=160, cigar_stride=152) as ctx:
        d, cg, st = ctx.align(a, p)
    assert st[3] == wfe.PAIR_OUT_OF_RANGE and st[5] == wfe.PAIR_OUT_OF_RANGE and st[7] == wfe.PAIR_OUT_OF_RANGE
    too_long = (pairs["p_len"] > 160) | (pairs["t_len"] > 160)
    too_long[[3, 5, 7]] = False
    assert (st[too_long] == wfe.PAIR_TOO_LONG).all()
    ok = np.ones(len(pairs), bool)
    ok[[3, 5, 7]] = False
    ok &= ~too_long
    assert (st[ok] == wfe.PAIR_OK).all()
    od, ocg, ost, _ = oracle_run(ascii, pairs[ok], 152)
    np.testing.assert_array_equal(d[ok], od)


def test_pageable_buffers_in_place_with_the_flag():
    """WFE_FLAG_PAGEABLE_IN_PLACE: plain (pageable) inputs and outputs,
    including output arrays whose pages were never touched, are used in place
    through the CPU's page tables.  Results equal the staged path's in both
    layouts, and bad descriptors are flagged per pair as with pinned buffers."""
    torch_cuda()
    ascii, pairs = wfe.generate(60000, 150, p_min=0.05, seed=17)
    n, stride = len(pairs), 152
    with wfe.Context(max_seq_len=300, batch_size=7000, cigar_stride=stride) as ctx:
        want = ctx.align(ascii, pairs)
        assert ctx.stats()["mapped_batches"] == 0
    flags = wfe.FLAG_PAGEABLE_IN_PLACE
    with wfe.Context(max_seq_len=300, batch_size=7000, cigar_stride=stride, flags=flags) as ctx:
        # fresh pages: 9 MB of CIGAR slots, made present by several host threads
        out = (np.empty(n, np.int32), np.empty((n, stride), np.int8), np.empty(n, np.uint8))
        got = ctx.align(ascii, pairs, out=out)
        assert ctx.stats()["mapped_batches"] == 9
        assert ctx.stats()["h2d_bytes"] == 0 and ctx.stats()["d2h_bytes"] == 0
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[2], want[2])
        assert_same_cigars(got[1], want[1])
        # pinned outputs with pageable inputs, and the reverse
        got = ctx.align(ascii, pairs, out=tuple(_pinned(o) for o in out))
        np.testing.assert_array_equal(got[0], want[0])
        assert_same_cigars(got[1], want[1])
        got = ctx.align(_pinned(ascii), _pinned(pairs))
        np.testing.assert_array_equal(got[0], want[0])
        assert_same_cigars(got[1], want[1])

        # strided layout
        sub = pairs[:2000]
        unp = 304
        buf = np.zeros(2 * unp * len(sub), np.uint8)
        for i, q in enumerate(sub):
            buf[2 * i * unp: 2 * i * unp + q["p_len"]] = ascii[q["p_off"]: q["p_off"] + q["p_len"]]
            buf[(2 * i + 1) * unp: (2 * i + 1) * unp + q["t_len"]] = ascii[q["t_off"]: q["t_off"] + q["t_len"]]
        ctx.reset_stats()
        gs = ctx.align_strided(buf, unp, sub["p_len"].copy(), sub["t_len"].copy())
        assert ctx.stats()["mapped_batches"] == 1
        np.testing.assert_array_equal(gs[0], want[0][:2000])
        assert_same_cigars(gs[1], want[1][:2000])

        # bad descriptors are flagged per pair, not refused
        bad = pairs[:100].copy()
        bad[3]["p_off"] = len(ascii) + 1000
        bad[5]["t_len"] = len(ascii)
        d, cg, st = ctx.align(ascii, bad)
        assert st[3] == wfe.PAIR_OUT_OF_RANGE and st[5] == wfe.PAIR_OUT_OF_RANGE
        ok = np.ones(100, bool)
        ok[[3, 5]] = False
        assert (st[ok] == wfe.PAIR_OK).all()
        np.testing.assert_array_equal(d[ok], want[0][:100][ok])


def test_pinned_strided_layout():
    torch_cuda()
    seqs = []
    ascii, pairs = wfe.generate(3000, 140, p_min=0.05, seed=15)
    unp = 304
    buf = np.zeros(2 * unp * len(pairs), np.uint8)
    for i, q in enumerate(pairs):
        buf[2 * i * unp: 2 * i * unp + q["p_len"]] = ascii[q["p_off"]: q["p_off"] + q["p_len"]]
        buf[(2 * i + 1) * unp: (2 * i + 1) * unp + q["t_len"]] = ascii[q["t_off"]: q["t_off"] + q["t_len"]]
    pl, tl = pairs["p_len"].copy(), pairs["t_len"].copy()
    with wfe.Context(max_seq_len=300, batch_size=1000) as ctx:
        want = ctx.align_strided(buf, unp, pl, tl)
        got = ctx.align_strided(_pinned(buf), unp, _pinned(pl), _pinned(tl))
        assert ctx.stats()["mapped_batches"] == 3
    np.testing.assert_array_equal(got[0], want[0])
    assert_same_cigars(got[1], want[1])
    compare_with_oracle(ascii, pairs, 152, *want)


def _long_tier_pairs():
    """Unrelated random pairs (distance about half the length) and a few
    near-identical long ones."""
    rng = np.random.default_rng(5)
    seqs = []
    def rand(L):
        return np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, L)].tobytes()

    for L in [700, 900, 1200, 1500, 2000, 2600] * 3 + [4300, 4700]:
        seqs.append((rand(L), rand(L + int(rng.integers(-30, 30)))))
    # and a few near-identical long pairs, so tiers 5-6 also see long runs
    for L in [3000, 4900]:
        t = rand(L)
        p = bytearray(t)
        for j in rng.choice(L, 40, replace=False):
            p[j] = b"ACGT"[(b"ACGT".index(p[j]) + 1) % 4]
        seqs.append((bytes(p), t))
    return wfe.pairs_from_list(seqs)


def test_long_tiers_without_distance_limit():
    """The pairs reach the CTA-per-pair tiers: shared-memory wavefront up to
    distance 2047 (tier 5), global-memory wavefront beyond (tier 6)."""
    ascii, pairs = _long_tier_pairs()
    with wfe.Context(max_seq_len=5000, cigar_stride=12000) as ctx:
        ctx.set_policy([5000], [3])  # handed on from the register tiers, through the bound pass
        dist, cg, st = ctx.align(ascii, pairs)
        stats = ctx.stats()
    assert dist.max() > 2047
    assert stats["tier_passed"][4] > 0 and stats["tier_passed"][5] > 0, stats
    assert (st == 0).all()
    compare_with_oracle(ascii, pairs, 12000, dist, cg, st)


def test_long_tiers_in_one_slab_each():
    """wfe_create_with_scratch with bounds below one slab: tiers 5 and 6 each
    align one pair at a time, with the same results."""
    torch_cuda()
    ascii, pairs = _long_tier_pairs()
    with wfe.Context(max_seq_len=5000, cigar_stride=12000) as ctx:
        ctx.set_policy([5000], [3])
        want = ctx.align(ascii, pairs)
    with wfe.Context(max_seq_len=5000, cigar_stride=12000, long_scratch=(1, 1)) as ctx:
        ctx.set_policy([5000], [3])
        got = ctx.align(ascii, pairs)
        stats = ctx.stats()
    assert stats["tier_passed"][4] > 0 and stats["tier_passed"][5] > 0, stats
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[2], want[2])
    assert_same_cigars(got[1], want[1])


def test_distance_classes_and_bounds():
    """Tier 5 first: the bound pass routes the pairs into the distance classes
    (limits 255, 511, 1023 and 2047 for 5,000-base sequences) and straight
    to tier 6 past 2047; short and long distances, near-identical and
    unrelated pairs, unequal lengths.  The same results with the bound pass
    off (one launch of tier 5 over every pair), and the oracle's."""
    torch_cuda()
    rng = np.random.default_rng(77)
    ascii, pairs = wfe.generate(600, 200, 4800, p_min=0.0, p_max=0.3, seed=77)
    seqs = [(ascii[q["p_off"]:q["p_off"] + q["p_len"]].tobytes(), ascii[q["t_off"]:q["t_off"] + q["t_len"]].tobytes())
            for q in pairs]
    a2, p2 = _long_tier_pairs()
    seqs += [(a2[q["p_off"]:q["p_off"] + q["p_len"]].tobytes(), a2[q["t_off"]:q["t_off"] + q["t_len"]].tobytes())
             for q in p2]
    t = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 3000)].tobytes()
    seqs += [(t, t), (t[:1000], t), (t, t[:2200]), (b"", t[:300]), (b"A", b"")]
    ascii, pairs = wfe.pairs_from_list(seqs)
    got = {}
    for bound in (True, False):
        with wfe.Context(max_seq_len=5000, cigar_stride=12000, batch_size=400) as ctx:
            ctx.set_policy([5000], [5], bound=bound)
            got[bound] = ctx.align(ascii, pairs)
            stats = ctx.stats()
        assert stats["tier_passed"][5] > 0, stats
        if bound:
            # the bound pass and more than one class per batch
            assert stats["tier_launches"][5] > 2 * stats["batches"], stats
    dist, cg, st = got[True]
    assert (st == 0).all() and dist.max() > 2047 and (dist < 255).sum() > 50
    np.testing.assert_array_equal(dist, got[False][0])
    np.testing.assert_array_equal(st, got[False][2])
    assert_same_cigars(cg, got[False][1])
    compare_with_oracle(ascii, pairs, 12000, dist, cg, st)


@pytest.mark.parametrize("first_tier", [5, 6])
def test_cta_tiers_first_with_and_without_cap(first_tier):
    """The CTA-per-pair tiers as the first tier of every pair: identical
    pairs (distance 0), empty and one-base sequences, short and long pairs,
    with no cap and with a distance cap that stops some of them."""
    torch_cuda()
    rng = np.random.default_rng(41)
    ascii, pairs = wfe.generate(1500, 50, 2500, p_min=0.0, p_max=0.12, seed=41)
    seqs = [(ascii[q["p_off"]:q["p_off"] + q["p_len"]].tobytes(), ascii[q["t_off"]:q["t_off"] + q["t_len"]].tobytes())
            for q in pairs]
    t = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 700)].tobytes()
    seqs += [(t, t), (b"", b""), (b"", b"ACGT"), (b"ACGT", b""), (b"A", b"C"), (b"A", b"A"), (t[:40], t)]
    ascii, pairs = wfe.pairs_from_list(seqs)
    for cap in (0, 100):
        with wfe.Context(max_seq_len=3000, cigar_stride=4096, max_distance=cap, batch_size=700) as ctx:
            ctx.set_policy([3000], [first_tier])
            dist, cg, st = ctx.align(ascii, pairs)
            assert ctx.stats()["tier_launches"][first_tier] > 0
        if cap:
            assert (st == wfe.PAIR_OVER_MAX_DISTANCE).any() and (st == wfe.PAIR_OK).any()
        else:
            assert (st == wfe.PAIR_OK).all()
        compare_with_oracle(ascii, pairs, 4096, dist, cg, st, max_distance=cap)


def test_length_buckets_same_results():
    """Mixed lengths sorted into length buckets, each with its own first tier
    and launch shapes: every result equals the oracle's and the one-bucket
    path's."""
    torch_cuda()
    ascii, pairs = wfe.generate(6000, 100, 3000, p_min=0.01, p_max=0.15, seed=17)
    with wfe.Context(max_seq_len=3200, cigar_stride=2048, batch_size=2500) as ctx:
        one = ctx.align(ascii, pairs)
        for predict in (False, True):
            # [2, 2, 1, 1, 1]: the host launches tier 2 for short buckets after
            # longer buckets' chains have queued device-side tier-2 launches
            for tiers in ([0, 0, 1, 2, 3], [-1, -1, -1, -1, -1], [0, 1, 2, 3, 5], [5, 5, 5, 5, 5],
                          [2, 2, 1, 1, 1], [1, 2, 1, 2, 1]):
                ctx.set_policy([256, 512, 1024, 2048, 3200], tiers, predict=predict)
                got = ctx.align(ascii, pairs)
                np.testing.assert_array_equal(got[0], one[0])
                np.testing.assert_array_equal(got[2], one[2])
                assert_same_cigars(got[1], one[1])
            assert ctx.policy()[0] == [256, 512, 1024, 2048, 3200]
            assert ctx.policy()[2] == predict
    compare_with_oracle(ascii, pairs, 2048, *one)


def test_length_buckets_with_distance_cap():
    """With max_distance, routing (by bucket and by prediction) never sends
    a pair past the tier where the capped chain ends."""
    torch_cuda()
    ascii, pairs = wfe.generate(4000, 100, 1500, p_min=0.01, p_max=0.15, seed=19)
    with wfe.Context(max_seq_len=1700, cigar_stride=1024, max_distance=63) as ctx:
        for predict in (False, True):
            ctx.set_policy([256, 512, 1700], [0, 0, 0], predict=predict)
            got = ctx.align(ascii, pairs)
            assert (got[2] == wfe.PAIR_OVER_MAX_DISTANCE).any() and (got[2] == wfe.PAIR_OK).any()
            compare_with_oracle(ascii, pairs, 1024, *got, max_distance=63)


def test_autotune_installs_and_caches(tmp_path):
    torch = torch_cuda()
    ascii, pairs = wfe.generate(8000, 100, 3000, p_min=0.01, p_max=0.15, seed=18)
    d_ascii = torch.from_numpy(ascii).cuda()
    d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
    cache = str(tmp_path / "tune.jsonl")
    buckets = [256, 512, 1024, 2048, 3200]
    with wfe.Context(max_seq_len=3200, cigar_stride=2048) as ctx:
        tiers = ctx.autotune(d_ascii, d_pairs, len(pairs), buckets, cache, predict=True)
        assert len(tiers) == 5 and all(0 <= t <= 6 for t in tiers)
        assert ctx.policy() == (buckets, tiers, True)
        assert ctx.stats()["pairs"] == 0  # tuning runs are not counted
        got = ctx.align(ascii, pairs)
    assert open(cache).read().count("first_tier") == 1
    with wfe.Context(max_seq_len=3200, cigar_stride=2048) as ctx2:
        assert ctx2.autotune(d_ascii, d_pairs, len(pairs), buckets, cache, predict=True) == tiers  # from the cache
    assert open(cache).read().count("first_tier") == 1
    with wfe.Context(max_seq_len=3200, cigar_stride=2048) as ctx3:
        ctx3.autotune(d_ascii, d_pairs, len(pairs), buckets, cache)  # other flags: a new entry
        assert ctx3.policy()[2] is False
    assert open(cache).read().count("first_tier") == 2
    compare_with_oracle(ascii, pairs, 2048, *got)


def test_exhaustive_tiny_pairs():
    """Every pair of sequences over ACGT of length 0-4 (341 x 341 pairs), and
    a sample of lengths 5-6: the small cases where sentinels, the first and
    last diagonals and empty sequences meet."""
    torch_cuda()
    import itertools
    seqs = [b""]
    for L in range(1, 5):
        seqs += [bytes(t) for t in itertools.product(b"ACGT", repeat=L)]
    pairs = [(p, t) for p in seqs for t in seqs]
    rng = np.random.default_rng(3)
    for _ in range(20000):
        lp, lt = int(rng.integers(5, 7)), int(rng.integers(0, 7))
        pairs.append((np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, lp)].tobytes(),
                      np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, lt)].tobytes()))
    ascii, desc = wfe.pairs_from_list(pairs)
    with wfe.Context(max_seq_len=8, cigar_stride=16, batch_size=50000) as ctx:
        dist, cg, st = ctx.align(ascii, desc)
    assert (st == wfe.PAIR_OK).all()
    compare_with_oracle(ascii, desc, 16, dist, cg, st)


def test_allocation_failure_is_reported_and_leaves_the_device_usable():
    """Buffers that cannot be allocated give WFE_ERR_OUT_OF_MEMORY: at
    creation (the context's device buffers) or at the first call that stages
    (the staging buffers); nothing is left half-made, in-place calls on such a
    context still work, and the next context works."""
    torch_cuda()
    with pytest.raises(wfe.WfeError) as e:
        # sequences of 50,000 bases: a slab of the global-wavefront tier holds a
        # backtrace store of ~625 MB, and a 1 TB slab budget asks for one per
        # resident CTA, several hundred GB
        wfe.Context(max_seq_len=50_000, batch_size=1000, cigar_stride=4096, long_scratch=(0, 1 << 40))
    assert e.value.code == wfe.ERR_OUT_OF_MEMORY
    ascii, pairs = wfe.generate(2000, 150, p_min=0.05, seed=9)
    # 200M pairs per batch: 45 GB of work lists per stage fit, 120 GB of ASCII staging does not
    with wfe.Context(max_seq_len=300, batch_size=200_000_000, cigar_stride=152) as ctx:
        with pytest.raises(wfe.WfeError) as e:
            ctx.align(ascii, pairs)
        assert e.value.code == wfe.ERR_OUT_OF_MEMORY
        got = ctx.align(_pinned(ascii), _pinned(pairs), out=tuple(
            _pinned(o) for o in (np.zeros(len(pairs), np.int32), np.zeros((len(pairs), 152), np.int8),
                                 np.zeros(len(pairs), np.uint8))))
    compare_with_oracle(ascii, pairs, 152, *got)
    with wfe.Context(max_seq_len=300, cigar_stride=152) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    compare_with_oracle(ascii, pairs, 152, dist, cg, st)

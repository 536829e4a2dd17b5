"""wfe_align_device_noalloc: the entry point for callers that cannot allocate
device memory (a host framework owns every allocation, a real-time loop
forbids it).  It must give exactly what wfe_align_device gives with the same
max_distance, call after call, although every call reuses one fixed device
array for its scratch.  This file is collected last (test_zz_*), so a run that
stops at the first failure has already run every other test."""
import numpy as np
import pytest

import wfe

pytestmark = pytest.mark.gpu


def _cigar_bytes(row):
    nz = np.flatnonzero(row == 0)
    return row[: nz[0] + 1].tobytes() if len(nz) else row.tobytes()


def _both(ascii, pairs, max_len, max_distance, stride, stream):
    import torch

    n = len(pairs)
    d_ascii = torch.from_numpy(ascii).cuda()
    d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()

    # the existing entry point, through a context
    ref_dist = torch.zeros(n, dtype=torch.int32, device="cuda")
    ref_cg = torch.zeros(n * stride, dtype=torch.int8, device="cuda")
    ref_st = torch.zeros(n, dtype=torch.uint8, device="cuda")
    with wfe.Context(max_seq_len=max_len, max_distance=max_distance, cigar_stride=stride) as ctx:
        ctx.align_device(d_ascii, d_pairs, n, max_len, ref_dist, ref_cg, ref_st, stream)
        stream.synchronize()

    # the allocation-free entry point; outputs pre-filled with junk
    dist = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    cg = torch.full((n * stride,), 55, dtype=torch.int8, device="cuda")
    st = torch.full((n,), 99, dtype=torch.uint8, device="cuda")
    wfe.align_device_noalloc(d_ascii, d_pairs, n, max_len, max_distance, dist, cg, stride, st, stream)
    stream.synchronize()

    a_d, b_d = ref_dist.cpu().numpy(), dist.cpu().numpy()
    a_s, b_s = ref_st.cpu().numpy(), st.cpu().numpy()
    np.testing.assert_array_equal(b_d, a_d)
    np.testing.assert_array_equal(b_s, a_s)
    a_c = ref_cg.cpu().numpy().reshape(n, stride)
    b_c = cg.cpu().numpy().reshape(n, stride)
    for i in range(n):
        assert _cigar_bytes(b_c[i]) == _cigar_bytes(a_c[i]), f"pair {i}"
    return b_d, b_s


def test_noalloc_matches_align_device_on_two_calls_in_a_row():
    import torch

    assert torch.cuda.is_available()
    stream = torch.cuda.Stream()
    # call 1: short reads, the reference's search range (distances <= 63)
    a1, p1 = wfe.generate(20000, 150, p_min=0.05, seed=31)
    d1, s1 = _both(a1, p1, 300, 63, 152, stream)
    assert (s1 == wfe.PAIR_OK).all() and d1.max() > 10
    # call 2, right after on the same stream: long, high-error pairs up to the
    # entry point's largest search range; the array still holds call 1's data
    a2, p2 = wfe.generate(3000, 100, 600, p_min=0.0, p_max=0.9, seed=32)
    d2, s2 = _both(a2, p2, 1200, wfe.NOALLOC_MAX_DISTANCE, 1000, stream)
    assert (s2 == wfe.PAIR_OVER_MAX_DISTANCE).any() and (s2 == wfe.PAIR_OK).any()
    assert d2[s2 == wfe.PAIR_OK].max() > 143


def test_noalloc_first_tier_alone_and_tier_3_alone():
    """A search range within the 4-lane tier's (max_distance 21): that tier
    alone, handing nothing on.  Sequences and CIGAR slots too wide for its
    shared memory (max_seq_len 3,000, 6,004-byte slots): tier 3 alone over
    every pair.  Both give what wfe_align_device gives."""
    import torch

    stream = torch.cuda.Stream()
    a1, p1 = wfe.generate(20000, 150, p_min=0.05, p_max=0.2, seed=33)
    d1, s1 = _both(a1, p1, 300, 21, 152, stream)
    assert (s1 == wfe.PAIR_OVER_MAX_DISTANCE).any() and (s1 == wfe.PAIR_OK).any()
    a2, p2 = wfe.generate(1500, 1000, 1400, p_min=0.02, p_max=0.2, seed=34)
    d2, s2 = _both(a2, p2, 3000, wfe.NOALLOC_MAX_DISTANCE, 6004, stream)
    assert (s2 == wfe.PAIR_OK).any() and d2[s2 == wfe.PAIR_OK].max() > 79


def test_noalloc_rejects_search_ranges_beyond_its_scratch():
    import torch

    a, p = wfe.generate(8, 150, p_min=0.05, seed=1)
    d_ascii = torch.from_numpy(a).cuda()
    d_pairs = torch.from_numpy(p.view(np.uint8)).cuda()
    out = torch.zeros(8, dtype=torch.int32, device="cuda")
    cg = torch.zeros(8 * 152, dtype=torch.int8, device="cuda")
    for bad in (0, -1, wfe.NOALLOC_MAX_DISTANCE + 1):
        with pytest.raises(wfe.WfeError) as e:
            wfe.align_device_noalloc(d_ascii, d_pairs, 8, 300, bad, out, cg, 152, None)
        assert e.value.code == wfe.ERR_INVALID_ARGUMENT


def test_noalloc_matches_the_oracle_and_allocates_nothing():
    """Direct parity with the CPU restatement of the reference, one pair over
    max_len (WFE_PAIR_TOO_LONG, as wfe_align_device reports it), and no
    change in the device's free memory across a call."""
    import torch

    import oracle

    stride, max_len, cap = 152, 150, 63
    a, p = wfe.generate(6000, 140, 160, p_min=0.02, p_max=0.12, seed=33)
    n = len(p)
    d_ascii = torch.from_numpy(a).cuda()
    d_pairs = torch.from_numpy(p.view(np.uint8)).cuda()
    dist = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    cg = torch.full((n * stride,), 55, dtype=torch.int8, device="cuda")
    st = torch.full((n,), 99, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    wfe.align_device_noalloc(d_ascii, d_pairs, n, max_len, cap, dist, cg, stride, st, stream)  # set-up call
    stream.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    wfe.align_device_noalloc(d_ascii, d_pairs, n, max_len, cap, dist, cg, stride, st, stream)
    stream.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes across a call"

    too_long = np.maximum(p["p_len"], p["t_len"]) > max_len
    assert too_long.any() and (~too_long).any()
    b_d, b_s = dist.cpu().numpy(), st.cpu().numpy()
    b_c = cg.cpu().numpy().reshape(n, stride)
    assert (b_s[too_long] == wfe.PAIR_TOO_LONG).all()
    assert (b_d[too_long] == -1).all()
    od, ocg, ost, _ = oracle.align_batch(a, p["p_off"], p["p_len"], p["t_off"], p["t_len"], stride, max_distance=cap)
    ok = ~too_long
    np.testing.assert_array_equal(b_d[ok], od[ok])
    np.testing.assert_array_equal(b_s[ok], ost[ok])
    assert (ost[ok] == wfe.PAIR_OVER_MAX_DISTANCE).any() or b_d[ok].max() > 10
    for i in np.flatnonzero(ok & (ost == wfe.PAIR_OK)):
        assert _cigar_bytes(b_c[i]) == _cigar_bytes(ocg[i]), f"pair {i}"

    # the same pairs through wfe_align_device agree on the too-long ones too
    ref_d = torch.zeros(n, dtype=torch.int32, device="cuda")
    ref_c = torch.zeros(n * stride, dtype=torch.int8, device="cuda")
    ref_s = torch.zeros(n, dtype=torch.uint8, device="cuda")
    with wfe.Context(max_seq_len=max_len, max_distance=cap, cigar_stride=stride) as ctx:
        ctx.align_device(d_ascii, d_pairs, n, max_len, ref_d, ref_c, ref_s, stream)
        stream.synchronize()
    np.testing.assert_array_equal(b_d, ref_d.cpu().numpy())
    np.testing.assert_array_equal(b_s, ref_s.cpu().numpy())


def test_noalloc_without_status_or_cigars():
    """d_status NULL and cigar_stride 0: distances only, still the oracle's."""
    import torch

    import oracle

    a, p = wfe.generate(3000, 150, p_min=0.05, seed=34)
    n = len(p)
    d_ascii = torch.from_numpy(a).cuda()
    d_pairs = torch.from_numpy(p.view(np.uint8)).cuda()
    dist = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    wfe.align_device_noalloc(d_ascii, d_pairs, n, 300, 63, dist, None, 0, None, None)
    torch.cuda.synchronize()
    od, _, _, _ = oracle.align_batch(a, p["p_off"], p["p_len"], p["t_off"], p["t_len"], 152, max_distance=63)
    np.testing.assert_array_equal(dist.cpu().numpy(), od)

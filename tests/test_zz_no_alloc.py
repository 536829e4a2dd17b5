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

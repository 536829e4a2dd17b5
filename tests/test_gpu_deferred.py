"""Tiers 2-6's scratch is allocated when a call first needs it: until then a
host call's chains stop at tier 1 and defer the pairs past distance 79, and
the call aligns them again once the scratch exists.  Every entry point must
give the oracle's results whether or not that happens, and a short-read
context must hold little device memory until it does."""
import numpy as np
import pytest

import wfe
from test_gpu_parity import _pinned, assert_same_cigars, compare_with_oracle, torch_cuda

pytestmark = pytest.mark.gpu


def high_error_pairs(n, seed):
    """Lengths 100-600 at edit probabilities up to 0.9: distances 0 to ~330,
    so that a chain from tier 0 reaches tiers 2-4 (max_seq_len 1,200 keeps
    tier 0 the first tier)."""
    return wfe.generate(n, 100, 600, p_min=0.0, p_max=0.9, seed=seed)


def strided(ascii, pairs, slot):
    buf = np.zeros(2 * slot * len(pairs), np.uint8)
    for i, q in enumerate(pairs):
        buf[2 * i * slot: 2 * i * slot + q["p_len"]] = ascii[q["p_off"]: q["p_off"] + q["p_len"]]
        buf[(2 * i + 1) * slot: (2 * i + 1) * slot + q["t_len"]] = ascii[q["t_off"]: q["t_off"] + q["t_len"]]
    return buf


@pytest.mark.parametrize("mode", ["pageable", "pageable_in_place", "pinned", "strided"])
def test_first_host_call_defers_and_realigns(mode):
    """The first call on a fresh context defers the 1,336 of 3,000 pairs past
    distance 79 (fewer than batch_size; two batches, so the indices of the
    second carry its offset) and aligns them again; a second call, with the
    scratch in place, runs whole chains.  Both match the oracle."""
    torch_cuda()
    ascii, pairs = high_error_pairs(3000, 51)
    flags = wfe.FLAG_PAGEABLE_IN_PLACE if mode == "pageable_in_place" else 0
    with wfe.Context(max_seq_len=1200, batch_size=2000, cigar_stride=2000, flags=flags) as ctx:
        slot = (int(max(pairs["p_len"].max(), pairs["t_len"].max())) + 15) // 16 * 16

        def run():
            if mode == "strided":
                return ctx.align_strided(strided(ascii, pairs, slot), slot, pairs["p_len"].copy(),
                                         pairs["t_len"].copy())
            if mode == "pinned":
                return ctx.align(_pinned(ascii), _pinned(pairs))
            return ctx.align(ascii, pairs)
        assert ctx.stats()["deep_scratch_bytes"] == 0
        first = run()
        stats = ctx.stats()
        second = run()
        after = ctx.stats()
    assert first[0].max() > 143 and stats["tier_passed"][1] > 0, stats
    assert stats["deferred_pairs"] == int((first[0] > 79).sum()) and stats["deep_scratch_bytes"] > 0, stats
    assert 0 < stats["deferred_pairs"] < 2000, stats
    assert after["deferred_pairs"] == stats["deferred_pairs"], after  # the second call deferred nothing
    for r in (first, second):
        compare_with_oracle(ascii, pairs, 2000, *r)


def test_more_deferred_pairs_than_the_list_holds():
    """More pairs pass distance 79 than batch_size: the call runs again
    whole, with the same results as a context whose scratch exists from the
    start (a first tier past 1 allocates it at once)."""
    torch_cuda()
    ascii, pairs = high_error_pairs(2000, 52)
    with wfe.Context(max_seq_len=1200, batch_size=64, cigar_stride=2000) as ctx:
        got = ctx.align(ascii, pairs)
        assert ctx.stats()["deferred_pairs"] > 64
    with wfe.Context(max_seq_len=1200, batch_size=64, cigar_stride=2000) as ctx:
        ctx.set_policy([1200], [2])
        want = ctx.align(ascii, pairs)
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[2], want[2])
    assert_same_cigars(got[1], want[1])  # up to each terminator: tiers pad the last word differently
    compare_with_oracle(ascii, pairs, 2000, *got)


def test_short_read_context_holds_little_device_memory():
    """A context for 100k-pair batches of 150-base reads (max_seq_len 300, as
    the command line makes it; results written in place, so no staging
    buffers either) holds its work lists only; the first device call adds
    tiers 2-6's scratch, and the results do not change."""
    torch = torch_cuda()
    ascii, pairs = wfe.generate(20000, 150, p_min=0.05, seed=53)
    n, stride = len(pairs), 152
    with wfe.Context(max_seq_len=300, batch_size=1000, cigar_stride=stride) as warm:
        warm.align(ascii, pairs[:100])  # the library's kernels loaded before measuring
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    with wfe.Context(max_seq_len=300, batch_size=100000, cigar_stride=stride,
                     flags=wfe.FLAG_PAGEABLE_IN_PLACE) as ctx:
        free1, _ = torch.cuda.mem_get_info()
        host = ctx.align(ascii, pairs)
        st_host = ctx.stats()
        free2, _ = torch.cuda.mem_get_info()
        d_ascii = torch.from_numpy(ascii).cuda()
        d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
        d_dist = torch.zeros(n, dtype=torch.int32, device="cuda")
        d_cg = torch.zeros(n * stride, dtype=torch.int8, device="cuda")
        d_st = torch.zeros(n, dtype=torch.uint8, device="cuda")
        ctx.align_device(d_ascii, d_pairs, n, 300, d_dist, d_cg, d_st)
        torch.cuda.synchronize()
        free3, _ = torch.cuda.mem_get_info()
        st_dev = ctx.stats()
        dev = (d_dist.cpu().numpy(), d_cg.view(n, stride).cpu().numpy(), d_st.cpu().numpy())
    mib = 1 << 20
    assert st_host["deep_scratch_bytes"] == 0 and st_dev["deep_scratch_bytes"] > 64 * mib, (st_host, st_dev)
    assert free0 - free1 < 48 * mib, (free0 - free1) / mib
    assert free1 - free2 < 8 * mib, (free1 - free2) / mib    # no pair passed distance 79
    assert free2 - free3 > 64 * mib, (free2 - free3) / mib   # the device call's scratch
    for r in (host, dev):
        compare_with_oracle(ascii, pairs, stride, *r)


def test_device_call_on_a_fresh_context_runs_whole_chains():
    """A device call returns before its chains end, so it allocates the
    scratch first and runs every tier: the results match the oracle, and a
    host call after it defers nothing."""
    torch = torch_cuda()
    ascii, pairs = high_error_pairs(1500, 54)
    n, stride = len(pairs), 2000
    d_ascii = torch.from_numpy(ascii).cuda()
    d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
    d_dist = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_cg = torch.zeros(n * stride, dtype=torch.int8, device="cuda")
    d_st = torch.zeros(n, dtype=torch.uint8, device="cuda")
    with wfe.Context(max_seq_len=1200, batch_size=500, cigar_stride=stride) as ctx:
        ctx.align_device(d_ascii, d_pairs, n, 1200, d_dist, d_cg, d_st)
        torch.cuda.synchronize()
        stats = ctx.stats()
        host = ctx.align(ascii, pairs)
    assert stats["tier_passed"][2] > 0, stats
    dev = (d_dist.cpu().numpy(), d_cg.view(n, stride).cpu().numpy(), d_st.cpu().numpy())
    for r in (dev, host):
        compare_with_oracle(ascii, pairs, stride, *r)


def test_deferred_pairs_under_a_distance_cap():
    """A cap between tier 1's reach and the deep tiers' (150): the chain is
    cut at tier 1 all the same, the pairs past 79 are deferred, and once
    realigned those past 150 get WFE_PAIR_OVER_MAX_DISTANCE, as the oracle
    with the same cap says."""
    torch_cuda()
    ascii, pairs = high_error_pairs(2500, 55)
    with wfe.Context(max_seq_len=1200, batch_size=3000, max_distance=150, cigar_stride=2000) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
        stats = ctx.stats()
    assert stats["deferred_pairs"] > 0 and (st == wfe.PAIR_OVER_MAX_DISTANCE).any(), stats
    compare_with_oracle(ascii, pairs, 2000, dist, cg, st, max_distance=150)

"""The request server (wfe_server_*, wfe_submit, wfe_poll): continuous
batching on the GPU.  Every request's results must be the same whether it
is aligned alone (one wfe_align call) or in the mix of concurrently
submitted requests, split over batches or not; integer work, so bit-exact."""
import threading
import time

import numpy as np
import pytest

import wfe
from test_gpu_parity import assert_same_cigars, compare_with_oracle, torch_cuda

pytestmark = pytest.mark.gpu

GEN_LEN = 2000           # longest generated text
MAX_LEN = 2300           # with room for the pattern's insertions


def request_sizes(rng, count, largest):
    """Log-uniform request sizes in [1, largest]."""
    return np.floor(np.exp(rng.uniform(0, np.log(largest + 1), count))).astype(int).clip(1, largest)


@pytest.fixture(scope="module")
def pool():
    torch_cuda()
    ascii, pairs = wfe.generate(30000, 100, GEN_LEN, p_min=0.01, p_max=0.10, seed=31)
    assert max(pairs["p_len"].max(), pairs["t_len"].max()) <= MAX_LEN
    return ascii, pairs


def alone(ascii, pairs):
    with wfe.Context(max_seq_len=MAX_LEN, batch_size=20000) as ctx:
        return ctx.align(ascii, pairs)


def check_same(req, want):
    np.testing.assert_array_equal(req.dist, want[0])
    np.testing.assert_array_equal(req.status, want[2])
    assert_same_cigars(req.cigar, want[1])


def test_mix_equals_alone(pool):
    """Requests of 1-512 pairs from four submitting threads; batches of at
    most 300 pairs (so every larger request is split) and a small arena,
    with several batches in flight."""
    ascii, pairs = pool
    rng = np.random.default_rng(5)
    sizes = request_sizes(rng, 160, 512)
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]]) % (len(pairs) - 512)
    reqs = [pairs[s:s + k] for s, k in zip(starts, sizes)]
    want = [alone(ascii, r) for r in reqs[:40]]
    full = alone(ascii, pairs)  # every request's results are slices of this one

    with wfe.Server(max_seq_len=MAX_LEN, lanes=4, batch_pairs=300, memory_bytes=8 << 20) as srv:
        submitted = [None] * len(reqs)

        def submit(part):
            for i in part:
                submitted[i] = srv.submit(ascii, reqs[i])
                time.sleep(float(rng.uniform(0, 2e-4)))

        threads = [threading.Thread(target=submit, args=(range(t, len(reqs), 4),)) for t in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        for r in submitted:
            assert srv.poll(r, timeout_us=120_000_000)
        st = srv.stats()
    for i, r in enumerate(submitted):
        s, k = starts[i], sizes[i]
        check_same(r, (full[0][s:s + k], full[1][s:s + k], full[2][s:s + k]))
        if i < len(want):
            check_same(r, want[i])
        assert r.info["pairs"] == k and r.info["done_ns"] >= r.info["start_ns"] >= r.info["submit_ns"]
    assert st["requests"] == len(reqs) and st["pairs"] == int(sizes.sum())
    assert st["batches"] > 1 and st["split_requests"] >= int((sizes > 300).sum())
    assert st["max_in_flight"] >= 2, st
    assert st["peak_memory"] <= 8 << 20


def test_results_match_oracle(pool):
    ascii, pairs = pool
    sub = pairs[:3000]
    with wfe.Server(max_seq_len=MAX_LEN, lanes=2, bucket_max_len=[256, 1024, MAX_LEN]) as srv:
        reqs = [srv.submit(ascii, sub[i:i + 300]) for i in range(0, len(sub), 300)]
        for r in reqs:
            assert srv.poll(r)
    dist = np.concatenate([r.dist for r in reqs])
    cg = np.concatenate([r.cigar for r in reqs])
    st = np.concatenate([r.status for r in reqs])
    compare_with_oracle(ascii, sub, wfe.reference_cigar_stride(MAX_LEN), dist, cg, st)


def test_scattered_request_is_gathered(pool):
    """Pairs spread over the whole buffer (span far above their bytes) are
    gathered pair by pair; pinned inputs and outputs work the same."""
    ascii, pairs = pool
    sub = pairs[::97][:250]
    want = alone(ascii, sub)
    torch = torch_cuda()
    h_ascii = torch.empty(len(ascii), dtype=torch.uint8, pin_memory=True).numpy()
    h_ascii[:] = ascii
    with wfe.Server(max_seq_len=MAX_LEN, lanes=2, memory_bytes=32 << 20) as srv:
        r1 = srv.submit(ascii, sub)
        r2 = srv.submit(h_ascii, sub)
        assert srv.poll(r1) and srv.poll(r2)
    check_same(r1, want)
    check_same(r2, want)


def test_tickets_and_errors(pool):
    ascii, pairs = pool
    with wfe.Server(max_seq_len=MAX_LEN, lanes=1) as srv:
        empty = srv.submit(ascii, pairs[:0])
        assert srv.poll(empty, timeout_us=0)
        assert empty.info["pairs"] == 0
        assert srv.poll_ticket(empty.ticket) == wfe.ERR_NOT_FOUND  # retired
        assert srv.poll_ticket(123456789) == wfe.ERR_NOT_FOUND
        bad = pairs[:4].copy()
        bad["t_off"][2] = len(ascii)  # outside the buffer
        with pytest.raises(wfe.WfeError) as e:
            srv.submit(ascii, bad)
        assert e.value.code == wfe.ERR_INVALID_ARGUMENT
        long_seq, _ = wfe.pairs_from_list([(b"A" * (MAX_LEN + 1), b"A")])
        with pytest.raises(wfe.WfeError) as e:
            srv.submit(long_seq, wfe.pairs_from_list([(b"A" * (MAX_LEN + 1), b"A")])[1])
        assert e.value.code == wfe.ERR_SEQ_TOO_LONG
        # a request waited on with a short limit, then to the end
        r = srv.submit(ascii, pairs[:5000])
        finished = srv.poll(r, timeout_us=1)
        if not finished:
            assert srv.poll(r)
        check_same(r, alone(ascii, pairs[:5000]))
        assert srv.stats()["requests"] == 2


def test_memory_admission_limits_batches(pool):
    """With an arena that holds a few dozen long pairs, every batch stays
    inside it and a large request is spread over many batches."""
    ascii, pairs = pool
    sub = pairs[:1200]
    want = alone(ascii, sub)
    arena = 256 << 10
    with wfe.Server(max_seq_len=MAX_LEN, lanes=3, memory_bytes=arena) as srv:
        r = srv.submit(ascii, sub)
        assert srv.poll(r)
        st = srv.stats()
    check_same(r, want)
    assert r.info["batches"] > 5 and st["peak_memory"] <= arena
    with pytest.raises(wfe.WfeError) as e:
        wfe.Server(max_seq_len=MAX_LEN, memory_bytes=1024)  # not one pair fits
    assert e.value.code == wfe.ERR_INVALID_ARGUMENT


def test_admission_refused_when_the_arena_does_not_fit(pool):
    """A server whose arena is larger than the free device memory is refused
    (WFE_ERR_BUSY) and the device stays usable."""
    ascii, pairs = pool
    with pytest.raises(wfe.WfeError) as e:
        wfe.Server(max_seq_len=MAX_LEN, memory_bytes=1 << 50)
    assert e.value.code == wfe.ERR_BUSY
    with wfe.Server(max_seq_len=MAX_LEN, lanes=1) as srv:
        r = srv.submit(ascii, pairs[:200])
        assert srv.poll(r)
    check_same(r, alone(ascii, pairs[:200]))

"""The CPU oracle pinned against the reference (no GPU).

The restatement in oracle/wfe_oracle.c must reproduce, on every golden vector
(produced by the reference's own kernels, tests/golden/make_golden.py): the
distance, the 2-bit operation chain of the 128-bit history, the encoded CIGAR
bytes of the whole slot, the packed words of compact_sequences, the -p
printer's text and check_cigar's verdict.  Where the reference library is
built (oracle/_ref), fresh random cases are compared with it live as well.
"""
import itertools
import os
import random

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_vectors.npz")


@pytest.fixture(scope="module")
def golden():
    z = np.load(GOLDEN)
    a = z["ascii"].tobytes()
    pairs = [(a[o[0]:o[0] + o[1]], a[o[2]:o[2] + o[3]]) for o in z["offsets"]]
    return z, pairs


def test_golden_distance_ops_cigar(golden):
    z, pairs = golden
    stride = z["cigars"].shape[1]
    n_cap = 0
    for i, (p, t) in enumerate(pairs):
        st, d, ops, _ = O.align(p, t, max_distance=63)
        if z["dist"][i] >= 64:
            assert st == O.PAIR_OVER_MAX and d == 64, i
            n_cap += 1
            continue
        assert st == O.PAIR_OK and d == z["dist"][i], i
        assert ops == O.ops_from_words(z["words"][i], d), i
        st2, cg, _ = O.cigar(p, t, d, ops, stride)
        assert st2 == O.PAIR_OK
        np.testing.assert_array_equal(cg, z["cigars"][i], err_msg=f"pair {i}")
    assert n_cap == int((z["dist"] >= 64).sum()) > 0


def test_golden_packed_words(golden):
    z, pairs = golden
    nwords = z["packed"].shape[2] // 4
    for i, (p, t) in enumerate(pairs):
        for j, s in enumerate((p, t)):
            ref_words = z["packed"][i, j].view("<u4")
            np.testing.assert_array_equal(O.pack(s, nwords), ref_words, err_msg=f"pair {i} seq {j}")


def test_golden_printer_and_check(golden):
    z, pairs = golden
    for i, (p, t) in enumerate(pairs):
        if z["dist"][i] >= 64:
            continue
        assert O.format_cigar(z["cigars"][i], compat=True) == str(z["compat"][i]), i
        ok, score = O.check_cigar(p, t, z["cigars"][i])
        assert ok == bool(z["ref_check"][i]), i
        if ok:
            assert score == z["dist"][i]


def test_alias_pairs_fail_byte_check(golden):
    """The reference aligns on 2-bit codes (N == G) but checks raw bytes, so
    a CIGAR that matches N against G fails its own check; the oracle agrees."""
    z, pairs = golden
    names = list(z["case_names"])
    alias = np.flatnonzero(z["case_ids"] == names.index("alias"))
    assert (~z["ref_check"][alias]).any()


def test_readme_pairs(golden):
    z, pairs = golden
    names = list(z["case_names"])
    idx = np.flatnonzero(z["case_ids"] == names.index("readme"))
    assert len(idx) == 3
    for i in idx:
        p, t = pairs[i]
        assert O.levenshtein(p, t) == z["dist"][i]


def _mutate(rng, text, p):
    out = []
    for c in text:
        if rng.random() < p:
            k = rng.randrange(3)
            if k == 0:
                out.append(rng.choice([b for b in "ACGT" if b != c]))
            elif k == 1:
                out += [rng.choice("ACGT"), c]
        else:
            out.append(c)
    return "".join(out).encode()


def test_distance_is_levenshtein_without_cap():
    """The unclamped recurrence terminates exactly at the edit distance, also
    far above the reference's 63 cap."""
    rng = random.Random(5)
    for _ in range(300):
        L = rng.choice([1, 7, 50, 150, 400, 1000])
        p = rng.choice([0.0, 0.05, 0.1, 0.3, 0.6])
        t = "".join(rng.choice("ACGT") for _ in range(L))
        pat = _mutate(rng, t, p)
        st, d, ops, _ = O.align(pat, t.encode(), 0)
        assert st == O.PAIR_OK
        assert d == O.levenshtein(pat, t.encode())
        st2, cg, ln = O.cigar(pat, t.encode(), d, ops, 4 * L + 16)
        ok, score = O.check_cigar(pat, t.encode(), cg)
        assert ok and score == d


def test_exhaustive_small_alphabet():
    """Every pair of sequences over {A, C, G} up to length 4."""
    seqs = [b""] + [bytes(s) for n in range(1, 5) for s in itertools.product(b"ACG", repeat=n)]
    rng = random.Random(3)
    sample = rng.sample([(a, b) for a in seqs for b in seqs], 6000)
    for p, t in sample:
        st, d, ops, _ = O.align(p, t, 0)
        assert d == O.levenshtein(p, t)
        _, cg, _ = O.cigar(p, t, d, ops, 32)
        ok, score = O.check_cigar(p, t, cg)
        assert ok and score == d


def test_cigar_truncation():
    p, t = b"ACGTACGTAC" * 3, b"TGCATGCATG" * 3
    st, d, ops, _ = O.align(p, t, 0)
    st2, cg, full = O.cigar(p, t, d, ops, 8)
    assert st2 == O.PAIR_CIGAR_TRUNCATED and full > 8
    assert (cg != 0).all()


def test_over_max_distance():
    p, t = b"A" * 50, b"C" * 50
    st, d, ops, _ = O.align(p, t, 10)
    assert st == O.PAIR_OVER_MAX and d == 11


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
def test_live_against_reference_kernels():
    rng = random.Random(99)
    pairs = []
    for _ in range(1500):
        L = rng.choice([0, 1, 3, 15, 16, 17, 31, 32, 33, 64, 100, 150])
        pr = rng.choice([0.0, 0.02, 0.05, 0.1, 0.2, 0.4])
        t = "".join(rng.choice("ACGT") for _ in range(L))
        pairs.append((_mutate(rng, t, pr), t.encode()))
    dist, words, cg = O.ref_align(pairs, 150)
    for i, (p, t) in enumerate(pairs):
        if not 0 <= dist[i] < 64:
            continue
        st, d, ops, _ = O.align(p, t, 63)
        assert d == dist[i] and ops == O.ops_from_words(words[i], d)
        _, mine, _ = O.cigar(p, t, d, ops, cg.shape[1])
        np.testing.assert_array_equal(mine, cg[i])


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built here")
def test_live_packing_roundtrip():
    rng = random.Random(7)
    for L in [1, 4, 15, 16, 17, 40, 150, 299]:
        s = "".join(rng.choice("ACGT") for _ in range(L)).encode()
        words = O.pack(s)
        assert O.ref_ascii_sequence(words, L) == s


def test_batch_matches_single():
    rng = random.Random(11)
    seqs = []
    for _ in range(200):
        t = "".join(rng.choice("ACGT") for _ in range(rng.randrange(0, 300)))
        seqs.append((_mutate(rng, t, 0.08), t.encode()))
    buf = b"".join(p + t for p, t in seqs)
    offs, pos = [], 0
    for p, t in seqs:
        offs.append((pos, len(p), pos + len(p), len(t)))
        pos += len(p) + len(t)
    offs = np.array(offs, dtype=np.int64)
    ascii = np.frombuffer(buf + b"\0" * 16, dtype=np.uint8)
    dist, cg, st, _ = O.align_batch(ascii, offs[:, 0], offs[:, 1], offs[:, 2], offs[:, 3], 320, nthreads=4)
    for i, (p, t) in enumerate(seqs):
        s1, d, ops, _ = O.align(p, t, 0)
        assert dist[i] == d
        _, c1, _ = O.cigar(p, t, d, ops, 320)
        np.testing.assert_array_equal(cg[i], c1)

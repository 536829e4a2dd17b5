"""The distance bound and the target's cone of the CTA-per-pair tiers,
restated on the CPU and checked against the oracle (no GPU).

Tiers 5 and 6 (long_kernel) compute, at score step d, only the cells of
[-d, d] with |k - kt| <= dub - d, where dub is an upper bound on the pair's
distance computed by bound_kernel: the tiers' recurrence restricted to a band
of 32 diagonals that follows the cell that has consumed the most bases.  This
file restates both, in the kernels' terms, and checks on seeded pairs that
  - the band's bound is never below the oracle's distance (and equals it on
    almost every pair);
  - the cut recurrence reads only cells it computed at the previous step or
    the -1 sentinels just beyond [-(d-1), d-1], and reaches the oracle's
    distance with the oracle's operation chain, for dub = the bound and for
    dub = the tier's limit;
  - with dub one below the distance there is no hit by dub, the condition on
    which long_kernel aligns the pair again without the bound.
The recurrence is the reference's (src/kernels.cu:111-180, 249-268).
"""
import random

import oracle as O

BAND = 32
HALF = 15


def extend(p: bytes, t: bytes, k: int, off: int) -> int:
    v, h = off - k, off
    if v < 0 or h < 0:
        return off
    while v < len(p) and h < len(t) and p[v] == t[h]:
        v += 1
        h += 1
    return h


def piggyback(up: int, self_: int, dn: int) -> int:
    """Best candidate with its operation in the low two bits: DEL > SUB > INS."""
    return max(up * 4 + 3, self_ * 4 + 6, dn * 4 + 5)


def band_bound(p: bytes, t: bytes) -> int:
    """bound_kernel's bound for one pair (-1: none)."""
    P, T = len(p), len(t)
    kt = T - P
    b = -HALF
    O_ = [-1] * BAND
    O_[HALF] = extend(p, t, 0, 0)
    if kt == 0 and O_[HALF] == T:
        return 0
    delta_next = 0
    for d in range(1, max(P, T) + 2):
        # the leader after step d-1 moves the band of step d+1
        delta = delta_next
        prog = [min(O_[lane], T) + min(O_[lane] - (b + lane), P) if O_[lane] >= 0 else None for lane in range(BAND)]
        best = max(x for x in prog if x is not None)
        lead = prog.index(best) - delta
        delta_next = (lead > HALF + 1) - (lead < HALF)
        b += delta
        N = [-1] * BAND
        hit = False
        for lane in range(BAND):
            k, s = b + lane, lane + delta
            up = O_[s + 1] if 0 <= s + 1 < BAND else -1
            se = O_[s] if 0 <= s < BAND else -1
            dn = O_[s - 1] if 0 <= s - 1 < BAND else -1
            if -d <= k <= d:
                off = piggyback(up, se, dn) >> 2
                if off >= k:
                    N[lane] = extend(p, t, k, off)
            hit |= k == kt and N[lane] == T
        O_ = N
        if hit:
            return d
    return -1


def cone_align(p: bytes, t: bytes, dub: int):
    """long_kernel's cut recurrence up to step dub: (distance, ops, cells)
    or (None, None, cells) with no hit by dub.  A read of a cell that the
    previous step did not compute raises KeyError."""
    P, T = len(p), len(t)
    kt = T - P
    cur = {0: extend(p, t, 0, 0), 1: -1, -1: -1, 2: -1, -2: -1}
    if kt == 0 and cur[0] == T:
        return 0, [], 0
    rows, cells = [], 0
    for d in range(1, dub + 1):
        klo, khi = max(-d, kt - (dub - d)), min(d, kt + (dub - d))
        nxt, row = {}, {}
        for k in range(klo, khi + 1):
            m = piggyback(cur[k + 1], cur[k], cur[k - 1])
            row[k] = m & 3
            nxt[k] = extend(p, t, k, m >> 2)
        cells += max(0, khi - klo + 1)
        for j in (d + 1, -d - 1, d + 2, -d - 2):
            nxt[j] = -1
        rows.append(row)
        cur = nxt
        if -d <= kt <= d and cur[kt] == T:
            ops, k = [], kt
            for s in range(d, 0, -1):
                op = rows[s - 1][k]
                ops.append(op)
                k += op - 2
            assert k == 0
            return d, ops[::-1], cells
    return None, None, cells


def _pairs(n: int, seed: int):
    rng = random.Random(seed)
    out = [(b"", b""), (b"", b"ACGT"), (b"ACGTA", b""), (b"A", b"C"), (b"ACGT" * 20, b"ACGT" * 20)]
    while len(out) < n:
        L = rng.randint(1, 220)
        pe = rng.choice([0.0, 0.02, 0.05, 0.1, 0.2, 0.3])
        t = bytes(rng.choice(b"ACGT") for _ in range(L))
        p = bytearray()
        for c in t:
            r = rng.random()
            if r < pe / 3:
                continue                                  # deletion
            if r < 2 * pe / 3:
                p += bytes([rng.choice(b"ACGT")])         # insertion before c
            elif r < pe:
                c = b"ACGT"[(b"ACGT".index(c) + rng.randint(1, 3)) % 4]  # substitution
            p.append(c)
        if rng.random() < 0.15:
            p += bytes(rng.choice(b"ACGT") for _ in range(rng.randint(1, 40)))  # unequal lengths
        out.append((bytes(p), t))
    return out


def test_bound_and_cone_match_the_oracle():
    pairs = _pairs(160, 7)
    exact = cut = full = 0
    for p, t in pairs:
        st, D, ops, _ = O.align(p, t)
        assert st == O.PAIR_OK
        bnd = band_bound(p, t)
        assert bnd >= D, (p, t, bnd, D)
        exact += bnd == D
        dub = max(bnd, abs(len(t) - len(p)))
        d1, ops1, c1 = cone_align(p, t, dub)
        assert (d1, ops1) == (D, ops)
        dstop = max(len(p), len(t)) + 1
        d2, ops2, _ = cone_align(p, t, dstop)
        assert (d2, ops2) == (D, ops)
        if D >= 1:
            d3, _, _ = cone_align(p, t, D - 1)
            assert d3 is None
        if D >= 20:
            cut += c1
            full += sum(2 * d + 1 for d in range(1, D + 1))
    assert exact >= 0.95 * len(pairs)
    assert full > 0 and cut <= 0.6 * full

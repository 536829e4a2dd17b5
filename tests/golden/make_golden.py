"""Generate the golden vectors in this directory from the reference itself.

Runs the reference's own kernels (src/kernels.cu of quim0/eWFA-GPU, compiled
for the CPU into oracle/_ref by oracle/Makefile) and its host helpers
(src/wavefront.cuh) on a fixed set of pairs and stores inputs and outputs in
ref_vectors.npz.  Needs the reference sources (at $WFE_REFERENCE_DIR, else
/root/reference), so it runs only where they are mounted; the fixture it writes
is committed and is all the tests read.

    python tests/golden/make_golden.py

Cases (all with the reference's -l 150, i.e. 304-byte ASCII slots, 80-byte
packed slots and 152-byte CIGAR slots):
  readme   the three example pairs of the reference's README.md
  cfg1     200 pairs, length 150, edit probability 0.02 (seed 11)
  cfg2     200 pairs, length 150, edit probability 0.05 (seed 12)
  err20    100 pairs, length 150, edit probability 0.2-0.45 (seed 13), distances
           close to the reference's 63 cap (pairs at 64 keep the reference's
           over-cap output)
  short    300 pairs, lengths 0..40, probabilities 0..0.5 (seed 14)
  alias    60 pairs with N and lower-case bases (seed 15)
  overcap  20 pairs, length 150, edit probability 0.7-0.9 (seed 16): most are
           above the reference's cap and keep its distance 64
"""
from __future__ import annotations

import os
import random
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "ewfa-gpu_gb300"))

import oracle  # noqa: E402

SEQ_LEN = 150
OUT = os.path.join(HERE, "ref_vectors.npz")


def readme_pairs():
    path = os.path.join(oracle.REF_SRC, "README.md")
    lines = [ln.strip() for ln in open(path) if ln.startswith((">", "<"))]
    pats = [ln[1:] for ln in lines if ln.startswith(">")]
    txts = [ln[1:] for ln in lines if ln.startswith("<")]
    return [(p.encode(), t.encode()) for p, t in zip(pats, txts)]


def mutate(rng, text, p, alphabet="ACGT"):
    out = []
    for c in text:
        if rng.random() < p:
            k = rng.randrange(3)
            if k == 0:
                out.append(rng.choice([b for b in alphabet if b != c]))
            elif k == 1:
                out.append(rng.choice(alphabet))
                out.append(c)
        else:
            out.append(c)
    return "".join(out)


def synth(seed, n, lens, probs, alphabet="ACGT"):
    rng = random.Random(seed)
    res = []
    for _ in range(n):
        L = rng.choice(lens)
        p = rng.choice(probs)
        t = "".join(rng.choice(alphabet) for _ in range(L))
        res.append((mutate(rng, t, p, alphabet).encode(), t.encode()))
    return res


def main():
    oracle.build(ref=True)
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libwfe_ref.so is missing (reference sources not mounted?)")
    cases = {
        "readme": readme_pairs(),
        "cfg1": synth(11, 200, [150], [0.02]),
        "cfg2": synth(12, 200, [150], [0.05]),
        "err20": synth(13, 100, [150], [0.20, 0.35, 0.45]),
        "short": synth(14, 300, list(range(0, 41)), [0.0, 0.05, 0.1, 0.2, 0.3, 0.5]),
        "alias": synth(15, 60, [20, 60, 150], [0.05, 0.2], alphabet="ACGTNacgt"),
        "overcap": synth(16, 20, [150], [0.7, 0.9]),
    }
    pairs, case_ids = [], []
    for ci, (name, ps) in enumerate(cases.items()):
        for p, t in ps:
            assert len(p) <= 2 * SEQ_LEN and len(t) <= 2 * SEQ_LEN
            pairs.append((p, t))
            case_ids.append(ci)
    n = len(pairs)
    dist, words, cigars = oracle.ref_align(pairs, SEQ_LEN)
    packed, packed_len = oracle.ref_compact(pairs, SEQ_LEN)
    compat = [oracle.ref_ascii_cigar(cigars[i]) if 0 <= dist[i] < 64 else "" for i in range(n)]
    valid = np.array([oracle.ref_check_cigar(p, t, cigars[i]) if 0 <= dist[i] < 64 else False
                      for i, (p, t) in enumerate(pairs)], dtype=bool)
    seq = b"".join(p + t for p, t in pairs)
    offs = np.zeros((n, 4), dtype=np.int64)
    pos = 0
    for i, (p, t) in enumerate(pairs):
        offs[i] = (pos, len(p), pos + len(p), len(t))
        pos += len(p) + len(t)
    np.savez_compressed(
        OUT,
        seq_len=np.int64(SEQ_LEN),
        case_names=np.array(list(cases.keys())),
        case_ids=np.array(case_ids, dtype=np.int32),
        ascii=np.frombuffer(seq, dtype=np.uint8),
        offsets=offs,
        dist=dist,
        words=words,
        cigars=cigars,
        packed=packed.reshape(n, 2, packed_len),
        compat=np.array(compat),
        ref_check=valid,
    )
    print(f"wrote {OUT}: {n} pairs, {int((dist >= 64).sum())} at the reference cap, "
          f"{int((dist < 0).sum())} not run")


if __name__ == "__main__":
    main()

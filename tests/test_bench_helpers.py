"""The bench's own checking helpers, on the CPU: the parity count it prints
beside every timed result, the CIGAR length it derives the written bytes
from, and the `config` both arms share."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def results(n=6, stride=8, seed=0):
    rng = np.random.default_rng(seed)
    dist = rng.integers(0, 30, n).astype(np.int32)
    cg = rng.integers(1, 100, (n, stride)).astype(np.int8)
    for i in range(n):
        cg[i, i:] = 0  # row i: a CIGAR of i bytes, then its terminator
    st = np.zeros(n, np.uint8)
    return dist, cg, st


def test_cigar_lengths_stop_at_the_terminator():
    cg = np.array([[5, 6, 0, 7], [0, 1, 2, 3], [1, 2, 3, 4]], np.int8)
    assert bench.cigar_lengths(cg).tolist() == [2, 0, 4]


def test_parity_counts_only_what_the_reference_defines():
    d, c, s = results()
    assert bench.parity((d, c, s), (d.copy(), c.copy(), s.copy()))["mismatches"] == 0
    # bytes after a terminator are not part of the CIGAR
    c2 = c.copy()
    c2[2, 5] = 9
    assert c[2, 2] == 0 and bench.parity((d, c2, s), (d, c, s))["mismatches"] == 0
    # a byte before it, a distance or a status is
    c3 = c.copy()
    c3[4, 1] = c3[4, 1] + 1
    assert bench.parity((d, c3, s), (d, c, s))["mismatches"] == 1
    d2 = d.copy()
    d2[0] += 1
    s2 = s.copy()
    s2[5] = 3
    assert bench.parity((d2, c, s2), (d, c, s))["mismatches"] == 2
    # a CIGAR one byte longer (its terminator moved) differs
    c4 = c.copy()
    c4[1, 1] = 7
    assert bench.parity((d, c4, s), (d, c, s))["mismatches"] == 1


def test_both_arms_share_the_config():
    for name in ("short", "long"):
        bench.select_workload(name)
        cfg = bench.workload_config(1, 123_000_000)
        assert set(cfg) == {"workload", "pairs_per_gpu", "batch", "length", "edit_prob", "seed", "cigar_stride",
                            "l2", "parallelism"}
        assert cfg["pairs_per_gpu"] % cfg["batch"] == 0
        assert cfg["cigar_stride"] % 4 == 0 and cfg["cigar_stride"] > cfg["length"]
    bench.select_workload("short")
    assert bench.workload_config(1, 1)["pairs_per_gpu"] == 1_000_000

"""The reference's own GPU kernels against libwfe on the same GB300.

The reference's src/kernels.cu, compiled for sm_100 (oracle/_ref, built
where the reference sources are mounted), runs through oracle's restatement
of its batch loop and dumps every CIGAR slot.  libwfe must produce the same
CIGAR bytes for every pair (all distances here are below the reference's 64
cap, so its output is defined)."""
import os
import tempfile

import numpy as np
import pytest

import oracle as O
import wfe

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not O.ref_cuda_available(),
                                 reason="the reference's kernels were not compiled (no reference sources)")]


def _cigar_bytes(row):
    nz = np.flatnonzero(row == 0)
    return row[: nz[0] + 1].tobytes() if len(nz) else row.tobytes()


@pytest.mark.parametrize("n,length,p,seed,batch,threads", [
    (10000, 150, 0.02, 1, 10000, 1),     # plain method, small, one batch
    (200000, 150, 0.05, 2, 100000, 2),   # short reads, batches of 100k, two host threads
    (30000, 100, 0.10, 5, 7000, 1),      # partial last batch
])
def test_same_cigars_as_reference_kernels(n, length, p, seed, batch, threads):
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "ref.bin")
        rec = O.ref_cuda_run(n, length, p, seed, batch=batch, threads=threads, dump=path)
        stride = length + (4 - length % 4)
        ref = np.fromfile(path, dtype=np.int8).reshape(n, stride)
    assert rec["n"] == n
    ascii, pairs = wfe.generate(n, length, p_min=p, seed=seed)
    with wfe.Context(max_seq_len=2 * length + 4, max_distance=63, cigar_stride=stride) as ctx:
        dist, cg, st = ctx.align(ascii, pairs)
    assert (st == 0).all()
    bad = [i for i in range(n) if _cigar_bytes(cg[i]) != _cigar_bytes(ref[i])]
    assert not bad, f"{len(bad)} CIGARs differ from the reference's kernels, first {bad[:5]}"
    # the reference writes no distances: its distance is the number of X/I/D
    live = np.cumsum(ref == 0, axis=1) == 0
    ref_d = (live & ((ref == ord("X")) | (ref == ord("I")) | (ref == ord("D")))).sum(1)
    np.testing.assert_array_equal(ref_d, dist)

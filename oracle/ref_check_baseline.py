"""CPU baseline: the reference's own host check path (Cigars::check_cigar,
src/wavefront.cuh:297-419) over every pair of the short-read workload, with 1
and with all host threads.  It needs oracle/_ref/libwfe_ref.so, which is built
from the reference's own files: where the reference is mounted, or from the
copies `make ref-stage` left in oracle/_ref/reference (never committed).  The
CIGARs to check come from the CPU restatement, or from the caller.

    python oracle/ref_check_baseline.py [N]
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "ewfa-gpu_gb300"))

import oracle  # noqa: E402
import wfe  # noqa: E402

UNP, STRIDE = 304, 152  # the reader's slot for -l 150 and the reference's cigar_max_len


def run(ascii: np.ndarray, pairs: np.ndarray, cg: np.ndarray) -> list:
    """Time check_cigar over every pair (the reference reader's 304-byte
    slots, CIGAR slots of 152 bytes) on 1 thread and on every host core;
    one record per thread count."""
    lib = os.path.join(HERE, "_ref", "libwfe_ref.so")
    if not os.path.exists(lib):
        raise OSError("oracle/_ref/libwfe_ref.so is missing (it builds only from the reference's files)")
    n = len(pairs)
    exe = os.path.join(HERE, "_ref", "ref_check_bench")
    subprocess.run(["gcc", "-O2", "-I", HERE, os.path.join(HERE, "ref_check_bench.c"), "-o", exe, lib,
                    f"-Wl,-rpath,{os.path.dirname(lib)}", "-lpthread"], check=True)
    cg = np.asarray(cg, dtype=np.int8).reshape(n, -1)
    if cg.shape[1] != STRIDE or max(pairs["p_len"].max(), pairs["t_len"].max()) > UNP:
        raise ValueError("the check baseline runs on the short-read layout (-l 150)")
    buf = np.zeros((n, 2, UNP), np.uint8)
    for which, off_f, len_f in ((0, "p_off", "p_len"), (1, "t_off", "t_len")):
        off, ln = pairs[off_f].astype(np.int64), pairs[len_f].astype(np.int64)
        for L in np.unique(ln):
            idx = np.flatnonzero(ln == L)
            buf[idx, which, :L] = ascii[off[idx][:, None] + np.arange(L)[None, :]]
    recs = []
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "pairs.bin")
        with open(path, "wb") as f:
            f.write(pairs["p_len"].astype(np.uint32).tobytes())
            f.write(pairs["t_len"].astype(np.uint32).tobytes())
            f.write(buf.tobytes())
            f.write(cg.tobytes())
        del buf
        for t in sorted({1, os.cpu_count() or 1}):
            out = subprocess.run([exe, path, str(n), str(t)], check=True, capture_output=True, text=True).stdout
            recs.append(json.loads(out))
    return recs


def main(n: int) -> None:
    ascii, pairs = wfe.generate(n, 150, p_min=0.05, seed=2)
    _, cg, _, _ = oracle.align_batch(ascii, pairs["p_off"], pairs["p_len"], pairs["t_off"], pairs["t_len"],
                                     STRIDE, nthreads=os.cpu_count() or 1)
    for r in run(ascii, pairs, cg):
        print(json.dumps(r))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 1_000_000)

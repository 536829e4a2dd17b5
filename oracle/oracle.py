"""ctypes access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Two libraries, both built by ``oracle/Makefile``:

* ``_build/libwfe_oracle.so`` -- the C restatement of the reference path
  (``wfe_oracle.c``), available wherever gcc is;
* ``_ref/libwfe_ref.so`` -- the reference's own ``src/kernels.cu`` compiled for
  the CPU with ``ref_shim/`` (only where the reference sources were present at
  build time; never on a machine without them).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module.  The product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libwfe_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libwfe_ref.so")
# the reference checkout, where it is mounted; else the copies of the few files
# the CPU build needs, staged into _ref/ (never committed) by `make ref-stage`
REF_SRC = os.environ.get("WFE_REFERENCE_DIR", "/root/reference")
REF_STAGED = os.path.join(HERE, "_ref", "reference")

OP_INS, OP_SUB, OP_DEL = 1, 2, 3
PAIR_OK, PAIR_OVER_MAX, PAIR_CIGAR_TRUNCATED = 0, 1, 2


REF_CUBIN = os.path.join(HERE, "_ref", "ref_kernels_sm100.cubin")
REF_HARNESS = os.path.join(HERE, "_build", "ref_cuda_harness")


def build(ref: bool | None = None) -> None:
    """Compile the restatement and the driver of the reference's GPU kernels;
    where the reference sources exist, also the reference-on-CPU library and
    the reference's kernels as an sm_100 cubin, and stage the files the CPU
    library needs into _ref/reference.  Where only that staged copy exists
    (a machine without the reference, e.g. the GPU machine), the CPU library is
    built from it."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    mounted = os.path.isdir(os.path.join(REF_SRC, "src"))
    staged = os.path.isdir(os.path.join(REF_STAGED, "src"))
    if ref is not False and mounted:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "ref-cubin", "ref-stage", f"REF={REF_SRC}"], check=True)
    elif ref is not False and staged:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_STAGED}"], check=bool(ref))
    if os.path.exists(REF_CUBIN):
        subprocess.run(["make", "-s", "-C", HERE, "ref-harness"], check=False)


def ref_cuda_available() -> bool:
    return os.path.exists(REF_CUBIN) and os.path.exists(REF_HARNESS)


def ref_cuda_run(n: int, length: int, p: float, seed: int, batch: int | None = None, threads: int = 1,
                 reps: int = 1, dump: str | None = None, steady: bool = False) -> dict:
    """Run the reference's own GPU kernels (sm_100 cubin) through the
    restated batch loop; returns the harness's JSON record.  steady: the
    allocations are made before the clock starts and freed after it stops
    (the batch loop alone is timed)."""
    import json
    cmd = [REF_HARNESS, "--cubin", REF_CUBIN, "-n", str(n), "-l", str(length), "-b", str(batch or n),
           "-t", str(threads), "--p", str(p), "--seed", str(seed), "--reps", str(reps)]
    if dump:
        cmd += ["--dump", dump]
    if steady:
        cmd += ["--steady"]
    out = subprocess.run(cmd, check=True, stdout=subprocess.PIPE, text=True).stdout
    return json.loads(out.strip().splitlines()[-1])


def ref_cuda_run_pairs(ascii: np.ndarray, pairs: np.ndarray, slot_len: int, batch: int, threads: int = 1,
                       reps: int = 1, steady: bool = False, dump: str | None = None) -> dict:
    """The reference's GPU kernels on given pairs (descriptor records with
    p_off, p_len, t_off, t_len into `ascii`): written to a pairs file, run
    with -l slot_len (every sequence at most 2 * slot_len bases)."""
    import json
    import tempfile
    n = len(pairs)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "pairs.bin")
        with open(path, "wb") as f:
            f.write(np.array([n, slot_len], np.uint64).tobytes())
            f.write(pairs["p_len"].astype(np.uint32).tobytes())
            f.write(pairs["t_len"].astype(np.uint32).tobytes())
            for q in pairs:
                f.write(ascii[q["p_off"]:q["p_off"] + q["p_len"]].tobytes())
                f.write(ascii[q["t_off"]:q["t_off"] + q["t_len"]].tobytes())
        cmd = [REF_HARNESS, "--cubin", REF_CUBIN, "--pairs-file", path, "-b", str(min(batch, n)),
               "-t", str(threads), "--reps", str(reps)]
        if steady:
            cmd += ["--steady"]
        if dump:
            cmd += ["--dump", dump]
        out = subprocess.run(cmd, check=True, stdout=subprocess.PIPE, text=True).stdout
    return json.loads(out.strip().splitlines()[-1])


class _Counts(C.Structure):
    _fields_ = [("cells", C.c_uint64), ("extend_words", C.c_uint64)]


_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = C.CDLL(ORACLE_SO)
        u8p, i8p, u32p, u64p, i32p = (C.POINTER(C.c_uint8), C.POINTER(C.c_int8),
                                      C.POINTER(C.c_uint32), C.POINTER(C.c_uint64),
                                      C.POINTER(C.c_int32))
        L.wfo_pack.argtypes = [C.c_char_p, C.c_uint32, u32p, C.c_uint32]
        L.wfo_align.argtypes = [C.c_char_p, C.c_uint32, C.c_char_p, C.c_uint32, C.c_int32,
                                i32p, u8p, C.c_size_t, C.POINTER(_Counts)]
        L.wfo_align.restype = C.c_int
        L.wfo_cigar.argtypes = [C.c_char_p, C.c_uint32, C.c_char_p, C.c_uint32, C.c_int32,
                                u8p, i8p, C.c_size_t, C.POINTER(C.c_size_t), u64p]
        L.wfo_cigar.restype = C.c_int
        L.wfo_check_cigar.argtypes = [C.c_char_p, C.c_uint32, C.c_char_p, C.c_uint32, i8p,
                                      C.c_size_t, i32p]
        L.wfo_check_cigar.restype = C.c_int
        L.wfo_format_cigar.argtypes = [i8p, C.c_size_t, C.c_char_p, C.c_size_t]
        L.wfo_format_cigar.restype = C.c_size_t
        L.wfo_format_cigar_compat.argtypes = [i8p, C.c_size_t, C.c_char_p, C.c_size_t]
        L.wfo_format_cigar_compat.restype = C.c_size_t
        L.wfo_levenshtein.argtypes = [C.c_char_p, C.c_uint32, C.c_char_p, C.c_uint32]
        L.wfo_levenshtein.restype = C.c_int32
        L.wfo_align_batch.argtypes = [C.c_void_p, u64p, u32p, u64p, u32p, C.c_size_t, C.c_int32,
                                      i32p, i8p, C.c_size_t, u8p, C.c_int, C.POINTER(_Counts)]
        L.wfo_align_batch.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        R = C.CDLL(REF_SO)
        i8p, u32p, u64p, i32p = (C.POINTER(C.c_int8), C.POINTER(C.c_uint32),
                                 C.POINTER(C.c_uint64), C.POINTER(C.c_int32))
        R.ref_max_seq_len_unpacked.argtypes = [C.c_size_t]
        R.ref_max_seq_len_unpacked.restype = C.c_size_t
        R.ref_max_seq_len_packed.argtypes = [C.c_size_t]
        R.ref_max_seq_len_packed.restype = C.c_size_t
        R.ref_compact.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_void_p]
        R.ref_align.argtypes = [C.c_void_p, C.c_size_t, u32p, u32p, C.c_size_t, i32p, u64p,
                                i8p, C.c_size_t]
        R.ref_check_cigar.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_uint32, C.c_uint32,
                                      i8p, C.c_size_t]
        R.ref_ascii_cigar.argtypes = [i8p, C.c_size_t, C.c_char_p, C.c_size_t]
        R.ref_ascii_cigar.restype = C.c_size_t
        R.ref_ascii_sequence.argtypes = [C.c_void_p, C.c_size_t, C.c_char_p]
        R.ref_cigar_from_bt.argtypes = [C.c_char_p, C.c_int, C.c_char_p, C.c_int, C.c_int32,
                                        u64p, C.c_char_p, C.c_size_t]
        R.ref_cigar_from_bt.restype = C.c_size_t
        _ref = R
    return _ref


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


# --------------------------------------------------------------------------
# restatement

def pack(seq: bytes, nwords: int | None = None) -> np.ndarray:
    if nwords is None:
        nwords = (len(seq) + 15) // 16
    out = np.zeros(max(nwords, 1), dtype=np.uint32)
    lib().wfo_pack(seq, len(seq), _ptr(out, C.c_uint32), nwords)
    return out[:nwords]


def align(p: bytes, t: bytes, max_distance: int = 0):
    """(status, distance, ops[list], counts) for one pair."""
    cap = max(len(p), len(t)) + 2
    ops = np.zeros(cap, dtype=np.uint8)
    d = C.c_int32(0)
    cnt = _Counts()
    st = lib().wfo_align(p, len(p), t, len(t), max_distance, C.byref(d), _ptr(ops, C.c_uint8),
                         cap, C.byref(cnt))
    if st < 0:
        raise RuntimeError("wfo_align failed")
    n = d.value if st == PAIR_OK else 0
    return st, d.value, ops[:n].tolist(), (cnt.cells, cnt.extend_words)


def cigar(p: bytes, t: bytes, distance: int, ops, cap: int):
    """(status, encoded cigar bytes as np.int8[cap], full length)."""
    o = np.asarray(list(ops) + [0], dtype=np.uint8)
    out = np.zeros(cap, dtype=np.int8)
    ln = C.c_size_t(0)
    st = lib().wfo_cigar(p, len(p), t, len(t), distance, _ptr(o, C.c_uint8),
                         _ptr(out, C.c_int8), cap, C.byref(ln), None)
    return st, out, ln.value


def check_cigar(p: bytes, t: bytes, cg: np.ndarray):
    s = C.c_int32(0)
    cg = np.ascontiguousarray(cg, dtype=np.int8)
    ok = lib().wfo_check_cigar(p, len(p), t, len(t), _ptr(cg, C.c_int8), cg.size, C.byref(s))
    return bool(ok), s.value


def format_cigar(cg: np.ndarray, compat: bool = False) -> str:
    cg = np.ascontiguousarray(cg, dtype=np.int8)
    fn = lib().wfo_format_cigar_compat if compat else lib().wfo_format_cigar
    need = fn(_ptr(cg, C.c_int8), cg.size, None, 0)
    buf = C.create_string_buffer(need + 1)
    fn(_ptr(cg, C.c_int8), cg.size, buf, need + 1)
    return buf.value.decode()


def levenshtein(p: bytes, t: bytes) -> int:
    return lib().wfo_levenshtein(p, len(p), t, len(t))


def align_batch(ascii: np.ndarray, p_off, p_len, t_off, t_len, cigar_stride: int,
                max_distance: int = 0, nthreads: int = 1):
    """Align every pair of a batch; returns (dist, cigars[n, stride], status, counts)."""
    n = len(p_len)
    p_off = np.ascontiguousarray(p_off, dtype=np.uint64)
    t_off = np.ascontiguousarray(t_off, dtype=np.uint64)
    p_len = np.ascontiguousarray(p_len, dtype=np.uint32)
    t_len = np.ascontiguousarray(t_len, dtype=np.uint32)
    dist = np.zeros(n, dtype=np.int32)
    cg = np.zeros((n, cigar_stride), dtype=np.int8)
    st = np.zeros(n, dtype=np.uint8)
    cnt = _Counts()
    lib().wfo_align_batch(ascii.ctypes.data, _ptr(p_off, C.c_uint64), _ptr(p_len, C.c_uint32),
                          _ptr(t_off, C.c_uint64), _ptr(t_len, C.c_uint32), n, max_distance,
                          _ptr(dist, C.c_int32), _ptr(cg, C.c_int8), cigar_stride,
                          _ptr(st, C.c_uint8), nthreads, C.byref(cnt))
    return dist, cg, st, (cnt.cells, cnt.extend_words)


# --------------------------------------------------------------------------
# reference kernels on the CPU

def ref_layout(pairs, seq_len: int):
    """The reference reader's host buffer: pattern i at 2*i*unp, text at
    (2*i+1)*unp, zero padded (utils/sequence_reader.cu:148-189)."""
    unp = ref().ref_max_seq_len_unpacked(seq_len)
    buf = np.zeros(2 * unp * max(len(pairs), 1), dtype=np.uint8)
    for i, (p, t) in enumerate(pairs):
        buf[2 * i * unp: 2 * i * unp + len(p)] = np.frombuffer(p, dtype=np.uint8)
        buf[(2 * i + 1) * unp: (2 * i + 1) * unp + len(t)] = np.frombuffer(t, dtype=np.uint8)
    return buf, unp


def ref_compact(pairs, seq_len: int):
    buf, unp = ref_layout(pairs, seq_len)
    plen_b = ref().ref_max_seq_len_packed(seq_len)
    packed = np.zeros(2 * plen_b * max(len(pairs), 1), dtype=np.uint8)
    ref().ref_compact(buf.ctypes.data, unp, plen_b, len(pairs), packed.ctypes.data)
    return packed, plen_b


def ref_align(pairs, seq_len: int, cigar_max_len: int | None = None):
    """Reference kernels end to end: (dist, words[n,2], cigars[n, cml])."""
    if cigar_max_len is None:
        cigar_max_len = seq_len + (4 - seq_len % 4)
    packed, plen_b = ref_compact(pairs, seq_len)
    n = len(pairs)
    pl = np.array([len(p) for p, _ in pairs], dtype=np.uint32)
    tl = np.array([len(t) for _, t in pairs], dtype=np.uint32)
    dist = np.zeros(n, dtype=np.int32)
    words = np.zeros((n, 2), dtype=np.uint64)
    cg = np.zeros((n, cigar_max_len), dtype=np.int8)
    rc = ref().ref_align(packed.ctypes.data, plen_b, _ptr(pl, C.c_uint32), _ptr(tl, C.c_uint32),
                         n, _ptr(dist, C.c_int32), _ptr(words, C.c_uint64), _ptr(cg, C.c_int8),
                         cigar_max_len)
    if rc != 0:
        raise RuntimeError(f"ref_align failed ({rc})")
    return dist, words, cg


def ref_ascii_cigar(cg: np.ndarray) -> str:
    cg = np.ascontiguousarray(cg, dtype=np.int8)
    buf = C.create_string_buffer(4 * cg.size + 64)
    ref().ref_ascii_cigar(_ptr(cg, C.c_int8), cg.size, buf, len(buf))
    return buf.value.decode()


def ref_ascii_sequence(words: np.ndarray, length: int) -> bytes:
    w = np.ascontiguousarray(words, dtype=np.uint32)
    out = C.create_string_buffer(length + 1)
    ref().ref_ascii_sequence(w.ctypes.data, length, out)
    return out.raw[:length]


def ref_check_cigar(p: bytes, t: bytes, cg: np.ndarray) -> bool:
    seq_len = max(len(p), len(t))
    buf, unp = ref_layout([(p, t)], seq_len)
    cg = np.ascontiguousarray(cg, dtype=np.int8)
    return bool(ref().ref_check_cigar(buf.ctypes.data, unp, 0, len(p), len(t),
                                      _ptr(cg, C.c_int8), cg.size))


def ops_from_words(words, distance: int):
    """2-bit fields 0..D-1 of the reference's 128-bit history."""
    w0, w1 = int(words[0]), int(words[1])
    return [((w0 if d < 32 else w1) >> (2 * (d % 32))) & 3 for d in range(distance)]

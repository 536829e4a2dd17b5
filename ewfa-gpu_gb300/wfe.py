"""Python binding of libwfe (include/wfe.h) over ctypes.

The alignment path is the CUDA library; this module only marshals buffers.
It never computes alignments itself and raises if the library is missing or
no CUDA device is present -- there is no CPU fallback.  Device buffers may be
torch CUDA tensors (torch is used only to allocate device memory and to name
streams) or raw integer device addresses.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libwfe.so")
GEN_PATH = os.path.join(PKG, "lib", "libwfe_gen.so")

# status codes (include/wfe.h)
OK = 0
ERR_INVALID_ARGUMENT, ERR_OUT_OF_MEMORY, ERR_SEQ_TOO_LONG, ERR_CUDA = 1, 2, 3, 4
ERR_NO_DEVICE, ERR_TIMEOUT, ERR_BUSY, ERR_INTERNAL, ERR_NOT_FOUND = 5, 6, 7, 8, 9
PAIR_OK, PAIR_OVER_MAX_DISTANCE, PAIR_CIGAR_TRUNCATED, PAIR_TOO_LONG, PAIR_BAD_HISTORY = 0, 1, 2, 3, 4
PAIR_OUT_OF_RANGE = 5
FLAG_NO_PIPELINE = 1
FLAG_KERNEL_TIMING = 2
FLAG_DEVICE_ONLY = 4
FLAG_PAGEABLE_IN_PLACE = 8
POLICY_PREDICT = 1
POLICY_NO_BOUND = 2

PAIR_DTYPE = np.dtype([("p_off", "<u8"), ("t_off", "<u8"), ("p_len", "<u4"), ("t_len", "<u4")])
assert PAIR_DTYPE.itemsize == 24

SYMBOLS = [
    "wfe_create", "wfe_create_with_scratch", "wfe_destroy", "wfe_strerror", "wfe_last_cuda_error", "wfe_get_stats",
    "wfe_reset_stats", "wfe_align", "wfe_align_strided", "wfe_align_device", "wfe_pack_device",
    "wfe_cigar_from_history_device", "wfe_format_cigar", "wfe_check_cigar", "wfe_align_device_noalloc",
    "wfe_read_pair_file", "wfe_free_pair_file", "wfe_host_alloc", "wfe_host_free", "wfe_device_count",
    "wfe_device_name", "wfe_set_policy", "wfe_get_policy", "wfe_autotune",
    "wfe_server_create", "wfe_server_destroy", "wfe_submit", "wfe_poll", "wfe_server_get_stats",
]
NOALLOC_MAX_DISTANCE = 271
NOALLOC_SCRATCH_BYTES = 16 << 20


class WfeError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {strerror(code)} ({code})" if what else f"{strerror(code)} ({code})")


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_seq_len", C.c_uint32), ("batch_size", C.c_uint32),
                ("max_distance", C.c_int32), ("cigar_stride", C.c_uint32), ("flags", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [("pairs", C.c_uint64), ("batches", C.c_uint64), ("kernel_launches", C.c_uint64),
                ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("tier_entered", C.c_uint64 * 8),
                ("tier_passed", C.c_uint64 * 8), ("tier_launches", C.c_uint64 * 8),
                ("tier_ms", C.c_double * 8), ("mapped_batches", C.c_uint64), ("deferred_pairs", C.c_uint64),
                ("deep_scratch_bytes", C.c_uint64)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_seq_len", C.c_uint32), ("cigar_stride", C.c_uint32),
                ("max_distance", C.c_int32), ("lanes", C.c_uint32), ("batch_pairs", C.c_uint32),
                ("memory_bytes", C.c_uint64), ("nbuckets", C.c_uint32), ("bucket_max_len", C.c_uint32 * 8),
                ("first_tier", C.c_int32 * 8), ("policy_flags", C.c_uint32)]


class RequestInfo(C.Structure):
    _fields_ = [("submit_ns", C.c_uint64), ("start_ns", C.c_uint64), ("done_ns", C.c_uint64),
                ("pairs", C.c_uint32), ("batches", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("requests", C.c_uint64), ("pairs", C.c_uint64), ("batches", C.c_uint64),
                ("split_requests", C.c_uint64), ("max_in_flight", C.c_uint32), ("lanes", C.c_uint32),
                ("memory_bytes", C.c_uint64), ("peak_memory", C.c_uint64), ("admit_ns", C.c_uint64),
                ("finish_ns", C.c_uint64)]


class PairFileC(C.Structure):
    _fields_ = [("ascii", C.c_void_p), ("ascii_bytes", C.c_size_t), ("pairs", C.c_void_p), ("n", C.c_size_t),
                ("longest", C.c_uint32), ("pinned", C.c_int)]


class GenConfig(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("len_min", C.c_uint32), ("len_max", C.c_uint32),
                ("p_min", C.c_double), ("p_max", C.c_double)]


_lib = None
_gen = None


def lib_path() -> str:
    return LIB_PATH


def load() -> C.CDLL:
    """Load libwfe.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libwfe is not built ({LIB_PATH}); run ewfa-gpu_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    vp, sz, u32, i32 = C.c_void_p, C.c_size_t, C.c_uint32, C.c_int32
    L.wfe_create.argtypes = [C.POINTER(Config), C.POINTER(C.c_void_p)]
    L.wfe_create_with_scratch.argtypes = [C.POINTER(Config), C.c_uint64, C.c_uint64, C.POINTER(C.c_void_p)]
    L.wfe_destroy.argtypes = [vp]
    L.wfe_destroy.restype = None
    L.wfe_strerror.argtypes = [C.c_int]
    L.wfe_strerror.restype = C.c_char_p
    L.wfe_last_cuda_error.argtypes = [vp]
    L.wfe_get_stats.argtypes = [vp, C.POINTER(Stats)]
    L.wfe_reset_stats.argtypes = [vp]
    L.wfe_align.argtypes = [vp, vp, sz, vp, sz, vp, vp, vp]
    L.wfe_align_strided.argtypes = [vp, vp, sz, vp, vp, sz, vp, vp, vp]
    L.wfe_align_device.argtypes = [vp, vp, vp, sz, u32, vp, vp, vp, vp]
    L.wfe_pack_device.argtypes = [vp, vp, sz, vp, u32, vp]
    L.wfe_cigar_from_history_device.argtypes = [vp, vp, sz, u32, vp, vp, vp, u32, vp, vp]
    L.wfe_format_cigar.argtypes = [vp, sz, C.c_char_p, sz, C.c_int]
    L.wfe_format_cigar.restype = sz
    L.wfe_check_cigar.argtypes = [C.c_char_p, u32, C.c_char_p, u32, vp, sz, C.POINTER(i32)]
    L.wfe_align_device_noalloc.argtypes = [vp, vp, sz, u32, i32, vp, vp, u32, vp, vp]
    L.wfe_set_policy.argtypes = [vp, u32, vp, vp, u32]
    L.wfe_get_policy.argtypes = [vp, C.POINTER(C.c_uint32), vp, vp, C.POINTER(C.c_uint32)]
    L.wfe_autotune.argtypes = [vp, vp, vp, sz, u32, vp, u32, C.c_char_p, vp]
    L.wfe_read_pair_file.argtypes = [C.c_char_p, sz, C.c_int, C.c_int, C.POINTER(PairFileC), C.c_char_p, sz]
    L.wfe_free_pair_file.argtypes = [C.POINTER(PairFileC)]
    L.wfe_free_pair_file.restype = None
    L.wfe_host_alloc.argtypes = [C.POINTER(C.c_void_p), sz]
    L.wfe_host_free.argtypes = [vp]
    L.wfe_host_free.restype = None
    L.wfe_device_count.argtypes = [C.POINTER(C.c_int)]
    L.wfe_device_name.argtypes = [C.c_int, C.c_char_p, sz, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.wfe_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]
    L.wfe_server_destroy.argtypes = [vp]
    L.wfe_server_destroy.restype = None
    L.wfe_submit.argtypes = [vp, vp, sz, vp, sz, vp, vp, vp, C.POINTER(C.c_uint64)]
    L.wfe_poll.argtypes = [vp, C.c_uint64, C.c_int64, C.POINTER(RequestInfo)]
    L.wfe_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
    for name in SYMBOLS:
        getattr(L, name)
    _lib = L
    return L


def gen_lib() -> C.CDLL:
    global _gen
    if _gen is None:
        if not os.path.exists(GEN_PATH):
            raise RuntimeError(f"libwfe_gen is not built ({GEN_PATH})")
        G = C.CDLL(GEN_PATH)
        G.wfe_gen_batch.argtypes = [C.POINTER(GenConfig), C.c_uint64, C.c_size_t, C.c_void_p, C.c_size_t,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        G.wfe_gen_batch.restype = C.c_size_t
        G.wfe_gen_pair_cap.argtypes = [C.POINTER(GenConfig)]
        G.wfe_gen_pair_cap.restype = C.c_size_t
        G.wfe_gen_file.argtypes = [C.POINTER(GenConfig), C.c_uint64, C.c_size_t, C.c_char_p]
        _gen = G
    return _gen


def strerror(code: int) -> str:
    try:
        return load().wfe_strerror(code).decode()
    except RuntimeError:
        return f"status {code}"


def _check(code: int, what: str) -> None:
    if code != OK:
        raise WfeError(code, what)


def _addr(x) -> int:
    """Device or host address of a torch tensor, numpy array or int."""
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return int(x.data_ptr())


def reference_cigar_stride(max_seq_len: int) -> int:
    """cigar_max_len of the reference for -l max_seq_len (src/wavefront.cuh:48-50)."""
    return max_seq_len + (4 - max_seq_len % 4)


# --------------------------------------------------------------------------
# workload generator

def generate(n: int, len_min: int, len_max: int | None = None, p_min: float = 0.05,
             p_max: float | None = None, seed: int = 1, first: int = 0, nthreads: int | None = None):
    """Synthetic pairs in one contiguous ASCII buffer: (ascii uint8[], pairs PAIR_DTYPE[])."""
    cfg = GenConfig(seed, len_min, len_max if len_max is not None else len_min, p_min,
                    p_max if p_max is not None else p_min)
    cap = n * gen_lib().wfe_gen_pair_cap(C.byref(cfg)) + 64
    ascii = np.zeros(cap, dtype=np.uint8)
    p_off = np.zeros(n, dtype=np.uint64)
    t_off = np.zeros(n, dtype=np.uint64)
    p_len = np.zeros(n, dtype=np.uint32)
    t_len = np.zeros(n, dtype=np.uint32)
    nt = nthreads or min(16, os.cpu_count() or 1)
    total = gen_lib().wfe_gen_batch(C.byref(cfg), first, n, ascii.ctypes.data, cap, p_off.ctypes.data,
                                    p_len.ctypes.data, t_off.ctypes.data, t_len.ctypes.data, nt)
    if total == C.c_size_t(-1).value:
        raise RuntimeError("generator buffer too small")
    pairs = np.zeros(n, dtype=PAIR_DTYPE)
    pairs["p_off"], pairs["t_off"], pairs["p_len"], pairs["t_len"] = p_off, t_off, p_len, t_len
    out = np.zeros(total + 64, dtype=np.uint8)
    out[:total] = ascii[:total]
    return out, pairs


def generate_file(path: str, n: int, len_min: int, len_max: int | None = None, p_min: float = 0.05,
                  p_max: float | None = None, seed: int = 1, first: int = 0) -> None:
    cfg = GenConfig(seed, len_min, len_max if len_max is not None else len_min, p_min,
                    p_max if p_max is not None else p_min)
    if gen_lib().wfe_gen_file(C.byref(cfg), first, n, path.encode()) != 0:
        raise RuntimeError(f"could not write {path}")


def read_pair_file(path: str, max_pairs: int = 1 << 62, nthreads: int = 0, pin: bool = False):
    """wfe_read_pair_file: (ascii uint8[], pairs PAIR_DTYPE[], longest) copied
    out of the library's buffers."""
    f = PairFileC()
    err = C.create_string_buffer(256)
    rc = load().wfe_read_pair_file(path.encode(), max_pairs, nthreads or (os.cpu_count() or 1), int(pin),
                                   C.byref(f), err, 256)
    if rc != OK:
        raise WfeError(rc, err.value.decode() or "wfe_read_pair_file")
    try:
        ascii = np.ctypeslib.as_array((C.c_uint8 * (f.ascii_bytes + 64)).from_address(f.ascii)).copy()
        pairs = np.ctypeslib.as_array((C.c_uint8 * (24 * f.n)).from_address(f.pairs)).copy().view(PAIR_DTYPE) \
            if f.n else np.zeros(0, PAIR_DTYPE)
        return ascii, pairs, f.longest
    finally:
        load().wfe_free_pair_file(C.byref(f))


def pairs_from_list(seqs):
    """[(pattern bytes, text bytes)] -> (ascii, pairs) back to back."""
    parts, recs, pos = [], [], 0
    for p, t in seqs:
        recs.append((pos, pos + len(p), len(p), len(t)))
        parts += [p, t]
        pos += len(p) + len(t)
    ascii = np.frombuffer(b"".join(parts) + b"\0" * 64, dtype=np.uint8).copy()
    pairs = np.array(recs, dtype=PAIR_DTYPE) if recs else np.zeros(0, dtype=PAIR_DTYPE)
    return ascii, pairs


# --------------------------------------------------------------------------
# context

class Context:
    """One libwfe context (device buffers, streams) -- the counterpart of one
    reference Sequences object (src/wavefront.cuh:435-505).

    flags=FLAG_PAGEABLE_IN_PLACE lets align() use ordinary numpy arrays in
    place on a GB300 (the GPU reads the CPU's page tables): 1M x 150-base
    pairs with fresh output arrays take ~4 ms instead of ~29 ms staged.  Bad
    descriptors are then reported per pair, as with pinned arrays, instead
    of failing the call.

    long_scratch=(tier5_bytes, tier6_bytes) bounds the device memory of the
    CTA-per-pair tiers' slabs (wfe_create_with_scratch); None keeps the
    defaults."""

    def __init__(self, max_seq_len: int, batch_size: int = 100000, max_distance: int = 0,
                 cigar_stride: int = 0, device: int = 0, flags: int = 0, long_scratch=None):
        L = load()
        self.cfg = Config(device, max_seq_len, batch_size, max_distance, cigar_stride, flags)
        h = C.c_void_p()
        if long_scratch is None:
            rc = L.wfe_create(C.byref(self.cfg), C.byref(h))
        else:
            b5, b6 = long_scratch
            rc = L.wfe_create_with_scratch(C.byref(self.cfg), int(b5), int(b6), C.byref(h))
        if rc != OK:
            raise WfeError(rc, f"wfe_create (cuda error {L.wfe_last_cuda_error(None)})")
        self._h = h
        self.cigar_stride = cigar_stride or reference_cigar_stride(max_seq_len)
        self.max_seq_len = max_seq_len

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().wfe_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def last_cuda_error(self) -> int:
        return load().wfe_last_cuda_error(self._h)

    def stats(self) -> dict:
        s = Stats()
        _check(load().wfe_get_stats(self._h, C.byref(s)), "wfe_get_stats")
        return {"pairs": s.pairs, "batches": s.batches, "kernel_launches": s.kernel_launches,
                "h2d_bytes": s.h2d_bytes, "d2h_bytes": s.d2h_bytes,
                "tier_entered": list(s.tier_entered), "tier_passed": list(s.tier_passed),
                "tier_launches": list(s.tier_launches), "tier_ms": list(s.tier_ms),
                "mapped_batches": s.mapped_batches, "deferred_pairs": s.deferred_pairs,
                "deep_scratch_bytes": s.deep_scratch_bytes}

    def reset_stats(self) -> None:
        _check(load().wfe_reset_stats(self._h), "wfe_reset_stats")

    def set_policy(self, bucket_max_len, first_tier=None, predict: bool = False, bound: bool = True) -> None:
        """Length buckets (ascending max lengths), each bucket's first tier
        (-1 = by length), distance prediction and the distance bounds of the
        CTA-per-pair tiers; see wfe_set_policy."""
        bm = np.ascontiguousarray(bucket_max_len, dtype=np.uint32)
        ft = None if first_tier is None else np.ascontiguousarray(first_tier, dtype=np.int32)
        flags = (POLICY_PREDICT if predict else 0) | (0 if bound else POLICY_NO_BOUND)
        _check(load().wfe_set_policy(self._h, len(bm), _addr(bm), _addr(ft), flags), "wfe_set_policy")

    def policy(self):
        nb, fl = C.c_uint32(0), C.c_uint32(0)
        bm = np.zeros(8, np.uint32)
        ft = np.zeros(8, np.int32)
        _check(load().wfe_get_policy(self._h, C.byref(nb), _addr(bm), _addr(ft), C.byref(fl)), "wfe_get_policy")
        return bm[:nb.value].tolist(), ft[:nb.value].tolist(), bool(fl.value & POLICY_PREDICT)

    def autotune(self, d_ascii, d_pairs, n: int, bucket_max_len, cache_path: str | None = None,
                 predict: bool = False):
        """Measure every bucket's best first tier on device-resident pairs; returns the tiers."""
        bm = np.ascontiguousarray(bucket_max_len, dtype=np.uint32)
        out = np.zeros(len(bm), np.int32)
        _check(load().wfe_autotune(self._h, _addr(d_ascii), _addr(d_pairs), n, len(bm), _addr(bm),
                                   POLICY_PREDICT if predict else 0,
                                   cache_path.encode() if cache_path else None, _addr(out)), "wfe_autotune")
        return out.tolist()

    def align(self, ascii: np.ndarray, pairs: np.ndarray, out=None):
        """Host buffers in, host buffers out: (dist int32[n], cigar int8[n, stride], status uint8[n])."""
        n = len(pairs)
        pairs = np.ascontiguousarray(pairs, dtype=PAIR_DTYPE)
        ascii = np.ascontiguousarray(ascii)
        if out is None:
            out = (np.zeros(n, np.int32), np.zeros((n, self.cigar_stride), np.int8), np.zeros(n, np.uint8))
        dist, cg, st = out
        # the library writes through raw pointers: outputs must be whole, contiguous arrays
        for a, dt, size in ((dist, np.int32, n), (cg, np.int8, n * self.cigar_stride), (st, np.uint8, n)):
            if a.dtype != dt or a.size != size or not a.flags.c_contiguous or not a.flags.writeable:
                raise ValueError(f"output must be a writable C-contiguous {np.dtype(dt).name} array of {size} "
                                 f"elements (got {a.dtype}, {a.size}, contiguous={a.flags.c_contiguous})")
        _check(load().wfe_align(self._h, _addr(ascii), ascii.nbytes, _addr(pairs), n, _addr(dist),
                                _addr(cg), _addr(st)), "wfe_align")
        return dist, cg, st

    def align_strided(self, ascii: np.ndarray, stride: int, p_len, t_len):
        n = len(p_len)
        p_len = np.ascontiguousarray(p_len, dtype=np.uint32)
        t_len = np.ascontiguousarray(t_len, dtype=np.uint32)
        dist, cg, st = np.zeros(n, np.int32), np.zeros((n, self.cigar_stride), np.int8), np.zeros(n, np.uint8)
        _check(load().wfe_align_strided(self._h, _addr(ascii), stride, _addr(p_len), _addr(t_len), n,
                                        _addr(dist), _addr(cg), _addr(st)), "wfe_align_strided")
        return dist, cg, st

    def align_device(self, d_ascii, d_pairs, n: int, max_len: int, d_dist, d_cigar, d_status,
                     stream=None) -> None:
        """Device buffers in and out, asynchronous on `stream` (int handle or torch stream)."""
        s = stream.cuda_stream if hasattr(stream, "cuda_stream") else (stream or 0)
        _check(load().wfe_align_device(self._h, _addr(d_ascii), _addr(d_pairs), n, max_len, _addr(d_dist),
                                       _addr(d_cigar), _addr(d_status), s), "wfe_align_device")


# --------------------------------------------------------------------------
# serving

class Request:
    """A submitted request: its ticket and the buffers its results go to."""
    __slots__ = ("ticket", "ascii", "pairs", "dist", "cigar", "status", "info")

    def __init__(self, ticket, ascii, pairs, dist, cigar, status):
        self.ticket, self.ascii, self.pairs = ticket, ascii, pairs
        self.dist, self.cigar, self.status = dist, cigar, status
        self.info = None


class Server:
    """wfe_server: requests of any size submitted at any time, aligned in
    continuously formed batches on several streams (see wfe_server_create)."""

    def __init__(self, max_seq_len: int, cigar_stride: int = 0, max_distance: int = 0, lanes: int = 0,
                 batch_pairs: int = 0, memory_bytes: int = 0, bucket_max_len=None, first_tier=None,
                 predict: bool = False, device: int = 0, bound: bool = True):
        cfg = ServerConfig()
        cfg.device, cfg.max_seq_len, cfg.cigar_stride, cfg.max_distance = device, max_seq_len, cigar_stride, \
            max_distance
        cfg.lanes, cfg.batch_pairs, cfg.memory_bytes = lanes, batch_pairs, memory_bytes
        if bucket_max_len:
            cfg.nbuckets = len(bucket_max_len)
            for i, m in enumerate(bucket_max_len):
                cfg.bucket_max_len[i] = m
                cfg.first_tier[i] = -1 if first_tier is None else first_tier[i]
        cfg.policy_flags = (POLICY_PREDICT if predict else 0) | (0 if bound else POLICY_NO_BOUND)
        h = C.c_void_p()
        _check(load().wfe_server_create(C.byref(cfg), C.byref(h)), "wfe_server_create")
        self._h = h
        self.cigar_stride = cigar_stride or reference_cigar_stride(max_seq_len)

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().wfe_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, ascii: np.ndarray, pairs: np.ndarray, out=None) -> Request:
        """Queue a request; the arrays are kept alive by the returned Request."""
        n = len(pairs)
        pairs = np.ascontiguousarray(pairs, dtype=PAIR_DTYPE)
        if out is None:
            out = (np.zeros(n, np.int32), np.zeros((n, self.cigar_stride), np.int8), np.zeros(n, np.uint8))
        dist, cg, st = out
        t = C.c_uint64(0)
        _check(load().wfe_submit(self._h, _addr(ascii), ascii.nbytes, _addr(pairs), n, _addr(dist), _addr(cg),
                                 _addr(st), C.byref(t)), "wfe_submit")
        return Request(t.value, ascii, pairs, dist, cg, st)

    def poll(self, req: Request, timeout_us: int = -1) -> bool:
        """True when the request has finished (req.info filled); False on timeout."""
        info = RequestInfo()
        rc = load().wfe_poll(self._h, req.ticket, timeout_us, C.byref(info))
        if rc == ERR_TIMEOUT:
            return False
        _check(rc, "wfe_poll")
        req.info = {"submit_ns": info.submit_ns, "start_ns": info.start_ns, "done_ns": info.done_ns,
                    "pairs": info.pairs, "batches": info.batches}
        return True

    def poll_ticket(self, ticket: int, timeout_us: int = 0) -> int:
        """Raw wfe_poll status of a ticket."""
        return load().wfe_poll(self._h, ticket, timeout_us, None)

    def stats(self) -> dict:
        s = ServerStats()
        _check(load().wfe_server_get_stats(self._h, C.byref(s)), "wfe_server_get_stats")
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}


def pack_device(d_ascii, d_pairs, n: int, d_words, words_per_seq: int, stream=None) -> None:
    s = stream.cuda_stream if hasattr(stream, "cuda_stream") else (stream or 0)
    _check(load().wfe_pack_device(_addr(d_ascii), _addr(d_pairs), n, _addr(d_words), words_per_seq, s),
           "wfe_pack_device")


def cigar_from_history_device(d_ascii, d_pairs, n: int, max_len: int, d_dist, d_history, d_cigar,
                              cigar_stride: int, d_status, stream=None) -> None:
    s = stream.cuda_stream if hasattr(stream, "cuda_stream") else (stream or 0)
    _check(load().wfe_cigar_from_history_device(_addr(d_ascii), _addr(d_pairs), n, max_len, _addr(d_dist),
                                                _addr(d_history), _addr(d_cigar), cigar_stride,
                                                _addr(d_status), s), "wfe_cigar_from_history_device")


def align_device_noalloc(d_ascii, d_pairs, n: int, max_len: int, max_distance: int, d_dist, d_cigar,
                         cigar_stride: int, d_status, stream=None) -> None:
    """wfe_align_device_noalloc: device buffers in and out, no allocation and
    no context, for callers that cannot allocate device memory; scratch is the
    library's fixed 16 MiB device array shared by every call (calls must not
    overlap on the GPU)."""
    s = stream.cuda_stream if hasattr(stream, "cuda_stream") else (stream or 0)
    _check(load().wfe_align_device_noalloc(_addr(d_ascii), _addr(d_pairs), n, max_len, max_distance,
                                           _addr(d_dist), _addr(d_cigar), cigar_stride, _addr(d_status), s),
           "wfe_align_device_noalloc")


def format_cigar(cigar: np.ndarray, compat: bool = False) -> str:
    cg = np.ascontiguousarray(cigar, dtype=np.int8)
    n = load().wfe_format_cigar(cg.ctypes.data, cg.size, None, 0, int(compat))
    buf = C.create_string_buffer(n + 1)
    load().wfe_format_cigar(cg.ctypes.data, cg.size, buf, n + 1, int(compat))
    return buf.value.decode()


def check_cigar(pattern: bytes, text: bytes, cigar: np.ndarray):
    cg = np.ascontiguousarray(cigar, dtype=np.int8)
    score = C.c_int32(0)
    ok = load().wfe_check_cigar(pattern, len(pattern), text, len(text), cg.ctypes.data, cg.size,
                                C.byref(score))
    return bool(ok), score.value

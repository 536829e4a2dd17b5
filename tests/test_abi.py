"""The C ABI library without a GPU: it loads, exports every entry point that
include/*.h declares, and its host utilities agree with the oracle."""
import os
import re

import numpy as np
import pytest

import oracle as O
import wfe

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_vectors.npz")


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(wfe_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_function():
    lib = wfe.load()
    decl = declared_functions()
    assert "wfe_align" in decl and "wfe_create" in decl
    for name in decl:
        assert hasattr(lib, name), name
    assert set(decl) <= set(wfe.SYMBOLS) | set(decl)


def test_strerror():
    assert wfe.strerror(0) == "success"
    assert "memory" in wfe.strerror(wfe.ERR_OUT_OF_MEMORY)
    assert wfe.strerror(12345) == "unknown status"


def _no_gpu():
    try:
        import torch
        return not torch.cuda.is_available()
    except Exception:
        return True


@pytest.mark.skipif(not _no_gpu(), reason="checks the no-device path")
def test_create_without_device_fails_cleanly():
    with pytest.raises(wfe.WfeError) as e:
        wfe.Context(max_seq_len=150)
    assert e.value.code == wfe.ERR_NO_DEVICE
    with pytest.raises(wfe.WfeError) as e:
        wfe.Context(max_seq_len=150, long_scratch=(1 << 20, 1 << 20))
    assert e.value.code == wfe.ERR_NO_DEVICE


def test_create_rejects_bad_config():
    import ctypes as C
    cfg = wfe.Config(0, 0, 0, 0, 0, 0)
    h = C.c_void_p()
    assert wfe.load().wfe_create(C.byref(cfg), C.byref(h)) == wfe.ERR_INVALID_ARGUMENT
    assert wfe.load().wfe_create_with_scratch(C.byref(cfg), 1 << 20, 1 << 20, C.byref(h)) == wfe.ERR_INVALID_ARGUMENT


def test_format_and_check_match_oracle_on_golden():
    z = np.load(GOLDEN)
    a = z["ascii"].tobytes()
    for i, o in enumerate(z["offsets"]):
        if z["dist"][i] >= 64:
            continue
        cg = z["cigars"][i]
        assert wfe.format_cigar(cg, compat=True) == str(z["compat"][i])
        assert wfe.format_cigar(cg) == O.format_cigar(cg)
        p, t = a[o[0]:o[0] + o[1]], a[o[2]:o[2] + o[3]]
        ok, score = wfe.check_cigar(p, t, cg)
        assert ok == bool(z["ref_check"][i])
        if ok:
            assert score == z["dist"][i]


def test_format_examples():
    def enc(*items):
        out = []
        for it in items:
            if isinstance(it, int):
                while it > 0:
                    out.append(-min(it, 127))
                    it -= min(it, 127)
            else:
                out.append(ord(it))
        return np.array(out + [0], dtype=np.int8)

    cg = enc(20, "X", 129, "D", 3)
    assert wfe.format_cigar(cg) == "20M1X129M1D3M"
    # the reference's printer: the operation's character code as the M count,
    # and the last M run dropped (src/wavefront.cuh:161-181)
    assert wfe.format_cigar(cg, compat=True) == "88MX68MD"
    assert wfe.format_cigar(enc("I", "I", 5, "X", "X", "X")) == "2I5M3X"
    assert wfe.format_cigar(enc(254)) == "254M"
    assert wfe.format_cigar(np.zeros(4, np.int8)) == ""


def test_check_rejects_bad_cigars():
    p, t = b"ACGT", b"ACGT"
    good = np.array([-4, 0], np.int8)
    assert wfe.check_cigar(p, t, good) == (True, 0)
    assert not wfe.check_cigar(p, t, np.array([-3, 0], np.int8))[0]              # too short
    assert not wfe.check_cigar(p, t, np.array([-3, ord("X"), 0], np.int8))[0]    # X on a match
    assert not wfe.check_cigar(p, t, np.array([-5, 0], np.int8))[0]              # past the end
    assert not wfe.check_cigar(p, t, np.array([ord("Q"), 0], np.int8))[0]        # unknown letter


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the ABI structs have the C sizes and offsets."""
    import ctypes as C
    import subprocess
    src = tmp_path / "layout.c"
    checks = {
        "wfe_config": (wfe.Config, ["device", "max_seq_len", "batch_size", "max_distance", "cigar_stride", "flags"]),
        "wfe_stats": (wfe.Stats, ["pairs", "tier_entered", "tier_ms", "mapped_batches", "deferred_pairs",
                                  "deep_scratch_bytes"]),
        "wfe_server_config": (wfe.ServerConfig, ["memory_bytes", "nbuckets", "bucket_max_len", "first_tier",
                                                 "policy_flags"]),
        "wfe_request_info": (wfe.RequestInfo, ["submit_ns", "done_ns", "pairs", "batches"]),
        "wfe_server_stats": (wfe.ServerStats, ["split_requests", "max_in_flight", "lanes", "peak_memory"]),
        "wfe_pair_file": (wfe.PairFileC, ["ascii_bytes", "n", "longest", "pinned"]),
    }
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "wfe.h"', "int main(void) {"]
    for name, (_, fields) in checks.items():
        lines.append(f'printf("%zu\\n", sizeof({name}));')
        lines += [f'printf("%zu\\n", offsetof({name}, {f}));' for f in fields]
    lines.append("return 0; }")
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True,
                                          check=True).stdout.split()]
    want = []
    for name, (cls, fields) in checks.items():
        want.append(C.sizeof(cls))
        want += [getattr(cls, f).offset for f in fields]
    assert got == want


def test_constants_match_the_header():
    """Every WFE_ status, pair status, flag and limit of include/wfe.h has the
    same value in the Python mirror."""
    txt = open(os.path.join(ROOT, "include", "wfe.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    found = {}
    for name, val in re.findall(r"#define\s+WFE_([A-Z0-9_]+)\s+(\(?[0-9]+u?(?:\s*<<\s*[0-9]+)?\)?)", txt):
        found[name] = eval(val.replace("u", ""))
    for name, val in re.findall(r"\bWFE_((?:ERR|PAIR)_[A-Z_]+|OK)\s*=\s*([0-9]+)", txt):
        found[name] = int(val)
    skip = {"H", "ABI_VERSION", "MAX_BUCKETS"}
    checked = 0
    for name, val in found.items():
        if name in skip:
            continue
        assert hasattr(wfe, name), name
        assert getattr(wfe, name) == val, name
        checked += 1
    assert checked >= 22 and found["FLAG_PAGEABLE_IN_PLACE"] == 8


def test_align_rejects_unusable_output_arrays():
    """The Python binding checks the output arrays before the library writes
    through their pointers (no device needed: the check comes first)."""
    import types
    ctx = types.SimpleNamespace(cigar_stride=8, _h=None)
    ascii, pairs = wfe.pairs_from_list([(b"ACGT", b"ACGA")] * 3)
    good = (np.zeros(3, np.int32), np.zeros((3, 8), np.int8), np.zeros(3, np.uint8))
    bad_cases = [
        (np.zeros(3, np.int64), good[1], good[2]),              # wrong dtype
        (good[0], np.zeros((3, 16), np.int8)[:, ::2], good[2]),  # not contiguous
        (good[0], good[1], np.zeros(2, np.uint8)),              # too short
    ]
    ro = np.zeros(3, np.int32)
    ro.flags.writeable = False
    bad_cases.append((ro, good[1], good[2]))                    # read-only
    for out in bad_cases:
        with pytest.raises(ValueError):
            wfe.Context.align(ctx, ascii, pairs, out=out)

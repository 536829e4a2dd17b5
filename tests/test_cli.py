"""wfe.aligner, the reference's command line on libwfe."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
import wfe

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ALIGNER = os.path.join(ROOT, "ewfa-gpu_gb300", "bin", "wfe.aligner")
GEN = os.path.join(ROOT, "ewfa-gpu_gb300", "bin", "wfe.gen")


def _run(*args, check=False):
    return subprocess.run([ALIGNER, *map(str, args)], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                          check=check)


def _gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_gpu(), reason="checks the no-device path")
def test_no_device_message():
    r = _run("-f", "x", "-n", "1", "-l", "10")
    assert r.returncode == 1
    assert "No available CUDA devices detected." in r.stderr


def test_generator_tool_writes_reference_format(tmp_path):
    f = tmp_path / "g.seq"
    subprocess.run([GEN, str(f), "4", "30", "30", "0.1", "0.1", "9"], check=True)
    lines = f.read_text().splitlines()
    assert [l[0] for l in lines] == [">", "<"] * 4
    ascii, pairs = wfe.generate(4, 30, p_min=0.1, seed=9)
    assert lines[2][1:].encode() == ascii[pairs["p_off"][1]:pairs["p_off"][1] + pairs["p_len"][1]].tobytes()


def _expected(path, n, stride, compat=False, max_distance=0):
    text = open(path, "rb").read().split(b"\n")
    pairs = [(text[2 * i][1:], text[2 * i + 1][1:]) for i in range(n)]
    out = []
    for p, t in pairs:
        st, d, ops, _ = O.align(p, t, max_distance)
        if st != O.PAIR_OK:
            out.append("")
            continue
        _, cg, _ = O.cigar(p, t, d, ops, stride)
        out.append(O.format_cigar(cg, compat=compat))
    return out


def _printed(stdout):
    lines = [l for l in stdout.splitlines() if ":" in l and l.split(":")[0].isdigit()]
    return {int(l.split(":", 1)[0]): l.split(": ", 1)[1] if ": " in l else "" for l in lines}


@pytest.mark.gpu
def test_cli_prints_the_oracle_cigars(tmp_path):
    f = tmp_path / "in.seq"
    n = 3000
    wfe.generate_file(str(f), n, 150, p_min=0.05, seed=3)
    want = _expected(str(f), n, 152)
    r = _run("-f", f, "-n", n, "-l", 150, "-p", check=True)
    assert r.stdout.startswith("Using device")
    assert "Aligned executed. Wall time" in r.stdout
    got = _printed(r.stdout)
    assert [got[i] for i in range(n)] == want
    # several threads and batches: the same lines in the same order
    r2 = _run("-f", f, "-n", n, "-l", 150, "-b", 400, "-t", 3, "-p", check=True)
    got2 = _printed(r2.stdout)
    assert [got2[i] for i in range(n)] == want
    # without -p or --check the share is aligned in windows of two batches
    r3 = _run("-f", f, "-n", n, "-l", 150, "-b", 400, "-t", 2, check=True)
    assert "Aligned executed. Wall time" in r3.stdout and not _printed(r3.stdout)


@pytest.mark.gpu
def test_cli_compat_print_and_check(tmp_path):
    f = tmp_path / "in.seq"
    n = 1000
    wfe.generate_file(str(f), n, 100, p_min=0.02, p_max=0.3, seed=4)
    want = _expected(str(f), n, 100, compat=True, max_distance=63)
    r = _run("-f", f, "-n", n, "-l", 100, "-p", "--compat-print", "--max-distance", 63, "--check", check=True)
    got = _printed(r.stdout)
    assert [got[i] for i in range(n)] == want
    assert "Correct alignments:" in r.stderr


@pytest.mark.gpu
def test_cli_file_errors(tmp_path):
    bad = tmp_path / "bad.seq"
    bad.write_text(">ACGT\n>ACGT\n")
    r = _run("-f", bad, "-n", 1, "-l", 10)
    assert r.returncode == 1 and "Invalid sequence format" in r.stderr
    r = _run("-f", tmp_path / "missing.seq", "-n", 1, "-l", 10)
    assert r.returncode == 1
    r = _run("-n", 1, "-l", 10)
    assert r.returncode == 1 and "Options:" in r.stderr
    short = tmp_path / "short.seq"
    short.write_text(">ACGT\n<ACGA\n")
    r = _run("-f", short, "-n", 3, "-l", 10, "-p", check=True)
    got = _printed(r.stdout)
    assert got[0] == "3M1X" and got[1] == "" and got[2] == ""

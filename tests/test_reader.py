"""wfe_read_pair_file, the pair-file reader of the C ABI (no GPU)."""
import numpy as np
import pytest

import wfe


def _seqs(ascii, pairs):
    return [(ascii[q["p_off"]:q["p_off"] + q["p_len"]].tobytes(), ascii[q["t_off"]:q["t_off"] + q["t_len"]].tobytes())
            for q in pairs]


@pytest.mark.parametrize("threads", [1, 3, 8, 16])
def test_reads_generated_file(tmp_path, threads):
    f = tmp_path / "a.seq"
    wfe.generate_file(str(f), 20000, 100, 300, p_min=0.0, p_max=0.2, seed=6)
    ascii, pairs, longest = wfe.read_pair_file(str(f), nthreads=threads)
    ga, gp = wfe.generate(20000, 100, 300, p_min=0.0, p_max=0.2, seed=6)
    assert len(pairs) == 20000
    assert _seqs(ascii, pairs) == _seqs(ga, gp)
    assert longest == max(gp["p_len"].max(), gp["t_len"].max())


def test_limits_line_endings_and_tails(tmp_path):
    f = tmp_path / "b.seq"
    f.write_bytes(b">ACGT\r\n<ACGA\r\n>TT\n<T\n>GG")  # CRLF, LF, last line without '\n'
    ascii, pairs, _ = wfe.read_pair_file(str(f))
    assert _seqs(ascii, pairs) == [(b"ACGT", b"ACGA"), (b"TT", b"T"), (b"GG", b"")]
    ascii, pairs, _ = wfe.read_pair_file(str(f), max_pairs=2)
    assert len(pairs) == 2


def test_format_errors(tmp_path):
    f = tmp_path / "c.seq"
    f.write_bytes(b">ACGT\n>ACGT\n")
    with pytest.raises(wfe.WfeError) as e:
        wfe.read_pair_file(str(f))
    assert "Invalid sequence format on line 1" in str(e.value)
    with pytest.raises(wfe.WfeError):
        wfe.read_pair_file(str(tmp_path / "missing.seq"))
    empty = tmp_path / "d.seq"
    empty.write_bytes(b"")
    ascii, pairs, longest = wfe.read_pair_file(str(empty))
    assert len(pairs) == 0 and longest == 0

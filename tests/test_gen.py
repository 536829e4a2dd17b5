"""The synthetic workload generator (no GPU)."""
import numpy as np

import oracle as O
import wfe


def test_deterministic_and_rangeable():
    a1, p1 = wfe.generate(500, 150, p_min=0.05, seed=3)
    a2, p2 = wfe.generate(500, 150, p_min=0.05, seed=3, nthreads=1)
    np.testing.assert_array_equal(p1, p2)
    np.testing.assert_array_equal(a1, a2)
    # pairs [200, 300) generated on their own are the same pairs
    a3, p3 = wfe.generate(100, 150, p_min=0.05, seed=3, first=200)
    for j in range(100):
        i = 200 + j
        s1 = a1[p1["p_off"][i]:p1["p_off"][i] + p1["p_len"][i]]
        s3 = a3[p3["p_off"][j]:p3["p_off"][j] + p3["p_len"][j]]
        np.testing.assert_array_equal(s1, s3)


def test_shapes_and_error_rate():
    a, p = wfe.generate(4000, 150, p_min=0.05, seed=1)
    assert (p["t_len"] == 150).all()
    assert set(np.unique(a[: int(p["t_off"][-1] + p["t_len"][-1])])) <= set(b"ACGT")
    # expected edits 7.5 per pair; the edit distance is a little lower
    d = [O.levenshtein(a[p["p_off"][i]:p["p_off"][i] + p["p_len"][i]].tobytes(),
                       a[p["t_off"][i]:p["t_off"][i] + p["t_len"][i]].tobytes()) for i in range(400)]
    assert 5.5 < np.mean(d) < 8.5


def test_mixed_lengths_log_uniform():
    _, p = wfe.generate(20000, 100, 10000, p_min=0.01, p_max=0.15, seed=4)
    t = p["t_len"].astype(np.float64)
    assert t.min() >= 100 and t.max() <= 10000
    # log-uniform: the median is near sqrt(100 * 10000) = 1000
    assert 800 < np.median(t) < 1250


def test_file_format(tmp_path):
    f = tmp_path / "x.seq"
    wfe.generate_file(str(f), 5, 40, p_min=0.1, seed=2)
    lines = f.read_text().splitlines()
    assert len(lines) == 10
    assert all(l.startswith(">") for l in lines[0::2]) and all(l.startswith("<") for l in lines[1::2])
    a, p = wfe.generate(5, 40, p_min=0.1, seed=2)
    assert lines[1][1:].encode() == a[p["t_off"][0]:p["t_off"][0] + 40].tobytes()

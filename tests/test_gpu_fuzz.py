"""Randomised differential tests: libwfe against the CPU oracle over seeded
random configurations -- lengths from 0 to 1,200 bases, edit probabilities up
to 0.4, distance caps, CIGAR slots too small for some CIGARs, batch sizes,
length buckets with and without distance prediction, the CTA-per-pair tier
as the first tier of every pair (the bound pass, the target's cone and the
distance classes, or one launch without bounds), and every host and
device entry point (pageable staged, pageable in place, pinned in place,
device buffers, the reference reader's strided layout).  Integer work: every
distance, status and CIGAR byte must match."""
import numpy as np
import pytest

import wfe
from test_gpu_parity import _pinned, compare_with_oracle, torch_cuda

pytestmark = pytest.mark.gpu

MODES = ["pageable", "pageable_in_place", "pinned", "device", "strided"]


def random_case(k):
    rng = np.random.default_rng(7000 + k)
    n = int(rng.integers(300, 3000))
    len_min = int(rng.choice([0, 1, 8, 40, 150, 300]))
    len_max = int(min(1200, max(len_min, 1) * int(rng.choice([1, 2, 4]))))
    p_lo, p_hi = sorted(float(x) for x in rng.uniform(0.0, 0.4, 2))
    ascii, pairs = wfe.generate(n, len_min, len_max, p_min=p_lo, p_max=p_hi, seed=7000 + k)
    longest = int(max(pairs["p_len"].max(), pairs["t_len"].max(), 1))
    return rng, ascii, pairs, longest, dict(
        n=n, lens=(len_min, len_max), p=(round(p_lo, 3), round(p_hi, 3)),
        max_len=longest + int(rng.integers(0, 40)),
        max_distance=int(rng.choice([0, 0, 3, 10, 25, 63])),
        batch=int(rng.choice([37, 256, 1000, 100000])),
        stride=int(rng.choice([8, 40, wfe.reference_cigar_stride(longest), 2 * longest + 8])),
        mode=MODES[k % len(MODES)],
        policy=str(rng.choice(["default", "buckets", "predict", "tier5", "tier5_nobound"])))


def run_case(ascii, pairs, c):
    flags = wfe.FLAG_PAGEABLE_IN_PLACE if c["mode"] == "pageable_in_place" else 0
    n, S = len(pairs), c["stride"]
    with wfe.Context(max_seq_len=c["max_len"], batch_size=c["batch"], max_distance=c["max_distance"],
                     cigar_stride=S, flags=flags) as ctx:
        if c["policy"] in ("tier5", "tier5_nobound"):
            ctx.set_policy([c["max_len"]], [5], bound=c["policy"] == "tier5")
        elif c["policy"] != "default":
            cuts = sorted({max(1, c["max_len"] // 4), max(1, c["max_len"] // 2), c["max_len"]})
            ctx.set_policy(cuts, predict=c["policy"] == "predict")
        if c["mode"] in ("pageable", "pageable_in_place"):
            return ctx.align(ascii, pairs)
        if c["mode"] == "pinned":
            return ctx.align(_pinned(ascii), _pinned(pairs))
        if c["mode"] == "strided":
            slot = (c["max_len"] + 15) // 16 * 16
            buf = np.zeros(2 * slot * n, np.uint8)
            for i, q in enumerate(pairs):
                buf[2 * i * slot: 2 * i * slot + q["p_len"]] = ascii[q["p_off"]: q["p_off"] + q["p_len"]]
                buf[(2 * i + 1) * slot: (2 * i + 1) * slot + q["t_len"]] = ascii[q["t_off"]: q["t_off"] + q["t_len"]]
            return ctx.align_strided(buf, slot, pairs["p_len"].copy(), pairs["t_len"].copy())
        torch = torch_cuda()
        d_ascii = torch.from_numpy(ascii).cuda()
        d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
        d_dist = torch.zeros(n, dtype=torch.int32, device="cuda")
        d_cg = torch.zeros(max(1, n * S), dtype=torch.int8, device="cuda")
        d_st = torch.zeros(n, dtype=torch.uint8, device="cuda")
        ctx.align_device(d_ascii, d_pairs, n, c["max_len"], d_dist, d_cg, d_st)
        torch.cuda.synchronize()
        return d_dist.cpu().numpy(), d_cg.cpu().numpy()[: n * S].reshape(n, S), d_st.cpu().numpy()


@pytest.mark.parametrize("k", range(60))
def test_random_configuration_matches_oracle(k):
    torch_cuda()
    _, ascii, pairs, _, c = random_case(k)
    dist, cg, st = run_case(ascii, pairs, c)
    compare_with_oracle(ascii, pairs, c["stride"], dist, cg, st, max_distance=c["max_distance"])

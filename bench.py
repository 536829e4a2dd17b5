#!/usr/bin/env python
"""Benchmark of the alignment path on GB300: alignments/s on the short-read
workload (1,000,000 pairs of 150 bases, per-position edit probability 0.05,
batches of 100,000 pairs, synthetic data from a fixed seed).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step aligns one batch of 100,000 pairs: distances and full CIGARs.
  value  device-resident throughput: the batch's ASCII and descriptors are
         already in HBM, results stay in HBM; timed with CUDA events on the
         launching stream.  Steps cycle over the 10 batches of the workload
         (300 MB of ASCII + 152 MB of CIGAR slots > the 129 MB L2); the timed
         steps are one wfe_align_device call over the batches repeated in HBM.
  e2e    the same workload through the host-buffer C call wfe_align with
         pinned host buffers: every batch's inputs come from pinned host memory
         and its distances, status and CIGARs go back to pinned host memory
         inside the timed region.  The library reads and writes pinned buffers
         in place over the CPU-GPU link (NVLink-C2C on GB300); the bytes that
         cross it per step are reported.  The passes over the workload are one
         call over its descriptors repeated in pinned memory; calls of the
         workload's own size are timed beside it.
--impl reference times the CPU restatement of the reference's algorithm
(oracle/, the reference has no CPU aligner of its own and its sources are
not on this machine) on every host core.

One process per GPU (torchrun for N > 1): every rank aligns its own
1,000,000-pair shard (weak scaling, no collective on the data path); rank 0
prints one JSON line with the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ewfa-gpu_gb300"))

import numpy as np  # noqa: E402

import wfe  # noqa: E402

METRIC = "alignments/sec"
# fixed-length throughput workloads: pairs, batch, length, edit probability,
# seed, committed ncu summary of the dominant kernel
THROUGHPUT = {
    "short": (1_000_000, 100_000, 150, 0.05, 2, "tier0_short_reads.txt"),
    "long": (200_000, 20_000, 1000, 0.10, 3, "tier5_long_reads.txt"),
}
E2E_REPEATS = 8  # passes over the workload in one timed wfe_align call, at most (pinned host memory)


def select_workload(name: str) -> None:
    """Set the module's workload constants (the short-read workload unless
    another is asked for)."""
    global PAIRS, BATCH, LENGTH, EDIT_P, SEED, PROFILE, WORKLOAD, CIGAR_STRIDE, MAX_SEQ_LEN
    PAIRS, BATCH, LENGTH, EDIT_P, SEED, PROFILE = THROUGHPUT[name]
    WORKLOAD = (f"{name} reads: {PAIRS:,} pairs x {LENGTH} bases, edit probability {EDIT_P}, "
                f"batches of {BATCH:,}; distance + full CIGAR per pair")
    CIGAR_STRIDE = wfe.reference_cigar_stride(LENGTH)   # the reference's cigar_max_len for -l LENGTH
    MAX_SEQ_LEN = 2 * LENGTH                             # the reference reader's slot holds 2*l bases


select_workload("short")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="short workload: skip the long, mixed and serve runs that the line reports beside it")
    ap.add_argument("--workload", choices=["short", "long", "mixed", "serve"], default="short",
                    help="short: the short-read throughput workload (the metric's configuration); "
                         "long: 200,000 pairs of 1,000 bases at edit probability 0.10; "
                         "mixed: uneven lengths, plain fixed-shape launches vs length buckets; "
                         "serve: Poisson request stream, the request server vs one call per request")
    ap.add_argument("--requests", type=int, default=0, help="serve workload: number of requests (default 1,000)")
    ap.add_argument("--rates", default="", help="serve workload: loads as fractions of the measured peak, "
                                                 "comma-separated (default 0.1,0.25,0.5,0.75,0.9,1.0,1.2)")
    ap.add_argument("--pairs", type=int, default=0, help="mixed workload: number of pairs (default 2,000,000)")
    ap.add_argument("--profile-batch", type=int, default=0,
                    help="profiling case: run the --profile-kernel kernels twice over ONE batch of this "
                         "many pairs of the workload (a warm-up, then the launch to capture), and exit")
    ap.add_argument("--profile-kernel", choices=["tier", "aux"], default="tier")
    ap.add_argument("--link", action="store_true",
                    help="measure the CPU-GPU link: DMA copies between pinned host memory and HBM, and exit")
    ap.add_argument("--profile-first-tier", type=int, default=-1)
    ap.add_argument("--profile-case", choices=["workload"] + sorted(PROFILE_CASES), default="workload",
                    help="profiling case: the --workload's pairs, or pairs for the CTA-per-pair tiers: "
                         "deep (5,000-7,000 bases, p 0.06-0.10, distances of hundreds: tier 5's regime in the "
                         "mixed workload), far (4,000-5,000 bases, p 0.70-0.80, distances around 2,000 and "
                         "beyond: tier 6's)")
    ap.add_argument("--profile-host-inputs", action="store_true",
                    help="profiling case: the ASCII and descriptors in pinned host memory, read by the "
                         "kernels in place over the CPU-GPU link (as wfe_align does with pinned buffers)")
    return ap.parse_args()


def run_link() -> int:
    """Bandwidth of the CPU-GPU link (NVLink-C2C on GB300): DMA copies of
    32 MiB - 1 GiB between pinned host memory and HBM, each direction alone
    (best of 5, CUDA events) and both at once."""
    import torch
    torch.cuda.set_device(0)
    res = {}
    for mb in (32, 256, 1024):
        n = mb << 20
        h = torch.empty(n, dtype=torch.uint8, pin_memory=True)
        h.fill_(1)
        d = torch.empty(n, dtype=torch.uint8, device="cuda")
        s = torch.cuda.Stream()
        for direction in ("h2d", "d2h"):
            best = 1e9
            for _ in range(5):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                with torch.cuda.stream(s):
                    if direction == "h2d":
                        d.copy_(h, non_blocking=True)
                    else:
                        h.copy_(d, non_blocking=True)
                e1.record(s)
                torch.cuda.synchronize()
                best = min(best, e0.elapsed_time(e1))
            res[f"{direction}_{mb}MiB_GBs"] = round(n / best / 1e6, 1)
    n = 256 << 20
    h1, h2 = (torch.empty(n, dtype=torch.uint8, pin_memory=True) for _ in range(2))
    d1, d2 = (torch.empty(n, dtype=torch.uint8, device="cuda") for _ in range(2))
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(s1):
        d1.copy_(h1, non_blocking=True)
    with torch.cuda.stream(s2):
        h2.copy_(d2, non_blocking=True)
    torch.cuda.synchronize()
    res["both_directions_256MiB_each_GBs"] = round(2 * n / (time.perf_counter() - t0) / 1e9, 1)
    print(json.dumps({"link": res}))
    return 0


def histories_from_cigars(cg: np.ndarray) -> np.ndarray:
    """The reference's 128-bit history of each pair (two uint64 words): the
    operation of score step d (X = 2, I = 1, D = 3) in 2-bit field d - 1,
    fields 0-31 in the first word (src/kernels.cu:154-171)."""
    code = np.zeros(256, np.uint64)
    code[ord("X")], code[ord("I")], code[ord("D")] = 2, 1, 3
    b = cg.view(np.uint8)
    term = np.cumsum(b == 0, axis=1) > 0
    op = np.where(term | (cg <= 0), 0, code[b])
    idx = np.cumsum(op > 0, axis=1) - 1
    words = np.zeros((len(cg), 2), np.uint64)
    for w in range(2):
        sel = (op > 0) & (idx // 32 == w)
        sh = (2 * (idx % 32)).astype(np.uint64)
        words[:, w] = np.where(sel, op << sh, 0).sum(axis=1, dtype=np.uint64)
    return words


# Profiling cases for the CTA-per-pair tiers: lengths (log-uniform), edit
# probability (uniform), seed, max_seq_len, CIGAR stride, and the slab bounds
# of tiers 5 and 6 (a few GB on the device in all).
PROFILE_CASES = {
    "deep": (5000, 7000, 0.06, 0.10, 44, 7400, 4096, (2 << 30, 1 << 30)),
    "far": (4000, 5000, 0.70, 0.80, 46, 5200, 12000, (1 << 30, 2 << 30)),
}


def run_profile_case(args) -> int:
    """Profiling cases: every kernel runs twice over one batch of n pairs of
    the workload (the first launch warms up, ncu captures the second):
      tier     the alignment chain from its first tier (--profile-first-tier)
      aux      wfe_pack_device, the distance-prediction and routing kernels of
               a bucketed batch, and the CIGAR-from-history kernel fed the
               histories of this workload's alignments."""
    import torch
    torch.cuda.set_device(0)
    n = args.profile_batch
    max_seq_len, stride, scratch = MAX_SEQ_LEN, CIGAR_STRIDE, None
    if args.profile_case == "workload":
        ascii, pairs = wfe.generate(n, LENGTH, p_min=EDIT_P, seed=SEED)
    else:
        lmin, lmax, pmin, pmax, seed, max_seq_len, stride, scratch = PROFILE_CASES[args.profile_case]
        ascii, pairs = wfe.generate(n, lmin, lmax, p_min=pmin, p_max=pmax, seed=seed)
    if args.profile_host_inputs:
        d_ascii = torch.from_numpy(ascii).pin_memory()
        d_pairs = torch.from_numpy(pairs.view(np.uint8)).pin_memory()
    else:
        d_ascii = torch.from_numpy(ascii).cuda()
        d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
    d_dist = torch.zeros(n, dtype=torch.int32, device="cuda")
    d_cigar = torch.zeros(n * stride, dtype=torch.int8, device="cuda")
    d_status = torch.zeros(n, dtype=torch.uint8, device="cuda")
    out = {"profile_batch": n, "kernel": args.profile_kernel, "case": args.profile_case,
           "host_inputs": bool(args.profile_host_inputs)}
    with wfe.Context(max_seq_len=max_seq_len, batch_size=n, cigar_stride=stride, long_scratch=scratch) as ctx:
        if args.profile_kernel == "tier":
            if args.profile_first_tier >= 0:
                ctx.set_policy([max_seq_len], [args.profile_first_tier])
            for _ in range(2):
                ctx.align_device(d_ascii, d_pairs, n, max_seq_len, d_dist, d_cigar, d_status)
                torch.cuda.synchronize()
            out["tier_launches"] = ctx.stats()["tier_launches"][:7]
            out["tier_passed"] = ctx.stats()["tier_passed"][:7]
            dist = d_dist.cpu().numpy().astype(np.float64)
            out["distance"] = {"mean": float(dist.mean()), "max": float(dist.max()),
                               "cells_per_pair": float(np.mean(dist * dist + 2 * dist))}
        else:
            if args.profile_case != "workload":
                raise SystemExit("--profile-kernel aux runs on the --workload's pairs")
            wps = (MAX_SEQ_LEN + 15) // 16
            d_words = torch.zeros(2 * n * wps, dtype=torch.int32, device="cuda")
            for _ in range(2):
                wfe.pack_device(d_ascii, d_pairs, n, d_words, wps)
            ctx.set_policy([LENGTH // 2, MAX_SEQ_LEN], [0, 0], predict=True)
            for _ in range(2):
                ctx.align_device(d_ascii, d_pairs, n, MAX_SEQ_LEN, d_dist, d_cigar, d_status)
            torch.cuda.synchronize()
            cg = d_cigar.view(n, CIGAR_STRIDE).cpu().numpy()
            d_hist = torch.from_numpy(histories_from_cigars(cg).view(np.int64).reshape(-1)).cuda()
            d_cg2 = torch.zeros_like(d_cigar)
            d_st2 = torch.zeros_like(d_status)
            for _ in range(2):
                wfe.cigar_from_history_device(d_ascii, d_pairs, n, MAX_SEQ_LEN, d_dist, d_hist, d_cg2,
                                              CIGAR_STRIDE, d_st2)
            torch.cuda.synchronize()
            out["history_cigars_equal"] = bool(torch.equal(d_cg2, d_cigar))
    mb = (len(ascii) + n * (stride + 29)) / 2**20
    out.update({"device_MiB": round(mb, 1), "status_ok": bool((d_status.cpu().numpy() == 0).all())})
    print(json.dumps(out))
    return 0


MIXED_PAIRS, MIXED_LMIN, MIXED_LMAX, MIXED_PMIN, MIXED_PMAX, MIXED_SEED = 2_000_000, 100, 10_000, 0.01, 0.15, 4
MIXED_BUCKETS = [256, 512, 1024, 2048, 4096, 11_000]


def run_mixed(args) -> int:
    """Uneven sizes: lengths log-uniform in [100, 10,000], edit probability
    uniform in [0.01, 0.15].  The same device-resident pairs are aligned
    (1) with the plain fixed-shape launches: one launch shape for every pair,
        sized for the longest sequence (no length buckets, and the CTA-per-pair
        tier as one launch: no distance bounds, no distance classes), and
    (2) with length buckets: pairs sorted by length on the device, each
        bucket aligned with shapes sized to it, first tiers chosen by the
        autotuner on a sample, and
    (3) as (2) with distance prediction: every pair starts at the tier its
        128-base prefix distance, extrapolated to its length, calls for,
    in batches of 100,000; all must give the same distances and CIGARs."""
    import torch
    torch.cuda.set_device(0)
    n = args.pairs or MIXED_PAIRS
    ascii, pairs = wfe.generate(n, MIXED_LMIN, MIXED_LMAX, p_min=MIXED_PMIN, p_max=MIXED_PMAX, seed=MIXED_SEED)
    max_len = int(max(pairs["p_len"].max(), pairs["t_len"].max()))
    max_seq = MIXED_BUCKETS[-1]
    assert max_len <= max_seq
    stride = 4096
    d_ascii = torch.from_numpy(ascii).cuda()
    d_pairs = torch.from_numpy(pairs.view(np.uint8)).cuda()
    outs = {}
    res = {}
    cache = os.path.join(tempfile.gettempdir(), "wfe_autotune.jsonl")
    modes = ("plain", "bucketed", "predicted")
    for mode in modes:
        d_dist = torch.zeros(n, dtype=torch.int32, device="cuda")
        d_cg = torch.zeros(n * stride, dtype=torch.int8, device="cuda")
        d_st = torch.full((n,), 255, dtype=torch.uint8, device="cuda")  # 255: never written
        with wfe.Context(max_seq_len=max_seq, batch_size=BATCH, cigar_stride=stride,
                         flags=wfe.FLAG_KERNEL_TIMING) as ctx:
            tiers = None
            t_tune = 0.0
            if mode == "plain":
                ctx.set_policy([max_seq], bound=False)
            else:
                t0 = time.perf_counter()
                tiers = ctx.autotune(d_ascii, d_pairs, n, MIXED_BUCKETS, cache, predict=mode == "predicted")
                t_tune = time.perf_counter() - t0
            s = torch.cuda.Stream()
            ctx.align_device(d_ascii, d_pairs, min(n, BATCH), max_seq, d_dist, d_cg, d_st, s)  # warm-up
            torch.cuda.synchronize()
            ctx.reset_stats()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            ctx.align_device(d_ascii, d_pairs, n, max_seq, d_dist, d_cg, d_st, s)
            e1.record(s)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            st = ctx.stats()
            res[mode] = {"seconds": ms / 1e3, "alignments_per_s": n / (ms / 1e3), "first_tiers": tiers,
                         "tune_seconds": round(t_tune, 3), "kernel_launches": st["kernel_launches"],
                         "tier_launches": st["tier_launches"][:7], "tier_passed": st["tier_passed"][:7],
                         "chain_ms_by_first_tier": [round(x, 2) for x in st["tier_ms"][:7]]}
        outs[mode] = (d_dist.cpu().numpy(), d_st.cpu().numpy(), d_cg)
    same_dist = all(np.array_equal(outs["plain"][0], outs[m][0]) for m in modes)
    same_status = all(np.array_equal(outs["plain"][1], outs[m][1]) for m in modes)
    same_status = same_status and all(torch.equal(outs["plain"][2], outs[m][2]) for m in modes)  # CIGAR slots
    ok_status = all(bool((outs[m][1] == 0).all()) for m in modes)
    dist = outs["plain"][0]
    line = {"metric": "alignments/sec", "workload": "mixed", "pairs": n, "unit": "alignments/s",
            "config": {"lengths": f"log-uniform [{MIXED_LMIN}, {MIXED_LMAX}]",
                       "edit_prob": f"uniform [{MIXED_PMIN}, {MIXED_PMAX}]", "seed": MIXED_SEED, "batch": BATCH,
                       "buckets": MIXED_BUCKETS, "cigar_stride": stride},
            **res,
            "speedup": {m: res["plain"]["seconds"] / res[m]["seconds"] for m in modes[1:]},
            "gcups": {m: n * float(np.mean(pairs["p_len"].astype(np.float64) * pairs["t_len"])) /
                      res[m]["seconds"] / 1e9 for m in modes},
            "identical_results": same_dist and same_status, "all_ok": ok_status,
            "distance": {"mean": float(dist.mean()), "max": int(dist.max())}}
    b_dist, b_st, b_cg = outs["bucketed"]
    line["parity"] = oracle_sample_parity(ascii, pairs, (b_dist, b_cg, b_st), stride, MIXED_SEED)
    del outs
    line["ref_cuda"] = reference_on_subset(ascii, pairs, b_dist, b_st, b_cg, MIXED_BUCKETS, stride, MIXED_SEED)
    print(json.dumps(line))
    good = same_dist and same_status and ok_status and line["parity"]["mismatches"] == 0
    return 0 if good else 1


ORACLE_SAMPLE = 20_000      # pairs of the mixed and served workloads checked against the CPU oracle
REF_SUBSET = 100_000        # pairs of the reference's search range aligned by its own kernels
REF_CLASSES = [256, 512, 1024, 2048, 4096, 11_000]  # length classes, one reference run each


def oracle_sample_parity(ascii, pairs, got, stride: int, seed: int) -> dict:
    """Distances, statuses and CIGARs of a seeded sample of ORACLE_SAMPLE
    pairs against the CPU restatement of the reference (oracle/).  got =
    (dist, cigar slots -- numpy or a device tensor of n * stride bytes --,
    status)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build(ref=False)
    dist, cg, st = got
    n = len(pairs)
    idx = np.sort(np.random.default_rng(seed).choice(n, min(ORACLE_SAMPLE, n), replace=False))
    if hasattr(cg, "view") and not isinstance(cg, np.ndarray):
        import torch
        rows = cg.view(n, stride).index_select(0, torch.from_numpy(idx).to(cg.device)).cpu().numpy()
    else:
        rows = np.asarray(cg).reshape(n, stride)[idx]
    sub = pairs[idx]
    od, ocg, ost, _ = oracle.align_batch(ascii, sub["p_off"], sub["p_len"], sub["t_off"], sub["t_len"], stride,
                                         nthreads=os.cpu_count() or 1)
    rec = parity((np.asarray(dist)[idx], rows, np.asarray(st)[idx]), (od, ocg, ost))
    rec["sample"] = f"{len(idx):,} seeded pairs of {n:,}"
    return rec


def reference_on_subset(ascii, pairs, dist, status, cg, buckets, stride: int, seed: int) -> dict | None:
    """The reference's own CUDA kernels (sm_100 cubin) on the pairs of a
    workload that lie in its search range, distance <= 63
    (src/wavefront.cuh:462-466): a seeded sample of REF_SUBSET of them, run
    in length classes (one -l per class, slots of the class's longest
    sequence: the reference has one slot size per run), its batch loop timed
    with allocations outside the clock (steady), best of 3; the classes'
    times add up.  This build aligns the same pairs through wfe_align with
    pinned host buffers (length buckets and first tiers by the autotuner),
    best of 3.  The reference's CIGARs are compared with this build's."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import torch
    try:
        oracle.build(ref=False)
    except Exception:
        return None
    if not oracle.ref_cuda_available():
        return None
    n = len(pairs)
    inside = np.flatnonzero((np.asarray(status) == 0) & (np.asarray(dist) <= 63))
    idx = np.sort(np.random.default_rng(seed + 1).choice(inside, min(REF_SUBSET, len(inside)), replace=False))
    sub = pairs[idx]
    # this build's CIGARs of the sample
    if hasattr(cg, "view") and not isinstance(cg, np.ndarray):
        ours = cg.view(n, stride).index_select(0, torch.from_numpy(idx).to(cg.device)).cpu().numpy()
    else:
        ours = np.asarray(cg).reshape(n, stride)[idx]
    longest = np.maximum(sub["p_len"], sub["t_len"]).astype(np.int64)
    ref_s, mismatches, classes = 0.0, 0, []
    with tempfile.TemporaryDirectory() as tmp:
        lo = 0
        for hi in REF_CLASSES:
            sel = np.flatnonzero((longest > lo) & (longest <= hi))
            lo = hi
            if len(sel) == 0:
                continue
            slot = (int(longest[sel].max()) + 1) // 2  # the reader's -l: slots of 2 * l bases
            dump = os.path.join(tmp, f"cigars_{hi}.bin")
            rec = oracle.ref_cuda_run_pairs(ascii, sub[sel], slot, batch=BATCH, threads=1, reps=3, steady=True,
                                            dump=dump)
            ref_s += rec["best_wall_s"]
            cml = slot + (4 - slot % 4)
            rc = np.fromfile(dump, np.int8).reshape(len(sel), cml)
            w = min(cml, stride)
            mine = ours[sel, :w]
            lr, lm = cigar_lengths(rc[:, :w]), cigar_lengths(mine)
            upto = np.arange(w)[None, :] <= lr[:, None]
            same = (lr == lm) & np.all(np.where(upto, rc[:, :w], 0) == np.where(upto, mine, 0), axis=1)
            mismatches += int((~same).sum())
            classes.append({"max_len": hi, "pairs": int(len(sel)), "l": slot, "ref_s": rec["best_wall_s"]})
    # this build on the same pairs: a compact copy of their sequences in pinned memory
    h_ascii, h_pairs = compact_pairs(ascii, sub)
    hp_ascii = torch.empty(len(h_ascii), dtype=torch.uint8, pin_memory=True).numpy()
    hp_ascii[:] = h_ascii
    hp_pairs = torch.empty(len(sub) * wfe.PAIR_DTYPE.itemsize, dtype=torch.uint8,
                           pin_memory=True).numpy().view(wfe.PAIR_DTYPE)
    hp_pairs[:] = h_pairs
    m = len(sub)
    outs = (torch.empty(m, dtype=torch.int32, pin_memory=True).numpy(),
            torch.empty(m * stride, dtype=torch.int8, pin_memory=True).numpy().reshape(m, stride),
            torch.empty(m, dtype=torch.uint8, pin_memory=True).numpy())
    max_seq = int(longest.max())
    bk = [b for b in buckets if b < max_seq] + [max_seq]
    cache = os.path.join(tempfile.gettempdir(), "wfe_autotune.jsonl")
    with wfe.Context(max_seq_len=max_seq, batch_size=BATCH, cigar_stride=stride) as ctx:
        d_a = torch.from_numpy(h_ascii).cuda()
        d_p = torch.from_numpy(h_pairs.view(np.uint8)).cuda()
        tiers = ctx.autotune(d_a, d_p, m, bk, cache)
        del d_a, d_p
        ctx.align(hp_ascii, hp_pairs, out=outs)  # warm-up
        best = 1e30
        for _ in range(3):
            t0 = time.perf_counter()
            ctx.align(hp_ascii, hp_pairs, out=outs)
            best = min(best, time.perf_counter() - t0)
    same_as_device = bool(np.array_equal(outs[0], np.asarray(dist)[idx]))
    return {"subset": "pairs at distance <= 63 (the reference's search range), a seeded sample",
            "pairs": int(m), "of_pairs_in_range": int(len(inside)), "of_pairs": int(n),
            "ref_steady": {"value": m / ref_s, "seconds": ref_s, "classes": classes,
                           "region": "batch loop per class, allocations outside the clock, best of 3"},
            "e2e": {"value": m / best, "seconds": best, "first_tiers": tiers,
                    "transfer": "wfe_align, pinned host buffers read and written in place"},
            "e2e_over_ref_steady": (m / best) / (m / ref_s),
            "cigars_identical_to_reference": mismatches == 0, "cigar_mismatches": mismatches,
            "same_as_device_run": same_as_device}


def compact_pairs(ascii: np.ndarray, sub: np.ndarray):
    """The sequences of `sub` copied one after another (pattern, text) into
    a new buffer, with descriptors into it."""
    lens = np.stack([sub["p_len"], sub["t_len"]], axis=1).reshape(-1).astype(np.int64)
    offs = np.stack([sub["p_off"], sub["t_off"]], axis=1).reshape(-1).astype(np.int64)
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]])
    total = int(lens.sum())
    out = np.zeros(total + 64, np.uint8)
    for o, st, ln in zip(offs.tolist(), starts.tolist(), lens.tolist()):
        out[st:st + ln] = ascii[o:o + ln]
    desc = np.zeros(len(sub), wfe.PAIR_DTYPE)
    desc["p_off"], desc["t_off"] = starts[0::2], starts[1::2]
    desc["p_len"], desc["t_len"] = sub["p_len"], sub["t_len"]
    return out, desc


SERVE_REQUESTS, SERVE_MAX_PAIRS, SERVE_LMIN, SERVE_LMAX, SERVE_PMIN, SERVE_PMAX, SERVE_SEED = \
    1000, 4096, 100, 5000, 0.01, 0.10, 7
SERVE_BUCKETS = [256, 512, 1024, 2048, SERVE_LMAX]
SERVE_RATES = [0.1, 0.25, 0.5, 0.75, 0.9, 1.0, 1.2]


def run_serve(args) -> int:
    """Served stream: requests of 1-4,096 pairs (log-uniform), lengths
    log-uniform in [100, 5,000], edit probability uniform in [0.01, 0.10],
    arriving as a Poisson stream at 10 %-120 % of the server's measured peak
    throughput.  For each rate the same arrivals go (1) to the request
    server (continuous batching over 4 streams, device-memory admission) and
    (2) to the plain form, one blocking wfe_align call per request in
    arrival order.  Latency = completion - scheduled arrival.  Both forms use
    the same length buckets and first tiers (chosen by the autotuner on a
    sample) and must give identical results."""
    import threading
    import torch
    torch.cuda.set_device(0)
    rng = np.random.default_rng(SERVE_SEED)
    nreq = args.requests or SERVE_REQUESTS
    sizes = np.floor(np.exp(rng.uniform(0, np.log(SERVE_MAX_PAIRS + 1), nreq))).astype(np.int64)
    sizes = sizes.clip(1, SERVE_MAX_PAIRS)
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    total = int(sizes.sum())
    ascii, pairs = wfe.generate(total, SERVE_LMIN, SERVE_LMAX, p_min=SERVE_PMIN, p_max=SERVE_PMAX, seed=SERVE_SEED)
    max_seq = int(max(pairs["p_len"].max(), pairs["t_len"].max()))
    max_seq = max(max_seq, SERVE_LMAX)
    stride = wfe.reference_cigar_stride(SERVE_LMAX)
    h_ascii = torch.empty(len(ascii), dtype=torch.uint8, pin_memory=True).numpy()
    h_ascii[:] = ascii
    reqs = [pairs[s:s + k] for s, k in zip(starts, sizes)]

    # first tiers per length bucket, measured on a sample
    ns = min(total, 200_000)
    d_ascii = torch.from_numpy(ascii).cuda()
    d_pairs = torch.from_numpy(pairs[:ns].view(np.uint8)).cuda()
    buckets = SERVE_BUCKETS[:-1] + [max_seq]
    with wfe.Context(max_seq_len=max_seq, batch_size=SERVE_MAX_PAIRS * 4, cigar_stride=stride) as c:
        tiers = c.autotune(d_ascii, d_pairs, ns, buckets)
    del d_ascii, d_pairs

    outs = {m: (np.zeros(total, np.int32), np.zeros((total, stride), np.int8), np.zeros(total, np.uint8))
            for m in ("served", "plain")}

    def views(m, i):
        d, c, st = outs[m]
        s, k = starts[i], sizes[i]
        return d[s:s + k], c[s:s + k], st[s:s + k]

    srv = wfe.Server(max_seq_len=max_seq, cigar_stride=stride, lanes=4, memory_bytes=2 << 30,
                     bucket_max_len=buckets, first_tier=tiers)
    ctx = wfe.Context(max_seq_len=max_seq, batch_size=SERVE_MAX_PAIRS, cigar_stride=stride)
    ctx.set_policy(buckets, tiers)

    def serve(arrivals):
        """Submit request i at arrivals[i] (monotonic ns); per-request latency in ms."""
        handles = [None] * nreq
        for i in range(nreq):
            while True:
                dt = arrivals[i] - time.monotonic_ns()
                if dt <= 0:
                    break
                if dt > 200_000:
                    time.sleep((dt - 100_000) / 1e9)
            handles[i] = srv.submit(h_ascii, reqs[i], out=views("served", i))
        for h in handles:
            assert srv.poll(h)
        done = np.array([h.info["done_ns"] for h in handles], dtype=np.float64)
        return (done - arrivals) / 1e6, done.max()

    def plain(arrivals):
        lat = np.zeros(nreq)
        last = 0
        for i in range(nreq):
            while time.monotonic_ns() < arrivals[i]:
                dt = arrivals[i] - time.monotonic_ns()
                if dt > 200_000:
                    time.sleep((dt - 100_000) / 1e9)
            ctx.align(h_ascii, reqs[i], out=views("plain", i))
            last = time.monotonic_ns()
            lat[i] = (last - arrivals[i]) / 1e6
        return lat, last

    # warm-up, then the peak: every request submitted at once
    serve(np.full(nreq, time.monotonic_ns(), dtype=np.float64))
    t0 = time.monotonic_ns()
    _, t_end = serve(np.full(nreq, t0, dtype=np.float64))
    peak = total / ((t_end - t0) / 1e9)
    plain(np.full(nreq, time.monotonic_ns(), dtype=np.float64))
    t0 = time.monotonic_ns()
    _, t_end = plain(np.full(nreq, t0, dtype=np.float64))
    plain_peak = total / ((t_end - t0) / 1e9)

    rows = []
    identical = True
    rates = [float(x) for x in args.rates.split(",")] if args.rates else SERVE_RATES
    for f in rates:
        rate = f * peak / float(sizes.mean())  # requests per second
        gaps = rng.exponential(1.0 / rate, nreq)
        row = {"load": f, "offered_alignments_per_s": f * peak}
        for m, fn in (("served", serve), ("plain", plain)):
            base = time.monotonic_ns() + 2_000_000
            arrivals = base + np.cumsum(gaps) * 1e9
            lat, t_end = fn(arrivals)
            row[m] = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                      "mean_ms": float(lat.mean()),
                      "alignments_per_s": total / ((t_end - base) / 1e9)}
        identical &= bool(np.array_equal(outs["served"][0], outs["plain"][0]) and
                          np.array_equal(outs["served"][2], outs["plain"][2]))
        rows.append(row)
    # CIGARs of the two forms, up to each terminator
    cs, cp = outs["served"][1], outs["plain"][1]
    lens = np.argmax(cs == 0, axis=1)
    same_cg = bool(np.array_equal(lens, np.argmax(cp == 0, axis=1)))
    if same_cg:
        mask = np.arange(stride)[None, :] <= lens[:, None]
        same_cg = bool(np.array_equal(np.where(mask, cs, 0), np.where(mask, cp, 0)))
    st = srv.stats()
    srv.close()
    ctx.close()
    line = {"metric": "p50/p99 request latency and alignments/sec", "workload": "serve",
            "unit": "ms / alignments/s",
            "config": {"requests": nreq, "pairs": total, "request_pairs": f"log-uniform [1, {SERVE_MAX_PAIRS}]",
                       "lengths": f"log-uniform [{SERVE_LMIN}, {SERVE_LMAX}]",
                       "edit_prob": f"uniform [{SERVE_PMIN}, {SERVE_PMAX}]", "seed": SERVE_SEED,
                       "arrivals": "Poisson", "lanes": 4, "memory_bytes": 2 << 30, "buckets": buckets,
                       "first_tiers": tiers, "inputs": "pinned host memory"},
            "peak_alignments_per_s": {"served": peak, "plain": plain_peak},
            "rates": rows, "server": st,
            "identical_results": identical and same_cg,
            "all_ok": bool((outs["served"][2] == 0).all())}
    s_dist, s_cg, s_st = outs["served"]
    line["parity"] = oracle_sample_parity(ascii, pairs, (s_dist, s_cg, s_st), stride, SERVE_SEED)
    del outs
    line["ref_cuda"] = reference_on_subset(ascii, pairs, s_dist, s_st, s_cg, buckets, stride, SERVE_SEED)
    print(json.dumps(line))
    good = line["identical_results"] and line["all_ok"] and line["parity"]["mismatches"] == 0
    return 0 if good else 1


def run_other_workloads() -> dict:
    """The long, mixed and serve workloads, each run by this script in a
    process of its own (its own CUDA context and memory), summarised for the
    short-read line: throughput, the checks each makes (identical results
    between forms, oracle parity) and the reference's kernels on the pairs
    in its search range."""
    runs = {"long": ["--steps", "10", "--warmup", "3"], "mixed": [], "serve": ["--rates", "0.5,1.0,1.2"]}
    out = {}
    for name, extra in runs.items():
        cmd = [sys.executable, os.path.abspath(__file__), "--workload", name] + extra
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
        except subprocess.TimeoutExpired:
            out[name] = {"error": "timed out after 900 s"}
            continue
        lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
        if r.returncode != 0 or not lines:
            out[name] = {"error": f"exit {r.returncode}", "stderr": r.stderr[-400:], "stdout": r.stdout[-400:]}
            continue
        full = json.loads(lines[-1])
        out[name] = summarise(name, full)
        out[name]["run_seconds"] = round(time.perf_counter() - t0, 1)
        out[name]["command"] = "python bench.py " + " ".join(["--workload", name] + extra)
    return out


def summarise(name: str, d: dict) -> dict:
    """The fields of a workload's JSON line that the short-read line carries."""
    if name == "long":
        return {"workload": d["config"]["workload"], "value": d["value"], "unit": d["unit"],
                "ms_per_step": d["ms_per_step"], "e2e": d["e2e"]["value"], "gcups": d["gcups"]["value"],
                "parity": d.get("parity"), "cpu_baseline": (d.get("cpu_baseline") or {}).get("value"),
                "roofline_frac": d["roofline"]["frac"]}
    if name == "mixed":
        keep = ("alignments_per_s", "seconds", "first_tiers")
        return {"pairs": d["pairs"], "config": d["config"],
                **{m: {k: d[m][k] for k in keep} for m in ("plain", "bucketed", "predicted")},
                "speedup_over_plain": d["speedup"], "identical_results": d["identical_results"],
                "all_ok": d["all_ok"], "parity": d["parity"], "ref_cuda": d.get("ref_cuda"),
                "distance": d["distance"]}
    if name == "serve":
        rows = [{"load": r["load"], "served": {k: r["served"][k] for k in ("p50_ms", "p99_ms", "alignments_per_s")},
                 "plain": {k: r["plain"][k] for k in ("p50_ms", "p99_ms", "alignments_per_s")}}
                for r in d["rates"]]
        srv = d.get("server") or {}
        nb = max(1, srv.get("batches", 0))
        sched = {"batches": srv.get("batches"), "admit_us_per_batch": srv.get("admit_ns", 0) / nb / 1e3,
                 "finish_us_per_batch": srv.get("finish_ns", 0) / nb / 1e3,
                 "note": "host time per batch: admitting it on the scheduler thread (forming it, enqueueing "
                         "copies and kernels), what a device-resident request queue could remove; and copying "
                         "its results out on the finisher threads (summed over them)"}
        return {"config": d["config"], "peak_alignments_per_s": d["peak_alignments_per_s"], "rates": rows,
                "identical_results": d["identical_results"], "all_ok": d["all_ok"], "parity": d["parity"],
                "scheduler": sched, "ref_cuda": d.get("ref_cuda")}
    return d


def workload_config(world: int, ascii_bytes: int) -> dict:
    """The `config` of both arms' JSON lines (identical keys and values)."""
    nb = PAIRS // BATCH
    return {"workload": WORKLOAD, "pairs_per_gpu": PAIRS, "batch": BATCH, "length": LENGTH,
            "edit_prob": EDIT_P, "seed": SEED, "cigar_stride": CIGAR_STRIDE,
            "l2": (f"inputs larger than L2: steps cycle over {nb} batches "
                   f"({ascii_bytes / 1e6:.0f} MB ASCII, {PAIRS * CIGAR_STRIDE / 1e6:.0f} MB CIGAR slots)"),
            "parallelism": f"replicas x{world}"}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def shard_seed(rank: int) -> int:
    """Seed of one rank's shard: every rank aligns its own pairs (weak scaling)."""
    return SEED + 1000 * rank


def reduce_max(x: float, world: int, device=None) -> float:
    """Max of x over ranks (identity for one process)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int, device=None) -> None:
    if world > 1:
        import torch.distributed as dist
        if device is not None:
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        mhz = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in rows for j in range(4) if r[5 + j].lower() == "active"})
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled(key: str):
    """A figure of the dominant kernel's committed ncu summary (a line
    'key: N'), or None."""
    p = os.path.join(ROOT, "profiles", PROFILE)
    try:
        for line in open(p):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def profiled_traffic():
    """DRAM bytes per launch of the dominant kernel (ncu, scaled to one launch)."""
    return profiled("traffic_bytes_per_launch")


def pageable_e2e(ascii, pairs, reps, local, world, device, want_dist) -> dict:
    """wfe_align with ordinary (pageable) numpy arrays, as most callers hold
    them: the inputs as generated and fresh np.empty outputs allocated inside
    the timed region every step.  Staged (cudaMemcpyAsync through the
    driver's bounce buffers) and in place through the CPU's page tables
    (WFE_FLAG_PAGEABLE_IN_PLACE: the library makes the fresh output pages
    present on the host, batch by batch, ahead of the kernels)."""
    import torch
    out = {"unit": "alignments/s", "outputs": "fresh np.empty arrays every step"}
    for name, flags in (("staged", 0), ("in_place", wfe.FLAG_PAGEABLE_IN_PLACE)):
        ctx = wfe.Context(max_seq_len=MAX_SEQ_LEN, batch_size=BATCH, cigar_stride=CIGAR_STRIDE, device=local,
                          flags=flags)
        ctx.align(ascii, pairs)  # warm-up
        ctx.reset_stats()
        barrier(world, device)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            res = (np.empty(PAIRS, np.int32), np.empty((PAIRS, CIGAR_STRIDE), np.int8), np.empty(PAIRS, np.uint8))
            ctx.align(ascii, pairs, out=res)
        torch.cuda.synchronize()
        dt = reduce_max(time.perf_counter() - t0, world, device)
        st = ctx.stats()
        ctx.close()
        if not np.array_equal(res[0], want_dist):
            raise SystemExit(f"pageable ({name}) and pinned results differ")
        out[name] = world * reps * PAIRS / dt
        out[name + "_mapped_batches"] = int(st["mapped_batches"])
    return out


def link_roofline(achieved_bps: float) -> dict:
    """The e2e leg's bytes from host memory per second against the host-to-
    device DMA rate of the CPU-GPU link measured here (256 MiB from pinned
    memory, best of 3, CUDA events)."""
    import torch
    n = 256 << 20
    h = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    h.fill_(1)
    d = torch.empty(n, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        with torch.cuda.stream(s):
            d.copy_(h, non_blocking=True)
        e1.record(s)
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    peak = n / (best * 1e-3) / 1e9
    achieved = achieved_bps / 1e9
    return {"bound": "CPU-GPU link (NVLink-C2C), host to device", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": "measured: 256 MiB DMA from pinned memory in this run"}


def cigar_lengths(cg: np.ndarray) -> np.ndarray:
    """Bytes of each encoded CIGAR before its terminator."""
    z = cg == 0
    has = z.any(1)
    return np.where(has, z.argmax(1), cg.shape[1])


def cpu_baseline(ascii, pairs, nthreads):
    """The CPU restatement of the reference (oracle/) on all host cores, on
    the whole workload (about 1-2 s of CPU time per 1M pairs and core).
    Returns the baseline record and the oracle's outputs (distances, CIGAR
    slots, statuses), which the timed runs are then checked against."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build(ref=False)
    t0 = time.perf_counter()
    dist, cg, st, (cells, words) = oracle.align_batch(ascii, pairs["p_off"], pairs["p_len"], pairs["t_off"],
                                                      pairs["t_len"], CIGAR_STRIDE, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return ({"value": len(pairs) / dt, "unit": METRIC, "cores": nthreads, "kind": "port",
             "sample": f"all {len(pairs):,} pairs of the workload, {nthreads} threads, {dt:.2f} s",
             "counts": {"cells": int(cells), "extend_words": int(words), "pairs": len(pairs)}},
            (dist, cg, st))


def parity(got, want) -> dict:
    """Pairs whose distance, status or CIGAR bytes (up to and including the
    terminator) differ between two result sets (dist, cigar slots, status)."""
    gd, gc, gs = got
    wd, wc, ws = want
    gc = np.asarray(gc).reshape(len(gd), -1)
    wc = np.asarray(wc).reshape(len(wd), -1)
    gl, wl = cigar_lengths(gc), cigar_lengths(wc)
    upto = np.arange(gc.shape[1])[None, :] <= gl[:, None]
    same_cg = (gl == wl) & np.all(np.where(upto, gc, 0) == np.where(upto, wc, 0), axis=1)
    bad = (np.asarray(gd) != np.asarray(wd)) | (np.asarray(gs) != np.asarray(ws)) | ~same_cg
    return {"pairs": int(len(gd)), "mismatches": int(bad.sum()),
            "compared": "distance, status and the CIGAR bytes up to the terminator of every pair"}


def int32_peak(device: int) -> dict | None:
    """32-bit integer operations per second of the device, measured by
    ewfa-gpu_gb300/csrc/int_peak.cu (three-input adds and logic ops, every SM
    full; best of 5 launches)."""
    import ctypes as C
    path = os.path.join(ROOT, "ewfa-gpu_gb300", "lib", "libwfe_intpeak.so")
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    L.wfe_int32_peak.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    ops, ms = C.c_double(0), C.c_double(0)
    if L.wfe_int32_peak(device, 4096, 5, C.byref(ops), C.byref(ms)) != 0:
        return None
    return {"ops_per_s": ops.value, "best_ms": ms.value}


def int_roofline(base, peak, step_ms, pairs_per_step) -> dict | None:
    """The integer-op roofline of the alignment: algorithmic integer
    operations per batch, OPS_alg = 12 C + 8 E per pair (C wavefront cells,
    E 16-base extend-word compares of the reference's extend over all cells
    and the CIGAR replay, both counted by the CPU restatement over the
    workload; 12 and 8 are the integer operations of one cell's compute and
    one extend word in src/kernels.cu:136-152 and :84-100), divided by the
    time per batch of the timed region (consecutive batches' kernels overlap,
    so a single launch's duration would count the overlap twice) and by the
    measured 32-bit integer issue peak."""
    if not base or "counts" not in base or not peak:
        return None
    cnt = base["counts"]
    ops_pair = (12.0 * cnt["cells"] + 8.0 * cnt["extend_words"]) / cnt["pairs"]
    ops_launch = ops_pair * pairs_per_step
    achieved = ops_launch / (step_ms * 1e-3) / 1e12
    p = peak["ops_per_s"] / 1e12
    return {"bound": "int32 issue", "achieved": achieved, "peak": p, "unit": "Tops/s", "frac": achieved / p,
            "ops_per_pair": ops_pair, "ops_per_launch": ops_launch,
            "cells_per_pair": cnt["cells"] / cnt["pairs"], "extend_words_per_pair": cnt["extend_words"] / cnt["pairs"],
            "peak_kind": "measured: ewfa-gpu_gb300/csrc/int_peak.cu on this GPU"}


def reference_cuda_baseline():
    """The reference's own CUDA kernels (src/kernels.cu compiled for sm_100,
    as its `make SM=100 COMPUTE=100 all` does) through a restatement of its
    batch loop, on the same workload: -n 1000000 -l 150 -b 100000.
      value   timed like its wfe.aligner: wall time from before the
              allocations to after the last batch and the frees
              (src/aligner.cu:198-233), -t 1/2/4/8, best of 3 each;
      steady  the batch loop alone: allocations before the clock, frees
              after it (-t 1/2, best of 3), the region that the e2e figure
              of wfe_align on an existing context times.
    None where the kernels were not compiled (they need the reference
    sources)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    try:
        oracle.build(ref=False)
    except Exception:
        return None
    if not oracle.ref_cuda_available() or LENGTH != 150:
        return None  # the reference searches distances up to 63: only the short-read workload fits
    runs, steady = {}, {}
    for t in (1, 2, 4, 8):
        rec = oracle.ref_cuda_run(PAIRS, LENGTH, EDIT_P, SEED, batch=BATCH, threads=t, reps=3)
        runs[t] = rec["alignments_per_s"]
    for t in (1, 2):
        rec = oracle.ref_cuda_run(PAIRS, LENGTH, EDIT_P, SEED, batch=BATCH, threads=t, reps=3, steady=True)
        steady[t] = rec["alignments_per_s"]
    best_t = max(runs, key=runs.get)
    best_s = max(steady, key=steady.get)
    return {"value": runs[best_t], "unit": "alignments/s", "threads": best_t,
            "wall_ms": 1e3 * PAIRS / runs[best_t],
            "by_threads": {str(t): round(v) for t, v in runs.items()},
            "steady": {"value": steady[best_s], "threads": best_s, "ms": 1e3 * PAIRS / steady[best_s],
                       "by_threads": {str(t): round(v) for t, v in steady.items()},
                       "region": "batch loop only: allocations and module load before the clock, frees after"},
            "kind": "reference src/kernels.cu (sm_100 cubin) + restated src/wavefront.cu batch loop, "
                    "wall time as src/aligner.cu:198-233, best of 3"}


def cli_wall(reps: int = 5) -> dict | None:
    """wfe.aligner -f F -n PAIRS -l LENGTH -b BATCH -t 1 on a pair file of
    the workload (written by wfe.gen with the same generator and seed): the
    wall time it prints, which covers the reference's region -- after the
    file is read, context creation and teardown included.  Best and median
    of `reps` runs."""
    exe = os.path.join(ROOT, "ewfa-gpu_gb300", "bin", "wfe.aligner")
    gen = os.path.join(ROOT, "ewfa-gpu_gb300", "bin", "wfe.gen")
    if not (os.path.exists(exe) and os.path.exists(gen)):
        return None
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "pairs.seq")
        subprocess.run([gen, path, str(PAIRS), str(LENGTH), str(LENGTH), str(EDIT_P), str(EDIT_P), str(SEED)],
                       check=True, stdout=subprocess.DEVNULL)
        walls, procs = [], []
        for _ in range(reps):
            t0 = time.perf_counter()
            out = subprocess.run([exe, "-f", path, "-n", str(PAIRS), "-l", str(LENGTH), "-b", str(BATCH), "-t", "1"],
                                 check=True, capture_output=True, text=True).stdout
            procs.append(time.perf_counter() - t0)
            line = [x for x in out.splitlines() if x.startswith("Aligned executed. Wall time")][-1]
            walls.append(float(line.split()[-1].rstrip("s")))
    best = min(walls)
    return {"value": PAIRS / best, "unit": "alignments/s", "wall_ms": 1e3 * best,
            "median_wall_ms": 1e3 * statistics.median(walls), "runs": reps,
            "process_ms": {"best": 1e3 * min(procs), "median": 1e3 * statistics.median(procs),
                           "what": "the whole process, start to exit: device set-up, file read, alignment"},
            "command": f"wfe.aligner -f pairs.seq -n {PAIRS} -l {LENGTH} -b {BATCH} -t 1",
            "region": "the reference's: after the file is read, teardown included; the contexts are set up "
                      "by threads that run while the file is read, and the region waits for any part of "
                      "that set-up still running"}


def noalloc_throughput(d_ascii, d_pairs, want, stream, steps: int) -> dict:
    """wfe_align_device_noalloc on the device-resident workload: one call per
    batch (its fixed scratch array bounds the pairs in flight), timed like
    `value`, results compared with the context path's."""
    import torch
    d_dist = torch.zeros(PAIRS, dtype=torch.int32, device=d_ascii.device)
    d_cigar = torch.zeros(PAIRS * CIGAR_STRIDE, dtype=torch.int8, device=d_ascii.device)
    d_status = torch.zeros(PAIRS, dtype=torch.uint8, device=d_ascii.device)
    nb = PAIRS // BATCH
    pb = wfe.PAIR_DTYPE.itemsize

    def step(i):
        b = i % nb
        wfe.align_device_noalloc(d_ascii, d_pairs.data_ptr() + b * BATCH * pb, BATCH, MAX_SEQ_LEN,
                                 wfe.NOALLOC_MAX_DISTANCE, d_dist.data_ptr() + 4 * b * BATCH,
                                 d_cigar.data_ptr() + b * BATCH * CIGAR_STRIDE, CIGAR_STRIDE,
                                 d_status.data_ptr() + b * BATCH, stream)

    for i in range(nb):
        step(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        step(i)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    got = (d_dist.cpu().numpy(), d_cigar.view(PAIRS, CIGAR_STRIDE).cpu().numpy(), d_status.cpu().numpy())
    return {"value": steps * BATCH / (ms / 1e3), "unit": "alignments/s", "ms_per_step": ms / steps,
            "max_distance": wfe.NOALLOC_MAX_DISTANCE, "same_as_context_path": parity(got, want)["mismatches"] == 0,
            "note": "no context and no allocation: tier 0 (backtrace store in shared memory) over every pair, "
                    "then tier 3 over the pairs past distance 21 with its backtrace scratch in a fixed 16 MiB "
                    "device array (153 CTAs at most), one call per batch"}


def reference_check_baseline(ascii, pairs, cigars) -> dict | None:
    """The reference's own host check path (Cigars::check_cigar,
    src/wavefront.cuh:297-419, compiled from the reference's files into
    oracle/_ref) over every pair's CIGAR, on 1 thread and on every host core
    (contiguous shares, as src/aligner.cu:45-48 splits pairs).  A validity
    replay, not an aligner.  None where the library could not be built."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    if not oracle.ref_available():
        return None
    import ref_check_baseline as rcb
    try:
        recs = rcb.run(ascii, pairs, cigars)
    except (OSError, subprocess.CalledProcessError, ValueError):
        return None
    best = max(recs, key=lambda r: r["pairs_per_s"])
    return {"value": best["pairs_per_s"], "unit": "pairs checked/s", "threads": best["threads"],
            "by_threads": {str(r["threads"]): round(r["pairs_per_s"]) for r in recs},
            "valid": best["valid"], "pairs": best["pairs"], "cores": os.cpu_count(),
            "kind": "reference Cigars::check_cigar (src/wavefront.cuh:297-419) built from its sources, "
                    "best of 3; a validity replay of the CIGARs, not an aligner"}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    ascii, pairs = wfe.generate(PAIRS, LENGTH, p_min=EDIT_P, seed=SEED)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build(ref=False)
    nthreads = os.cpu_count() or 1
    nb = PAIRS // BATCH

    def step(i):
        sl = pairs[(i % nb) * BATCH:(i % nb + 1) * BATCH]
        oracle.align_batch(ascii, sl["p_off"], sl["p_len"], sl["t_off"], sl["t_len"], CIGAR_STRIDE,
                           nthreads=nthreads)

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    for i in range(args.steps):
        step(i)
    dt = time.perf_counter() - t0
    value = args.steps * BATCH / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "alignments/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator; no dataset)",
        "config": workload_config(world, len(ascii)),
        "cpu_baseline": {"value": value, "unit": "alignments/s", "cores": nthreads, "kind": "port",
                         "sample": f"{args.steps} batches of {BATCH:,} pairs, {nthreads} threads; the CPU "
                                   "restatement of the reference's kernels (the reference has no CPU aligner)"},
        "e2e": {"value": value, "unit": "alignments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.link:
        return run_link()
    if args.workload == "mixed":
        return run_mixed(args)
    if args.workload == "serve":
        return run_serve(args)
    select_workload(args.workload)
    if args.profile_batch:
        return run_profile_case(args)
    if args.impl == "reference":
        return run_reference(args)
    import torch
    world, rank, local = dist_env()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device")
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=device)

    # this rank's shard of the workload
    ascii, pairs = wfe.generate(PAIRS, LENGTH, p_min=EDIT_P, seed=shard_seed(rank))
    nb = PAIRS // BATCH
    stream = torch.cuda.Stream(device=device)

    # ---------------- value: inputs resident in HBM --------------------------
    # Step i aligns batch i mod nb.  The steps' descriptors are laid out one
    # after another (the workload's batches repeated; they all point into the
    # one ASCII buffer), with an output slot per step, so that the timed
    # steps are ONE wfe_align_device call: the library overlaps each batch's
    # last CTAs with the next batch's first on its two streams, as a caller
    # aligning many device-resident batches does.  Consecutive calls on one
    # stream are ordered, so each call boundary would drain the GPU once.
    warm = max(3, args.warmup)
    nrep = max(args.steps, warm, nb)
    order = np.arange(nrep) % nb
    pairs_rep = pairs[:nb * BATCH].reshape(nb, BATCH)[order].reshape(-1)
    d_ascii = torch.from_numpy(ascii).to(device)
    d_pairs_rep = torch.from_numpy(pairs_rep.view(np.uint8)).to(device)
    pair_bytes = wfe.PAIR_DTYPE.itemsize
    d_pairs = d_pairs_rep[:PAIRS * pair_bytes]  # the workload itself: the first nb steps
    d_dist = torch.zeros(nrep * BATCH, dtype=torch.int32, device=device)
    d_cigar = torch.zeros(nrep * BATCH * CIGAR_STRIDE, dtype=torch.int8, device=device)
    d_status = torch.zeros(nrep * BATCH, dtype=torch.uint8, device=device)
    # no kernel-timing events in the timed region (they cost ~1%); a separate
    # pass below times the launches
    ctx = wfe.Context(max_seq_len=MAX_SEQ_LEN, batch_size=BATCH, cigar_stride=CIGAR_STRIDE, device=local)

    def steps(first, count, c=None):
        """Steps first .. first+count-1 in one call."""
        (c or ctx).align_device(d_ascii, d_pairs_rep.data_ptr() + first * BATCH * pair_bytes, count * BATCH,
                                MAX_SEQ_LEN, d_dist.data_ptr() + 4 * first * BATCH,
                                d_cigar.data_ptr() + first * BATCH * CIGAR_STRIDE, d_status.data_ptr() + first * BATCH,
                                stream)

    with torch.cuda.stream(stream):
        steps(0, warm)
    torch.cuda.synchronize()
    ctx.reset_stats()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world, device)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        start.record(stream)
        steps(0, args.steps)
        end.record(stream)
        torch.cuda.synchronize()
    barrier(world, device)
    ms = start.elapsed_time(end)
    ms_max = reduce_max(ms, world, device)
    st = ctx.stats()
    value = world * args.steps * BATCH / (ms_max / 1e3)
    cells_per_pair = float(np.mean(pairs["p_len"].astype(np.float64) * pairs["t_len"]))
    with torch.cuda.stream(stream):
        if max(warm, args.steps) < nb:  # every batch of the workload is checked below
            steps(max(warm, args.steps), nb - max(warm, args.steps))
    torch.cuda.synchronize()
    # every repeat of a batch gave that batch's results
    repeats_identical = all(
        torch.equal(buf[i * BATCH * w:(i + 1) * BATCH * w], buf[(i % nb) * BATCH * w:(i % nb + 1) * BATCH * w])
        for i in range(nb, args.steps) for buf, w in ((d_dist, 1), (d_cigar, CIGAR_STRIDE), (d_status, 1)))
    if not repeats_identical:
        raise SystemExit("a repeated batch gave different results")
    # the launches' own spans, from a pass of the workload's nb batches on a
    # context with kernel timing (outside the timed region)
    with wfe.Context(max_seq_len=MAX_SEQ_LEN, batch_size=BATCH, cigar_stride=CIGAR_STRIDE, device=local,
                     flags=wfe.FLAG_KERNEL_TIMING) as ctx_t:
        with torch.cuda.stream(stream):
            steps(0, nb, ctx_t)
        torch.cuda.synchronize()
        ctx_t.reset_stats()
        with torch.cuda.stream(stream):
            steps(0, nb, ctx_t)
        torch.cuda.synchronize()
        st_t = ctx_t.stats()

    # algorithmic bytes of one batch: ASCII read once, descriptors, and the
    # distance, status and CIGAR bytes (with terminator) written
    cg = d_cigar[:PAIRS * CIGAR_STRIDE].view(PAIRS, CIGAR_STRIDE).cpu().numpy()
    st_h = d_status[:PAIRS].cpu().numpy()
    assert (st_h == 0).all(), "non-OK pair status in the benchmark workload"
    dev_out = (d_dist[:PAIRS].cpu().numpy(), cg, st_h)
    clen = np.minimum(cigar_lengths(cg) + 1, CIGAR_STRIDE)
    bytes_per_batch = []
    for b in range(nb):
        sl = slice(b * BATCH, (b + 1) * BATCH)
        bytes_per_batch.append(int(pairs["p_len"][sl].sum() + pairs["t_len"][sl].sum()) +
                               BATCH * (pair_bytes + 4 + 1) + int(clen[sl].sum()))
    alg_bytes = float(np.mean([bytes_per_batch[i % nb] for i in range(args.steps)]))
    tier_ms = st_t["tier_ms"]
    top = int(np.argmax(tier_ms))
    launch_ms = tier_ms[top] / max(1, st_t["tier_launches"][top])
    peak, peak_kind = measured_hbm_peak()
    # one tier-0 launch per step; consecutive launches overlap on two
    # streams, so the time a launch takes of the step is the time per step
    achieved = alg_bytes / (ms_max / args.steps / 1e3) / 1e9
    traffic = profiled_traffic()
    gpu_launches = int(st["kernel_launches"])

    # ---------------- e2e: host buffers through wfe_align ---------------------
    # The timed passes over the workload are wfe_align calls over up to
    # E2E_REPEATS passes each: the workload's descriptors repeated in pinned
    # memory (all pointing into the one ASCII buffer), an output slot per pair
    # of every pass, as a caller with that many pairs to align makes one call.
    # Calls of the workload's own size are timed beside it.
    reps = max(1, args.steps // nb)
    per_call = min(reps, E2E_REPEATS)
    h_ascii = torch.empty(len(ascii), dtype=torch.uint8, pin_memory=True).numpy()
    h_ascii[:] = ascii
    h_pairs_rep = torch.empty(per_call * PAIRS * pair_bytes, dtype=torch.uint8,
                              pin_memory=True).numpy().view(wfe.PAIR_DTYPE)
    h_pairs_rep[:] = np.tile(pairs, per_call)
    h_dist_rep = torch.empty(per_call * PAIRS, dtype=torch.int32, pin_memory=True).numpy()
    h_cigar_rep = torch.empty(per_call * PAIRS * CIGAR_STRIDE, dtype=torch.int8,
                              pin_memory=True).numpy().reshape(per_call * PAIRS, CIGAR_STRIDE)
    h_status_rep = torch.empty(per_call * PAIRS, dtype=torch.uint8, pin_memory=True).numpy()
    h_pairs, h_dist, h_cigar, h_status = (h_pairs_rep[:PAIRS], h_dist_rep[:PAIRS], h_cigar_rep[:PAIRS],
                                          h_status_rep[:PAIRS])
    ctx2 = wfe.Context(max_seq_len=MAX_SEQ_LEN, batch_size=BATCH, cigar_stride=CIGAR_STRIDE, device=local)
    ctx2.align(h_ascii, h_pairs, out=(h_dist, h_cigar, h_status))  # warm-up
    ctx2.reset_stats()
    barrier(world, device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    left = reps
    while left:
        k = min(left, per_call)
        ctx2.align(h_ascii, h_pairs_rep[:k * PAIRS],
                   out=(h_dist_rep[:k * PAIRS], h_cigar_rep[:k * PAIRS], h_status_rep[:k * PAIRS]))
        left -= k
    torch.cuda.synchronize()
    e2e_s = reduce_max(time.perf_counter() - t0, world, device)
    barrier(world, device)
    st2 = ctx2.stats()
    for i in range(1, min(reps, per_call)):
        sl = slice(i * PAIRS, (i + 1) * PAIRS)
        if not (np.array_equal(h_dist_rep[sl], h_dist) and np.array_equal(h_cigar_rep[sl], h_cigar)
                and np.array_equal(h_status_rep[sl], h_status)):
            raise SystemExit("a repeated pass gave different results")
    # the same passes as calls of the workload's size
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx2.align(h_ascii, h_pairs, out=(h_dist, h_cigar, h_status))
    torch.cuda.synchronize()
    e2e_calls_s = reduce_max(time.perf_counter() - t0, world, device)
    # bytes that crossed the CPU-GPU link per step: staged copies (counted by
    # the library) plus what the kernels read/wrote in place in pinned memory
    in_place = st2["mapped_batches"] == st2["batches"]
    # with pinned buffers the kernels read each batch's descriptors and
    # sequences in place and write distances, statuses and the used bytes of
    # each CIGAR slot (rounded to 4) in place: those are the bytes that cross
    # the CPU-GPU link; staged calls count their copies in the statistics
    if in_place:
        h2d = int(pairs["p_len"].sum() + pairs["t_len"].sum()) // nb + BATCH * pair_bytes
        out_len = np.minimum((cigar_lengths(h_cigar) + 4) // 4 * 4, CIGAR_STRIDE)
        d2h = BATCH * 5 + int(out_len.sum()) // nb
    else:
        h2d = int(st2["h2d_bytes"] // max(1, st2["batches"]))
        d2h = int(st2["d2h_bytes"] // max(1, st2["batches"]))
    e2e = {"value": world * reps * PAIRS / e2e_s, "unit": "alignments/s",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": reps * nb,
           "calls": (f"{-(-reps // per_call)} wfe_align call(s) of up to {per_call} passes over the workload "
                     "(its descriptors repeated in pinned memory, an output slot per pair of every pass)"),
           "calls_of_the_workload": {"value": world * reps * PAIRS / e2e_calls_s, "unit": "alignments/s",
                                     "what": f"the same {reps} passes as {reps} calls of {PAIRS} pairs"},
           "transfer": ("kernels read the pinned host inputs and write the pinned host outputs in place "
                        "over NVLink-C2C" if in_place else "staged cudaMemcpyAsync copies")}
    if not (np.array_equal(h_dist, d_dist[:PAIRS].cpu().numpy())):
        raise SystemExit("host-buffer and device-buffer results differ")
    e2e_out = (h_dist.copy(), h_cigar.copy(), h_status.copy())
    e2e["pageable"] = pageable_e2e(ascii, pairs, reps, local, world, device, h_dist)
    e2e["link_roofline"] = link_roofline(h2d * reps * nb / e2e_s)

    short = LENGTH == 150
    noalloc = noalloc_throughput(d_ascii, d_pairs, dev_out, stream, args.steps) if rank == 0 and short else None

    base = None
    ref_cuda = cli = ref_check = None
    checked = None
    int_peak = int32_peak(local) if rank == 0 else None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base, want = cpu_baseline(ascii, pairs, os.cpu_count() or 1)
        checked = {"value": parity(dev_out, want), "e2e": parity(e2e_out, want),
                   "against": "the CPU restatement of the reference (oracle/) on every pair of the workload"}
        if checked["value"]["mismatches"] or checked["e2e"]["mismatches"]:
            print(json.dumps({"parity": checked}), file=sys.stderr)
            raise SystemExit("the timed results differ from the oracle's")
        if short:
            ref_check = reference_check_baseline(ascii, pairs, want[1])
        del want
        if short:
            ref_cuda = reference_cuda_baseline()
            cli = cli_wall()
    int_roof = int_roofline(base, int_peak, ms_max / args.steps, BATCH)
    if base:
        base = {k: v for k, v in base.items() if k != "counts"}
    versus = None
    if ref_cuda:
        versus = {"definition": "this build's time over the reference CUDA build's on the same region",
                  "e2e_over_ref_steady": e2e["value"] / ref_cuda["steady"]["value"],
                  "value_over_ref_steady": value / ref_cuda["steady"]["value"]}
        if cli:
            versus["cli_over_ref_wall"] = cli["value"] / ref_cuda["value"]

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "alignments/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded generator; no dataset)",
            "config": workload_config(world, len(ascii)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "integer_pipes": {"alu_pipe_pct_of_peak": profiled("alu_pipe_pct_of_peak"),
                                           "issue_slots_busy_pct": profiled("issue_slots_busy_pct"),
                                           "source": "ncu, profiles/" + PROFILE,
                                           "note": "the kernel is bound by its integer pipes, not by HBM"},
                         "kernel": f"tier_kernel tier {top}" + (" and the tiers it hands pairs on to (one timed "
                                                                     "chain)" if any(st["tier_passed"]) else ""),
                         "alg_bytes_per_launch": alg_bytes,
                         "ms_per_launch": ms_max / args.steps,
                         "overlap": "one tier-0 launch per step; the timed steps are one wfe_align_device call "
                                    "(the workload's batches repeated in HBM, an output slot per step), whose "
                                    "batches alternate between two streams, so consecutive launches overlap and "
                                    "the time per step is the time a launch adds (each launch spans "
                                    f"{launch_ms:.3f} ms from start to end, events on its stream in a separate "
                                    "timing pass, while sharing the GPU with its neighbours)",
                         "int32": int_roof},
            "gcups": {"value": value * cells_per_pair / 1e9,
                      "definition": "equivalent DP cell updates: sum of p_len * t_len per second / 1e9"},
            "cpu_baseline": base,
            "parity": checked,
            "ref_cuda": ref_cuda,
            "cli": cli,
            "versus_ref_cuda": versus,
            "ref_check": ref_check,
            "noalloc": noalloc,
            "e2e": e2e,
            "gpu_launches": gpu_launches,
            "clocks": clocks.summary(),
            "tiers": {"launches": st["tier_launches"][:7], "passed_on": st["tier_passed"][:7],
                      "timing_pass": {"ms": [round(x, 4) for x in tier_ms[:7]], "launches": st_t["tier_launches"][:7],
                                      "what": "the workload's batches once more, on a context with kernel "
                                              "timing, outside the timed region"}},
        }
        if short and world == 1 and not args.no_cpu_baseline and not args.no_other_workloads:
            ctx.close()
            ctx2.close()
            del d_ascii, d_pairs, d_pairs_rep, d_dist, d_cigar, d_status
            torch.cuda.empty_cache()
            line["other_workloads"] = run_other_workloads()
        print(json.dumps(line))
    ctx.close()
    ctx2.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

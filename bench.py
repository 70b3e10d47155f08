"""Benchmark: exact self-join of the 1M-set long-set workload at Jaccard 0.8.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (seeded synthetic, no dataset): 1,000,000 sets, sizes lognormal(4.4, 0.8)
clamped to [10, 2000], universe 1,000,000, Zipf s=0.9 tokens drawn without
replacement, 5% planted near-duplicates with 5-15% token edits, tokens renumbered
by ascending frequency, collection sorted by size (112M tokens, 449 MB).

A step is one whole self-join: prefix-index build (entries + token histogram,
scan, list build), signatures, and the persistent filter+verify launch, with the collection already
resident in HBM (`value`), or through the public API from pinned host memory with
the pairs copied back (`e2e`).  Between timed steps a 512 MB buffer is written to
flush the 129 MB L2.  The reference-shaped block-pair path (one launch per block
pair, synchronous copies, as the reference's handlers do) is timed beside it as
the plain baseline.  Beside the headline, untimed by the step clock: the pair
set against the oracle (`parity`), the plain single-launch prefix filter and
the autotuner's configuration forced explicitly (`plain_single_launch_ms`,
`autotuned_ms`, `auto_ms`), and the first 64 joins of the batched workload in
one launch against one call at a time (`batch_leg`).  --impl reference times
the reference algorithm on the host cores (the CPU oracle, cpu_multi
semantics, all threads).  --sim cosine (or dice)
runs the same workload under that similarity (no block-pair leg: the reference's
handlers are Jaccard only).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "self-join ms & verified pairs/s at τ=0.8, batched+learned vs plain, 1 GB300"
WORKLOAD = ("1M-set long-set self-join, Jaccard 0.8: 1,000,000 sets, lognormal(4.4,0.8) sizes in [10,2000], "
            "universe 1,000,000, Zipf 0.9, 5% near-duplicates (5-15% edits)")
THRESHOLD = 0.8


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_name(sim):
    return WORKLOAD if sim == "jaccard" else WORKLOAD.replace("Jaccard 0.8", f"{sim} 0.8")


def make_workload(n_sets=None):
    from hyset_gb300 import synth
    return synth.generate(synth.C3, **({"n_sets": n_sets} if n_sets else {}))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.2)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(sim, n_sets, bits):
    """DRAM bytes per launch of the join kernel from the committed ncu summary
    and the configuration it was captured in, when this run's workload and
    kernel instance are the ones captured there (the full 1M-set Jaccard
    workload, 512-bit signatures; the probe batch is a launch parameter of the
    same kernel); otherwise (None, None)."""
    if sim != "jaccard" or n_sets or bits != 512:
        return None, None
    try:
        with open(os.path.join(ROOT, "profiles", "join_kernel_c3_traffic.json")) as f:
            m = json.load(f)
        return m.get("dram_bytes_per_launch"), m.get("kernel")
    except (OSError, ValueError):
        return None, None


def algorithmic_bytes(st, count, words, n_probes):
    """Bytes the probe-major filter+verify launch must touch, from its own work
    counters: per probe its (start, size) record (8); per prefix token the token
    and its list bounds (12); per index entry in a window the packed entry (4);
    per entry that passes the entry's side of the positional bound (all of
    them unless the records carry that bound) the candidate's (start, size)
    (8); per signature check both signatures (16 W); per token read by
    verification 4; per result pair 8."""
    prefix_tokens, items, bitmap_checks, verify_tokens = st[4], st[0], st[5], st[6]
    entries = st[7] or items
    return (8 * n_probes + 12 * prefix_tokens + 4 * entries + 8 * items + 16 * words * bitmap_checks
            + 4 * verify_tokens + 8 * count)


def cpu_baseline(c, threads, sample_note, sim="jaccard"):
    import oracle
    t0 = time.perf_counter()
    if threads == 1:
        pairs = oracle.join(c.tokens, c.starts, c.sizes, THRESHOLD, sim=sim)
        idx_s, join_s = oracle.last_timing()
    else:
        pairs = oracle.join_multi(c.tokens, c.starts, c.sizes, THRESHOLD, threads, sim=sim)
        idx_s, join_s = oracle.last_timing(multi=True)
    wall = time.perf_counter() - t0
    return len(pairs), join_s, idx_s, wall


def run_reference(args, ws, rank):
    """--impl reference: the reference algorithm (host::allpairs, cpu_multi split)
    on the host cores, every step the full join."""
    if rank != 0:
        return
    c = make_workload(args.sets)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(c, threads, "", args.sim)
    times, counts = [], []
    for _ in range(args.steps):
        n, join_s, idx_s, wall = cpu_baseline(c, threads, "", args.sim)
        times.append(join_s + idx_s)
        counts.append(n)
    ms = 1000.0 * statistics.mean(times)
    value = counts[0] / (ms / 1000.0)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generator)",
            "config": {"workload": workload_name(args.sim), "threshold": THRESHOLD, "sim": args.sim,
                       "result_pairs": counts[0]},
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                             "sample": "whole workload each step (index build + join), oracle restatement of "
                                       "host::allpairs with the cpu_multi sqrt split"},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def check_parity(ctx, coll, c, kw, p_lo, p_hi, sim):
    """One untimed join with its pairs copied back, compared as a set with the
    oracle's pairs of the same probe range; returns the parity record."""
    import numpy as np
    import oracle
    q = dict(kw)
    q["device_pairs"] = False
    r = ctx.self_join(coll, **q)
    threads = os.cpu_count() or 1
    if (p_lo, p_hi) == (0, c.n):
        exp = oracle.join_multi(c.tokens, c.starts, c.sizes, THRESHOLD, threads, sim=sim)
    else:
        exp = oracle.join_multi_range(c.tokens, c.starts, c.sizes, THRESHOLD, threads, (p_lo, p_hi - 1), sim=sim)

    def keys(p):
        p = np.asarray(p, np.uint64).reshape(-1, 2)
        return np.sort((p[:, 0] << np.uint64(32)) | p[:, 1])

    got, want = keys(r.pairs), keys(exp)
    ok = bool(got.size == r.count and np.array_equal(got, want))
    return {"parity": ok, "pairs": int(r.count), "oracle_pairs": int(want.size),
            "checked_against": f"oracle restatement of host::allpairs, probes [{p_lo}, {p_hi}), {threads} threads"}


def shard(n, ws, rank):
    """Probe range of this rank: sqrt split (later probes have longer candidate windows)."""
    import math
    pts = [0] + [int(n * math.sqrt((i + 1) / ws)) for i in range(ws)]
    pts[-1] = n
    return pts[rank], pts[rank + 1]


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch
    import hyset_gb300 as hs
    from hyset_gb300.handlers import FgssHandler

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    c = make_workload(args.sets)
    p_lo, p_hi = shard(c.n, ws, rank)
    ctx = hs.Context(local)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    kw = dict(threshold=THRESHOLD, sim=args.sim, technique=args.technique, bitmap=args.bitmap, device_pairs=True,
              probe_range=(p_lo, p_hi), probe_major=args.probe_major, verify_mode=args.vmode, fgss_batch=args.batch)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # untimed: work counters for the roofline, and the shard's pair set against
    # the oracle (the reference's host::allpairs restated, all host threads)
    st_run = ctx.self_join(coll, collect_stats=True, **kw)
    parity = check_parity(ctx, coll, c, kw, p_lo, p_hi, args.sim)
    for _ in range(args.warmup):
        ctx.self_join(coll, **kw)
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    dev_ms, kern_ms, counts, launches = [], [], [], 0
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        r = ctx.self_join(coll, **kw)
        dev_ms.append(r.device_ms)
        kern_ms.append(r.kernel_ms)
        counts.append(r.count)
        launches += r.launches
    barrier()
    clocks = sampler.stop()
    mean_ms = statistics.mean(dev_ms)
    if dist is not None:
        t = torch.tensor([mean_ms, float(counts[0])], device="cuda", dtype=torch.float64)
        mx = t.clone()
        dist.all_reduce(mx[:1], op=dist.ReduceOp.MAX)
        dist.all_reduce(t[1:], op=dist.ReduceOp.SUM)
        step_ms, total_pairs = float(mx[0]), int(t[1])
    else:
        step_ms, total_pairs = mean_ms, counts[0]
    value = total_pairs / (step_ms / 1000.0)

    # e2e through the public C ABI: pinned host arrays -> one upload+join call -> pairs to host
    tok_p = torch.from_numpy(c.tokens).pin_memory()
    siz_p = torch.from_numpy(c.sizes).pin_memory()
    sta_p = torch.from_numpy(c.starts).pin_memory()
    e2e_kw = dict(kw)
    e2e_kw["device_pairs"] = False
    whole = (p_lo, p_hi) == (0, c.n)
    if whole:
        e2e_kw.pop("probe_range")  # one call: upload and join (hyset_self_join_host)
    e2e_s = []
    for i in range(0 if args.no_e2e else args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if whole:
            er = ctx.self_join_host(tok_p.numpy(), siz_p.numpy(), sta_p.numpy(), **e2e_kw)
        else:  # a rank's shard: upload, then the join over its probe range
            ec = ctx.upload(tok_p.numpy(), siz_p.numpy(), sta_p.numpy())
            er = ctx.self_join(ec, **e2e_kw)
            ec.free()
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_s.append(dt)
    h2d = c.tokens.nbytes + c.sizes.nbytes + c.starts.nbytes
    if args.no_e2e:
        e2e_s, er = [float("nan")], None
    e2e_pairs_bytes = int(er.pairs.nbytes) if er is not None else 0
    e2e_mean = statistics.mean(e2e_s)
    if dist is not None:
        t = torch.tensor([e2e_mean], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_mean = float(t[0])
    e2e_value = total_pairs / e2e_mean

    # attribution of the headline (collection resident, L2 flushed, median of
    # five): the plain single-launch path (probe-major prefix filter, no
    # signatures, a lane per candidate, one probe per warp batch: no tuning at
    # all) and the autotuner's configuration (signature width, verification
    # mode, probe batch) forced explicitly, beside AUTO (selector + autotuner)
    def leg_ms(q, reps=5):
        ms = []
        for _ in range(reps):
            flush.fill_(1)
            torch.cuda.synchronize()
            ms.append(ctx.self_join(coll, **q).device_ms)
        return statistics.median(ms)

    plain_kw = dict(kw, technique="fgss", probe_major=True, bitmap=0, verify_mode=1, fgss_batch=1)
    tuned_kw = dict(kw, technique="fgss", probe_major=True, bitmap=r.bitmap_bits, verify_mode=r.verify_mode,
                    fgss_batch=r.probe_batch or 0)
    legs = {"plain_single_launch_ms": leg_ms(plain_kw), "autotuned_ms": leg_ms(tuned_kw), "auto_ms": leg_ms(kw)}
    # batching: the first 64 joins of the batched workload in one launch vs one call at a time
    batch = None if args.no_batch or rank != 0 else batch_leg(ctx, 64, 3, 1, flush)

    out = None
    if rank == 0:
        # the plain reference-shaped path: block pairs of 10,000 sets, one launch each
        hc = hs.from_arrays(c.tokens, c.sizes, 10000, THRESHOLD)
        plain = []
        for i in range(0 if args.no_plain or args.sim != "jaccard" else 2):
            h = FgssHandler(ctx, hc, coll, 10000, False, THRESHOLD)
            ph = hs.PairsHandler()
            h.set_output_handler(ph)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            h.join(hs.Partition(0, hc.blocks), hs.Partition(0, hc.blocks))
            plain.append(time.perf_counter() - t0)
            h.close()
        plain_ms = 1000.0 * min(plain) if plain else None
        peak, peak_kind = measured_peaks()
        words = st_run.bitmap_bits // 64
        st = st_run.stats
        alg = algorithmic_bytes(st, st_run.count, words, p_hi - p_lo)
        kms = statistics.mean(kern_ms)
        achieved = alg / (kms / 1000.0) / 1e9
        traffic, traffic_capture = ncu_traffic(args.sim, args.sets, st_run.bitmap_bits) if ws == 1 else (None, None)
        cpu = {"value": None}
        if not args.no_cpu:
            n_cpu, join_s, idx_s, wall = cpu_baseline(c, 1, "", args.sim)
            cpu = {"value": n_cpu / (join_s + idx_s), "unit": "pairs/s", "cores": 1, "kind": "port",
                   "sample": f"whole workload once: index {idx_s:.2f} s + join {join_s:.2f} s on 1 core "
                             f"(oracle restatement of host::allpairs)"}
        out = {"metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "strong",
               "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded generator)",
               "config": {"workload": workload_name(args.sim), "threshold": THRESHOLD, "sim": args.sim,
                          "technique": r.technique, "bitmap_bits": r.bitmap_bits, "verify_mode": r.verify_mode,
                          "result_pairs": total_pairs,
                          "parallelism": f"probe shards x{ws}" if ws > 1 else "single GPU",
                          "l2": "512 MB buffer written between timed steps; tokens 449 MB > L2",
                          "probe_batch": r.probe_batch, "selector": r.selector,
                          "plain_block_pair_ms": plain_ms,
                          "speedup_vs_block_pair": plain_ms / step_ms if plain_ms else None,
                          **legs,
                          "speedup_vs_plain_single_launch": legs["plain_single_launch_ms"] / legs["auto_ms"],
                          "kernel_ms": kms},
               "batch_leg": batch,
               "parity": parity["parity"], "parity_detail": parity,
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "traffic": traffic, "traffic_capture": traffic_capture,
                            "peak_kind": peak_kind, "algorithmic_bytes_per_launch": alg,
                            "kernel": "k_join (probe-major FGSS filter + verify, persistent)"},
               "cpu_baseline": cpu,
               "e2e": {"value": e2e_value, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
                       "d2h_bytes_per_step": e2e_pairs_bytes + 8, "ms_per_step": 1000.0 * e2e_mean},
               "clocks": clocks, "gpu_launches": launches}
        print(json.dumps(out), flush=True)
    coll.free()
    if not parity["parity"]:
        sys.exit(f"parity failure: {parity}")
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return out


def batch_leg(ctx, n_joins, steps, warmup, flush):
    """The batched workload's first `n_joins` joins (R-S joins of uneven sizes,
    mixed similarities and thresholds): all in one persistent launch captured
    in a CUDA graph (hyset_batch_join), against the same joins one call at a
    time with the same AUTO configurations.  Device times, L2 flushed."""
    import torch
    from hyset_gb300 import synth
    t0 = time.time()
    work = synth.batch_workload(n_joins)
    gen_s = time.time() - t0
    joins, colls = [], []
    for (rt, rs, rz), (st, ss, sz), kw in work:
        R = ctx.upload(rt, rz, rs)
        S = ctx.upload(st, sz, ss)
        colls += [R, S]
        joins.append((R, S, dict(kw, device_pairs=True)))
    res = ctx.batch_join(joins)  # plans, tunes and captures the batch
    for _ in range(warmup):
        res = ctx.batch_join(joins)
    batch_ms, seq_ms, launches = [], [], 0
    for _ in range(steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        res = ctx.batch_join(joins)
        batch_ms.append(res[0].device_ms)
    total = sum(r.count for r in res)
    for _ in range(max(1, steps // 2)):
        flush.fill_(1)
        torch.cuda.synchronize()
        t = 0.0
        for R, S, kw in joins:
            one = ctx.rs_join(R, S, **kw)
            t += one.device_ms
            launches += one.launches
        seq_ms.append(t)
    sets = int(sum(c.n for c in colls))
    for c in colls:
        c.free()
    bm, sm = statistics.mean(batch_ms), statistics.mean(seq_ms)
    return {"joins": n_joins, "sets": sets, "result_pairs": total, "batch_ms": bm, "one_at_a_time_ms": sm,
            "speedup_vs_one_at_a_time": sm / bm, "one_at_a_time_launches": launches // max(1, steps // 2),
            "generation_s": gen_s}


def run_batch(args):
    import torch
    import hyset_gb300 as hs
    ctx = hs.Context(0)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    leg = batch_leg(ctx, args.joins, args.steps, args.warmup, flush)
    print(json.dumps({"metric": "batched R-S joins: result pairs/s (one persistent launch in a CUDA graph)",
                      "value": leg["result_pairs"] / (leg["batch_ms"] / 1000.0), "unit": "pairs/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": leg["batch_ms"],
                      "higher_is_better": True,
                      "config": {"workload": f"{args.joins} R-S joins, |R|,|S| log-uniform [1e3, 2e5], mean size "
                                             "log-uniform [8, 300], mixed similarity, threshold U[0.5, 0.95]",
                                 **leg}}), flush=True)


def run_parse(args):
    """The collection reader (the step before the join): the workload's text
    form parsed on the GPU, from device memory (`value`) and from pinned host
    memory (`e2e`, copy included), against the reference reader's restatement
    on one host core over a bounded sample."""
    import numpy as np
    import torch
    import hyset_gb300 as hs
    import oracle
    from hyset_gb300 import synth
    c = make_workload(args.sets or None)
    n_bytes = int(hs_text_bytes(c))
    pinned = torch.empty(n_bytes, dtype=torch.uint8).pin_memory()
    text = synth.format_text(c.tokens, c.starts, c.sizes, out=pinned.numpy())
    assert text.size == n_bytes
    ctx = hs.Context(0)
    d_text = torch.empty(n_bytes, dtype=torch.uint8, device="cuda")
    d_text.copy_(pinned)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    dev_s, e2e_s = [], []
    for i in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        coll = ctx.parse((d_text.data_ptr(), n_bytes))
        dt = time.perf_counter() - t0
        if i == 0:
            tk, _, sz = coll.download()
            assert np.array_equal(tk, c.tokens) and np.array_equal(sz, c.sizes), "parse differs from the generator"
        coll.free()
        if i >= args.warmup:
            dev_s.append(dt)
    for i in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        coll = ctx.parse(text)
        dt = time.perf_counter() - t0
        coll.free()
        if i >= args.warmup:
            e2e_s.append(dt)
    dev, e2e = statistics.median(dev_s), statistics.median(e2e_s)
    # CPU: the reference reader's restatement on a bounded sample (first lines up to 128 MB)
    cut = int(text[:min(n_bytes, 128 << 20)].tobytes().rfind(b"\n")) + 1
    sample = text[:cut].tobytes()
    t0 = time.perf_counter()
    ct, cz, _ = oracle.read_text(sample)
    cpu_s = time.perf_counter() - t0
    assert np.array_equal(cz, c.sizes[:cz.size])
    peak, peak_kind = measured_peaks()
    alg = 2 * n_bytes + 4 * c.tokens.size + 12 * c.sizes.size  # two passes over the text, tokens, starts/sizes/meta
    print(json.dumps({
        "metric": "collection text parsed: bytes/s (read_collection on the GPU)", "value": n_bytes / dev / 1e9,
        "unit": "GB/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev * 1000,
        "higher_is_better": True, "dtype": "u8", "data": "synthetic (seeded generator, reference text format)",
        "config": {"workload": WORKLOAD.split(":")[0] + " as text", "text_bytes": n_bytes,
                   "tokens": int(c.tokens.size), "sets": int(c.sizes.size),
                   "timing": "host wall clock of the whole call (two launches, two synchronisations, validation)"},
        "roofline": {"bound": "hbm", "achieved": alg / dev / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg / dev / 1e9 / peak, "traffic": None, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_call": alg},
        "cpu_baseline": {"value": len(sample) / cpu_s / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                         "sample": f"first {len(sample) >> 20} MB of the text, oracle_read_text (getline/split/atoi)"},
        "e2e": {"value": n_bytes / e2e / 1e9, "unit": "GB/s", "h2d_bytes_per_step": n_bytes,
                "d2h_bytes_per_step": 32, "ms_per_step": e2e * 1000}}), flush=True)


def verify_candidates(c, n_probes=262144, per_probe=32, seed=0x5E7C, threshold=THRESHOLD):
    """Seeded candidate lists over the collection: sorted probe ids and, for
    each, `per_probe` candidates drawn uniformly from its length window (ids
    below the probe whose size is at least minsize(|probe|)), the shape of
    what a CPU filter hands the reference's device_handler."""
    import numpy as np
    from hyset_gb300 import similarity
    rng = np.random.default_rng(seed)
    n = c.n
    probes = np.sort(rng.choice(np.arange(1, n), size=min(n - 1, n_probes), replace=False)).astype(np.int64)
    sizes = c.sizes.astype(np.int64)
    minsize = np.array([similarity.minsize("jaccard", int(l), threshold) for l in range(int(sizes.max()) + 1)])
    lo = np.searchsorted(sizes, minsize[sizes[probes]], side="left")
    span = probes - lo
    keep = span > 0
    probes, lo, span = probes[keep], lo[keep], span[keep]
    cands = lo[:, None] + (rng.random((probes.size, per_probe)) * span[:, None]).astype(np.int64)
    offsets = np.arange(1, probes.size + 1, dtype=np.int64) * per_probe
    return probes.astype(np.uint32), offsets.astype(np.uint32), cands.reshape(-1).astype(np.uint32)


def run_verify(args):
    """The candidate verifier alone (hybrid::device_handler's kernels): seeded
    candidate lists of the 1M-set workload, resident in HBM, verified as the
    reference does (technique DIRECT: every candidate merged; a lane per
    candidate from staged prefixes, a warp per candidate, a plain lane per
    candidate) and with the XOR-signature bound first (AUTO: 256-bit
    signatures generated inside the timed call, then the staged lane mode).
    `value` is the fastest leg's candidates per second of device time."""
    import numpy as np
    import torch
    import hyset_gb300 as hs
    import oracle
    c = make_workload(args.sets or None)
    ctx = hs.Context(0)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    probes, offsets, cands = verify_candidates(c)
    t0 = time.perf_counter()
    exp, tokens_read = oracle.verify_csr((c.tokens, c.starts, c.sizes), probes, offsets, cands, THRESHOLD)
    cpu_s = time.perf_counter() - t0
    dp, do, dc = (torch.from_numpy(a.view(np.int32)).cuda() for a in (probes, offsets, cands))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    legs, bits = {}, {}
    for name, kw in (("staged_direct", dict(technique="direct", verify_mode=3)),
                     ("warp_direct", dict(technique="direct", verify_mode=2)),
                     ("lane_direct", dict(technique="direct", verify_mode=1)),
                     ("staged_signatures", dict(technique="auto", verify_mode=3))):
        km, dm = [], []
        for i in range(args.warmup + args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            r = ctx.verify_device(coll, dp.data_ptr(), do.data_ptr(), dc.data_ptr(), probes.size,
                                  threshold=THRESHOLD, **kw)
            if i == 0:
                assert oracle.as_set(r.pairs) == oracle.as_set(exp), f"verifier differs from the oracle ({name})"
            if i >= args.warmup:
                km.append(r.kernel_ms)
                dm.append(r.device_ms)
        legs[name] = {"kernel_ms": statistics.median(km), "device_ms": statistics.median(dm)}
        bits[name] = r.bitmap_bits
    best = min(legs, key=lambda k: legs[k]["device_ms"])
    dms, kms = legs[best]["device_ms"], legs[best]["kernel_ms"]
    peak, peak_kind = measured_peaks()
    C, P = int(cands.size), int(probes.size)
    # bytes the merges of the reference's verifier must read: tokens, ids, (start, size) records, pairs
    alg_direct = 4 * tokens_read + 4 * C + 8 * P + 8 * len(exp)
    w = bits["staged_signatures"] // 64
    # with the signature bound: ids, records and signatures of every candidate and probe, pairs
    # (the merges of the few candidates that pass the bound are not counted: a lower bound)
    alg_sig = 4 * C + 8 * C + 8 * w * C + (8 + 8 * w) * P + 8 * len(exp)
    alg = alg_sig if best == "staged_signatures" else alg_direct
    roof = {"bound": "hbm", "achieved": alg / kms / 1e6, "peak": peak, "unit": "GB/s",
            "frac": alg / kms / 1e6 / peak, "traffic": None, "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": alg, "kernel": f"k_verify_candidates ({best})"}
    print(json.dumps({
        "metric": "candidate pairs verified/s (hybrid::device_handler verifier)", "value": C / dms * 1e3,
        "unit": "pairs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dms,
        "higher_is_better": True, "dtype": "u32", "data": "synthetic (seeded generator and candidate lists)",
        "config": {"workload": WORKLOAD.split(":")[0] + ": candidate lists", "probes": P, "candidates": C,
                   "result_pairs": int(len(exp)), "tokens_read_by_merges": int(tokens_read), "legs": legs,
                   "best": best, "signature_bits": bits["staged_signatures"],
                   "direct_roofline_frac": alg_direct / legs["staged_direct"]["kernel_ms"] / 1e6 / peak,
                   "l2": "512 MB buffer written between timed steps"},
        "roofline": roof,
        "cpu_baseline": {"value": C / cpu_s, "unit": "pairs/s", "cores": 1, "kind": "port",
                         "sample": "all candidate lists once (oracle_verify_csr, verification.hpp:9-31)"}}),
          flush=True)


def run_configs(args):
    """--workload c1 / c2: the two smaller self-join configurations, each leg
    timed with the collection resident (CUDA events, L2 flushed, median of
    --steps after --warmup), every leg's pair set checked against the oracle.

    c1: 10,000 sets, Jaccard 0.8: the plain single-launch GPU path and AUTO
    against the reference algorithm on one host core (cpu_single) and on all
    of them (cpu_multi).
    c2: 200,000 sets, Jaccard 0.5 / 0.7 / 0.9: the reference's two GPU
    techniques, bitmap signatures of 64 and 256 bits and the prefix filter,
    beside AUTO."""
    import numpy as np
    import torch
    import hyset_gb300 as hs
    import oracle
    from hyset_gb300 import synth

    spec, taus = (synth.C1, [0.8]) if args.workload == "c1" else (synth.C2, [0.5, 0.7, 0.9])
    c = synth.generate(spec)
    ctx = hs.Context(0)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    threads = os.cpu_count() or 1
    peak, peak_kind = measured_peaks()

    def keys(p):
        p = np.asarray(p, np.uint64).reshape(-1, 2)
        return np.sort((p[:, 0] << np.uint64(32)) | p[:, 1])

    if args.workload == "c1":
        legs = {"plain_single_launch": dict(technique="fgss", probe_major=True, bitmap=0, verify_mode=1, fgss_batch=1),
                "auto": dict(technique="auto")}
    else:
        legs = {"bitmap64": dict(technique="bitmap", bitmap=64), "bitmap256": dict(technique="bitmap", bitmap=256),
                "fgss": dict(technique="fgss", probe_major=True), "auto": dict(technique="auto")}
    rows, launches, parity, headline = [], 0, True, None
    for tau in taus:
        exp = keys(oracle.join(c.tokens, c.starts, c.sizes, tau))
        idx_s, join_s = oracle.last_timing()
        cpu1_s = idx_s + join_s
        oracle.join_multi(c.tokens, c.starts, c.sizes, tau, threads)
        idx_s, join_s = oracle.last_timing(multi=True)
        cpun_s = idx_s + join_s
        row = {"threshold": tau, "result_pairs": int(exp.size), "cpu_single_ms": 1000 * cpu1_s,
               "cpu_multi_ms": 1000 * cpun_s, "cpu_threads": threads}
        for name, q in legs.items():
            kw = dict(threshold=tau, device_pairs=True, **q)
            r = ctx.self_join(coll, **dict(kw, device_pairs=False))
            ok = bool(np.array_equal(keys(r.pairs), exp))
            parity &= ok
            st = ctx.self_join(coll, collect_stats=True, **kw)
            for _ in range(args.warmup):
                ctx.self_join(coll, **kw)
            dev, kern = [], []
            for _ in range(args.steps):
                flush.fill_(1)
                torch.cuda.synchronize()
                x = ctx.self_join(coll, **kw)
                dev.append(x.device_ms)
                kern.append(x.kernel_ms)
                launches += x.launches
            leg = {"ms": statistics.median(dev), "kernel_ms": statistics.median(kern), "parity": ok,
                   "technique": st.technique, "bitmap_bits": st.bitmap_bits, "verify_mode": st.verify_mode,
                   "probe_batch": st.probe_batch}
            if st.technique == "fgss":
                alg = algorithmic_bytes(st.stats, st.count, st.bitmap_bits // 64, c.n)
                leg["roofline_frac"] = alg / (leg["kernel_ms"] / 1000.0) / 1e9 / peak
                leg["algorithmic_bytes"] = alg
            else:
                leg["window_pairs_per_s"] = st.stats[0] / (leg["kernel_ms"] / 1000.0)
            row[name] = leg
        rows.append(row)
        if headline is None or tau == 0.7:
            headline = (tau, row)
    tau, row = headline
    auto = row["auto"]
    line = {"metric": f"self-join ms & verified pairs/s, {args.workload} configuration, 1 GB300",
            "value": row["result_pairs"] / (auto["ms"] / 1000.0), "unit": "pairs/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": auto["ms"], "higher_is_better": True,
            "dtype": "u32", "data": "synthetic (seeded generator)",
            "config": {"workload": ("10,000 sets, sizes U[5,50], universe 5,000, Zipf 1.0, Jaccard 0.8"
                                    if args.workload == "c1" else
                                    "200,000 sets, lognormal(3.2,0.6) sizes in [2,500], universe 100,000, "
                                    "Zipf 1.1, 3% near-duplicates; Jaccard 0.5 / 0.7 / 0.9"),
                       "headline_threshold": tau, "thresholds": rows,
                       "l2": "512 MB buffer written between timed steps"},
            "roofline": {"bound": "hbm", "frac": auto.get("roofline_frac"), "peak": peak, "unit": "GB/s",
                         "peak_kind": peak_kind, "traffic": None,
                         "kernel": "AUTO leg's filter+verify launch"},
            "cpu_baseline": {"value": row["result_pairs"] / (row["cpu_single_ms"] / 1000.0), "unit": "pairs/s",
                             "cores": 1, "kind": "port",
                             "sample": "whole workload (index + join), oracle restatement of host::allpairs"},
            "parity": parity, "gpu_launches": launches}
    print(json.dumps(line), flush=True)
    coll.free()
    ctx.close()
    if not parity:
        sys.exit("parity failure")


def hs_text_bytes(c):
    from hyset_gb300 import synth
    lib = synth._load()
    import ctypes as C
    U32 = C.POINTER(C.c_uint32)
    return lib.hyset_format_text(c.tokens.ctypes.data_as(U32), c.starts.ctypes.data_as(U32),
                                 c.sizes.ctypes.data_as(U32), c.sizes.size, None, 0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--technique", default="auto")
    ap.add_argument("--sim", default="jaccard", choices=["jaccard", "cosine", "dice"])
    ap.add_argument("--bitmap", type=int, default=0, help="signature bits; 0 = the library's autotuner")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the block-pair baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-join batch leg")
    ap.add_argument("--sets", type=int, default=0, help="smaller case of the same workload (profiling)")
    ap.add_argument("--probe-major", action="store_true", help="FGSS: probe-major kernel instead of token-major")
    ap.add_argument("--batch", type=int, default=0, help="probe batch of the probe-major kernel; 0 = the autotuner")
    ap.add_argument("--vmode", type=int, default=0,
                    help="verification: 0 auto (the autotuner's samples choose), 1 lane, 2 warp per candidate")
    ap.add_argument("--workload", default="selfjoin", choices=["selfjoin", "batch", "parse", "verify", "c1", "c2"],
                    help="batch: the batched R-S workload; parse: the collection text reader; verify: the "
                         "candidate verifier alone; c1 / c2: the 10K-set and 200K-set configurations "
                         "(separate measurements, not the headline)")
    ap.add_argument("--joins", type=int, default=256)
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "parse":
        run_parse(args)
        return
    if args.workload == "verify":
        run_verify(args)
        return
    if args.workload in ("c1", "c2"):
        run_configs(args)
        return
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()

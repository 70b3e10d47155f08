"""Learned signature width for the prefix-filter join.

    python -m hyset_gb300.width_selector train [--collections 80] [--train 64] [--out DIR]

On the technique selector's grid of collections with 50,000 to 1,000,000 sets
(selector.grid, the same seeded configurations) the prefix filter is always
the fastest technique, so the technique network gains nothing there: it, the
rules and the cost model all pick it.  What does vary at that scale is the
width of the XOR signatures checked before verification (none, 128, 256 or
512 bits: on the 200,000-set workload at Jaccard 0.5 the join takes 3.2 ms
without signatures and 1.75 ms with 512 bits).  The library's autotuner finds
the width by timing samples of the probe range on the first join of a key;
this module trains a second network of the selector's shape (12 features ->
64 -> 64 -> 3, ReLU, trained on the GPU by hyset_mlp_train) to predict the
join's log-time at 128, 256 and 512 bits instead, so that a first join needs
no width samples:

  1. each grid collection's self-join is timed with the probe-major prefix
     filter (a lane per candidate, batch 3) at 0, 128, 256 and 512 bits
     (whole join, device time, best of three after a warm-up), and once with
     AUTO and no network installed, whose choice is the sampling autotuner's;
  2. the network is trained on the first `--train` collections;
  3. on the held-out collections each chooser's regret against the fastest
     width is reported: the network, the fixed rule (128 bits for mean sizes up
     to 48, else 256), 256 bits always, no signatures, and the autotuner.

The result ships as width_weights.json; Context() installs it
(hyset_width_selector_set).  The width never changes a join's output.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import selector

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "width_weights.json")
WIDTHS = [128, 256, 512]  # the network's outputs
TIMED = [0, 128, 256, 512]


def install_shipped(ctx, path: str = WEIGHTS):
    """Installs the shipped width network in a Context; returns its report or None."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        w = json.load(f)
    ctx.width_selector_set(np.array(w["params"], np.float32), np.array(w["mean"], np.float32),
                           np.array(w["scale"], np.float32))
    return {k: w[k] for k in ("trained_on", "held_out", "report") if k in w}


def time_widths(ctx, coll, tau, sim, reps=3):
    """Device milliseconds of the whole self-join at each timed width."""
    out = []
    for bits in TIMED:
        kw = dict(threshold=tau, sim=sim, technique="fgss", probe_major=True, verify_mode=1, fgss_batch=3,
                  bitmap=bits, device_pairs=True)
        ctx.self_join(coll, **kw)
        out.append(min(ctx.self_join(coll, **kw).device_ms for _ in range(reps)))
    return out


def collect(ctx, cfgs, log=print):
    rows = []
    for i, cfg in enumerate(cfgs):
        t0 = time.time()
        c = selector.make_collection(cfg)
        sim, tau = cfg["sim"], cfg["tau"]
        coll = ctx.upload(c.tokens, c.sizes, c.starts)
        f, base = ctx.features(coll, None, threshold=tau, sim=sim)
        ms = time_widths(ctx, coll, tau, sim)
        # the sampling autotuner's choice (AUTO, no network installed) and what
        # its first join costs on the host clock beyond a repeat of the join
        w0 = time.perf_counter()
        r1 = ctx.self_join(coll, threshold=tau, sim=sim, device_pairs=True)
        first = time.perf_counter() - w0
        w0 = time.perf_counter()
        r2 = ctx.self_join(coll, threshold=tau, sim=sim, device_pairs=True)
        again = time.perf_counter() - w0
        coll.free()
        rows.append(dict(collection=i, cfg=cfg, features=f.tolist(), base=base.tolist(), ms=ms,
                         autotuner_bits=r1.bitmap_bits, auto_technique=r1.technique,
                         auto_first_s=first, auto_repeat_s=again, auto_ms=r2.device_ms))
        log(f"[{i + 1}/{len(cfgs)}] n={c.n} mean={cfg['mean']:.0f} zipf={cfg['zipf']:.2f} {sim} tau={tau} "
            f"ms(0,128,256,512)={[round(x, 3) for x in ms]} autotuner={r1.bitmap_bits} "
            f"({time.time() - t0:.1f}s)")
    return rows


def rule_bits(row):
    return 128 if row["base"][1] <= 48.0 else 256


def train(ctx, rows, steps=3000, lr=2e-3, weight_decay=1e-4, seed=0):
    X = np.array([r["features"] for r in rows], np.float32)
    Y = np.log(np.maximum(np.array([r["ms"][1:] for r in rows], np.float64), 1e-3)).astype(np.float32)
    M = np.ones_like(Y, np.float32)
    mean = X.mean(axis=0)
    scale = np.where(X.std(axis=0) > 1e-6, X.std(axis=0), 1.0).astype(np.float32)
    Xn = ((X - mean) / scale).astype(np.float32)
    params, trace = ctx.mlp_train(selector.init_params(seed), Xn, Y, M, steps, lr, weight_decay)
    return params, mean, scale, trace


def evaluate(ctx, params, mean, scale, rows):
    """Regret of each chooser against the fastest timed width (none included)."""
    X = ((np.array([r["features"] for r in rows], np.float32) - mean) / scale).astype(np.float32)
    pred = ctx.mlp_forward(params, X)
    out = {"network": [], "rule": [], "bits_256": [], "no_signatures": [], "autotuner": []}
    for r, p in zip(rows, pred):
        ms = dict(zip(TIMED, r["ms"]))
        best = min(ms.values())
        picks = {"network": WIDTHS[int(np.argmin(p))], "rule": rule_bits(r), "bits_256": 256, "no_signatures": 0,
                 "autotuner": r["autotuner_bits"] if r["autotuner_bits"] in ms else 256}
        for k, b in picks.items():
            out[k].append(ms[b] / best - 1.0)
    return {k: {"mean_regret": float(np.mean(v)), "max_regret": float(np.max(v)),
                "optimal_fraction": float(np.mean(np.array(v) < 1e-9))} for k, v in out.items()}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--collections", type=int, default=80)
    ap.add_argument("--train", type=int, default=64)
    ap.add_argument("--steps", type=int, default=3000)
    args = ap.parse_args(argv)
    from .api import Context
    ctx = Context(0, selector=True, width=False)  # the technique network as shipped; widths by sampling
    rows = collect(ctx, selector.grid(args.collections))
    tr, te = rows[:args.train], rows[args.train:]
    params, mean, scale, trace = train(ctx, tr, steps=args.steps)
    tuning = [max(0.0, r["auto_first_s"] - r["auto_repeat_s"]) for r in te]
    report = {"held_out": evaluate(ctx, params, mean, scale, te), "train": evaluate(ctx, params, mean, scale, tr),
              "held_out_autotuner_first_join_extra_s": {"mean": float(np.mean(tuning)), "max": float(np.max(tuning))},
              "techniques_chosen_by_auto": sorted({r["auto_technique"] for r in rows}),
              "final_loss": float(trace[-1]) if len(trace) else None, "first_loss": float(trace[0])}
    os.makedirs(args.out, exist_ok=True)
    with open(os.path.join(args.out, "width_weights.json"), "w") as f:
        json.dump({"params": params.tolist(), "mean": mean.tolist(), "scale": scale.tolist(), "widths": WIDTHS,
                   "trained_on": len(tr), "held_out": len(te), "report": report}, f)
    with open(os.path.join(args.out, "width_samples.json"), "w") as f:
        json.dump(rows, f)
    print(json.dumps(report, indent=1))


if __name__ == "__main__":
    main()

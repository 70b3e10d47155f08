"""Technique selector: a small FP32 network trained on timings this library measures.

    python -m hyset_gb300.selector train [--out DIR] [--collections 80] [--train 64] [--rs 80]

The reference chooses a GPU technique per partition pair with an analytic linear
cost model whose coefficients it does not ship (include/hyset/cost.hpp:28-58,
src/cost_model.cu:296-323).  Here:
  1. a seeded grid of collections (Zipf s in [0.6, 1.4], mean set size in
     [10, 300], n in [50k, 1M] and [1k, 50k], threshold in [0.5, 0.95], Jaccard,
     cosine or dice) is generated for self-joins, and a grid of R-S joins
     (one collection split in two, |R|/|S| in [1/50, 1], 2k-400k sets in
     all) in the orientation the library runs them (the smaller side indexed);
  2. each join is timed on the GPU with each technique (bitmap, fgss,
     direct-verify), on evenly spread probe ranges, extrapolated to the whole
     probe set, plus the technique's full-size preparation (index build,
     signatures); the two halves of the probe range are extra samples;
  3. the network 12 -> 64 -> 64 -> 3 (log-milliseconds per technique) is trained
     on the GPU by this library's kernels (hyset_mlp_train), and the reference's
     analytic model is fitted by least squares on the same timings;
  4. on the held-out collections the regret of each chooser against the fastest
     technique is reported.
The trained selector ships as selector_weights.json; Context() installs it for
technique AUTO.  The choice never changes a join's output.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np

from ._lib import COST_TERMS, MLP_PARAMS, N_FEATURES

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "selector_weights.json")
TECHNIQUES = ["bitmap", "fgss", "direct"]  # the network's output order
F, H, O = N_FEATURES, 64, 3


def init_params(seed: int = 0) -> np.ndarray:
    """He-initialised parameters in the library's flat layout."""
    rng = np.random.default_rng(seed)
    parts = [rng.normal(0, math.sqrt(2.0 / F), (F, H)), np.zeros(H),
             rng.normal(0, math.sqrt(2.0 / H), (H, H)), np.zeros(H),
             rng.normal(0, math.sqrt(1.0 / H), (H, O)), np.zeros(O)]
    p = np.concatenate([a.ravel() for a in parts]).astype(np.float32)
    assert p.size == MLP_PARAMS
    return p


def install_shipped(ctx, path: str = WEIGHTS):
    """Installs the shipped selector in a Context; returns its metadata or None."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        w = json.load(f)
    params = np.array(w["params"], np.float32) if w.get("params") else None
    cost = np.array(w["cost"], np.float64).reshape(3, COST_TERMS) if w.get("cost") else None
    ctx.selector_set(params, np.array(w["mean"], np.float32), np.array(w["scale"], np.float32), cost)
    return {k: w[k] for k in ("trained_on", "held_out", "report") if k in w}


# ------------------------------------------------------------------ training data

SIMS = ["jaccard", "cosine", "dice"]


def grid(n_collections: int, seed: int = 2024, n_lo: int = 50_000, n_hi: int = 1_000_000, rs: bool = False):
    """Seeded grid configurations (ordered; the last ones are held out).  With
    rs=True each configuration is an R-S join: n_sets in all, split so that the
    smaller side holds r_frac of them."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n_collections:
        n = int(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi))))
        mean = math.exp(rng.uniform(math.log(10), math.log(300)))
        if n * mean > 8e7:  # keep every collection within a few hundred MB
            continue
        cfg = dict(n_sets=n, mean=mean, zipf=float(rng.uniform(0.6, 1.4)),
                   tau=round(float(rng.uniform(0.5, 0.95)), 3),
                   universe=int(math.exp(rng.uniform(math.log(50_000), math.log(1_000_000)))),
                   seed=int(rng.integers(1, 2**31)), sim=SIMS[int(rng.integers(0, 3))])
        if rs:
            ratio = math.exp(rng.uniform(math.log(1 / 50), 0.0))  # |R| / |S|
            cfg["r_frac"] = ratio / (1.0 + ratio)
        out.append(cfg)
    return out


def make_collection(cfg):
    from . import synth
    spec = dict(n_sets=cfg["n_sets"], universe=max(cfg["universe"], int(4 * cfg["mean"])),
                zipf_s=cfg["zipf"], size_dist=synth.LOGNORMAL, size_a=math.log(cfg["mean"]) - 0.18,
                size_b=0.6, size_min=2, size_max=min(2000, max(10, int(cfg["mean"] * 8))),
                dup_frac=0.03, dup_edit_lo=0.02, dup_edit_hi=0.15, seed=cfg["seed"])
    return synth.generate(synth.C2, **spec)


def split_collection(c, frac, seed):
    """(R, S) host triples (tokens, starts, sizes): each set of c goes to R with
    probability frac, so near-duplicates land on both sides."""
    side = np.random.default_rng(seed).random(c.n) < frac
    out = []
    for mask in (side, ~side):
        ids = np.nonzero(mask)[0]
        sizes = c.sizes[ids]
        starts = np.zeros(len(ids), np.uint32)
        if len(ids):
            starts[1:] = np.cumsum(sizes[:-1])
        sz = sizes.astype(np.int64)
        src = np.repeat(c.starts[ids].astype(np.int64) - starts.astype(np.int64), sz) + np.arange(int(sz.sum()))
        out.append((c.tokens[src], starts, sizes))
    return out


def _chunks(n, k, per):
    """k evenly spread probe ranges of `per` probes."""
    per = max(1, min(per, n // k if n >= k else n))
    starts = np.linspace(0, max(0, n - per), k).astype(np.int64)
    return [(int(s), int(s) + per) for s in starts]


def time_techniques(join, n, window_pairs, sample_probes=48_000, k=8, pair_budget=2e7):
    """Estimated whole-join milliseconds per technique, for the whole probe
    range and for its two halves: {part: [bitmap, fgss, direct]}.  `join(probe_range,
    **kw)` runs the join over a probe range of its n probes.  The enumeration
    techniques sample fewer probes where length windows are long (about
    pair_budget length-compatible pairs per chunk)."""
    half = n // 2
    est = {"all": [], "low": [], "high": []}
    per_probe = max(1.0, window_pairs / max(n, 1))
    for tech in TECHNIQUES:
        per = sample_probes // k if tech == "fgss" else int(max(1, min(sample_probes // k, pair_budget / per_probe)))
        chunks = _chunks(n, k, per)
        kw = dict(technique=tech, device_pairs=True, count_only=False)
        if tech == "fgss":
            kw.update(probe_major=True)
        # preparation of the whole collection (index build / signatures) from a one-probe call
        r0 = join((n - 1, n), **kw)
        prep = max(0.0, r0.device_ms - r0.kernel_ms)
        ks = []
        for lo, hi in chunks:
            best = None
            for _ in range(2):
                r = join((lo, hi), **kw)
                best = r.kernel_ms if best is None else min(best, r.kernel_ms)
            ks.append((lo, hi, best))
        for part, (plo, phi) in (("all", (0, n)), ("low", (0, half)), ("high", (half, n))):
            sel = [(hi - lo, ms) for lo, hi, ms in ks if lo >= plo and hi <= phi]
            probes = sum(p for p, _ in sel)
            kern = sum(ms for _, ms in sel)
            span = phi - plo
            est[part].append(prep + (kern * span / probes if probes else float("nan")))
    return est


def collect(ctx, cfgs, log=print, first_id=0):
    """Features and per-technique times of every configuration: a self-join,
    or (cfg with r_frac) an R-S join with the smaller side indexed."""
    rows = []
    for i, cfg in enumerate(cfgs):
        t0 = time.time()
        c = make_collection(cfg)
        sim, tau = cfg.get("sim", "jaccard"), cfg["tau"]
        if "r_frac" in cfg:
            (rt, rs_, rz), (st, ss, sz) = split_collection(c, cfg["r_frac"], cfg["seed"] + 1)
            R, S = ctx.upload(rt, rz, rs_), ctx.upload(st, sz, ss)
            n = S.n

            def join(pr, **kw):
                return ctx.rs_join(R, S, threshold=tau, sim=sim, probe_range=pr, orientation="as_given", **kw)
            colls = [R, S]
        else:
            R = S = ctx.upload(c.tokens, c.sizes, c.starts)
            n = c.n

            def join(pr, **kw):
                return ctx.self_join(R, threshold=tau, sim=sim, probe_range=pr, **kw)
            colls = [R]
        feats = {}
        for part, rng_ in (("all", None), ("low", (0, n // 2)), ("high", (n // 2, n))):
            f, base = ctx.features(R, None if S is R else S, threshold=tau, sim=sim, probe_range=rng_)
            feats[part] = (f.tolist(), base.tolist())
        times = time_techniques(join, n, feats["all"][1][6])
        for part in ("all", "low", "high"):
            rows.append(dict(collection=first_id + i, part=part, cfg=cfg, features=feats[part][0],
                             base=feats[part][1], ms=times[part]))
        for x in colls:
            x.free()
        kind = f"R-S {R.n}x{S.n}" if "r_frac" in cfg else f"self n={n}"
        log(f"[{i + 1}/{len(cfgs)}] {kind} mean={cfg['mean']:.0f} zipf={cfg['zipf']:.2f} {sim} tau={tau} "
            f"ms(bitmap,fgss,direct)={[round(x, 3) for x in times['all']]} ({time.time() - t0:.1f}s)")
    return rows


# ------------------------------------------------------------------ models

def fit_cost_model(rows):
    """Least-squares fit of the reference's analytic form per technique:
    ms ~ c . (1, size std, avg size, token-frequency std, n, n^2, universe, index, bitmap)."""
    coefs = np.zeros((3, COST_TERMS))
    for t in range(3):
        X, y = [], []
        for r in rows:
            b = r["base"]
            bits = (128.0 if b[1] <= 48 else 256.0) if t == 0 else 0.0
            X.append([1.0, b[0], b[1], b[2], b[3], b[3] ** 2, b[4], b[5], bits])
            y.append(r["ms"][t])
        X, y = np.array(X), np.array(y)
        scale = np.maximum(np.abs(X).max(axis=0), 1e-12)
        sol, *_ = np.linalg.lstsq(np.vstack([X / scale, 1e-3 * np.eye(COST_TERMS)]),
                                  np.concatenate([y, np.zeros(COST_TERMS)]), rcond=None)
        coefs[t] = sol / scale
    return coefs


def cost_predict(coefs, base):
    out = []
    for t in range(3):
        bits = (128.0 if base[1] <= 48 else 256.0) if t == 0 else 0.0
        x = np.array([1.0, base[0], base[1], base[2], base[3], base[3] ** 2, base[4], base[5], bits])
        out.append(abs(float(coefs[t] @ x)))
    return out


def rules_choice(row):
    """The method without a learned model: the library's fixed rules."""
    b = row["base"]
    return 0 if b[3] * b[3] <= 4e6 else 1  # enumerate tiny joins with signatures, else the prefix index


def train(ctx, rows_train, steps=3000, lr=2e-3, weight_decay=1e-4, seed=0):
    X = np.array([r["features"] for r in rows_train], np.float32)
    Y = np.log(np.maximum(np.array([r["ms"] for r in rows_train], np.float64), 1e-3)).astype(np.float32)
    M = np.isfinite(Y).astype(np.float32)
    Y = np.where(np.isfinite(Y), Y, 0.0).astype(np.float32)
    mean = X.mean(axis=0)
    scale = np.where(X.std(axis=0) > 1e-6, X.std(axis=0), 1.0).astype(np.float32)
    Xn = ((X - mean) / scale).astype(np.float32)
    params, trace = ctx.mlp_train(init_params(seed), Xn, Y, M, steps, lr, weight_decay)
    return params, mean, scale, trace


def evaluate(ctx, params, mean, scale, coefs, rows):
    X = ((np.array([r["features"] for r in rows], np.float32) - mean) / scale).astype(np.float32)
    pred = ctx.mlp_forward(params, X)
    out = {"mlp": [], "cost_model": [], "rules": [], "fgss_always": []}
    for r, p in zip(rows, pred):
        ms = np.array(r["ms"])
        best = float(np.nanmin(ms))
        picks = {"mlp": int(np.argmin(p)), "cost_model": int(np.argmin(cost_predict(coefs, r["base"]))),
                 "rules": rules_choice(r), "fgss_always": 1}
        for k, c in picks.items():
            out[k].append(float(ms[c] / best - 1.0))
    return {k: {"mean_regret": float(np.mean(v)), "max_regret": float(np.max(v)),
                "optimal_fraction": float(np.mean(np.array(v) < 1e-9))} for k, v in out.items()}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--collections", type=int, default=80)
    ap.add_argument("--train", type=int, default=64)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--small", type=int, default=40,
                    help="extra collections with 1k-50k sets (the batched R-S joins' range)")
    ap.add_argument("--small-train", type=int, default=32)
    ap.add_argument("--rs", type=int, default=80, help="R-S joins (2k-400k sets split in two)")
    ap.add_argument("--rs-train", type=int, default=56)
    args = ap.parse_args(argv)
    from .api import Context
    ctx = Context(0, selector=False)
    cfgs = grid(args.collections)
    small = grid(args.small, seed=4048, n_lo=1_000, n_hi=50_000)
    rs = grid(args.rs, seed=6072, n_lo=2_000, n_hi=400_000, rs=True)
    rows = collect(ctx, cfgs + small + rs)
    nb, ns = args.collections, args.small
    family = lambda r: "grid" if r["collection"] < nb else ("small" if r["collection"] < nb + ns else "rs")
    is_train = lambda r: {"grid": r["collection"] < args.train,
                          "small": r["collection"] - nb < args.small_train,
                          "rs": r["collection"] - nb - ns < args.rs_train}[family(r)]
    for r in rows:
        r["family"], r["train"] = family(r), bool(is_train(r))
    tr = [r for r in rows if r["train"]]
    te = [r for r in rows if not r["train"]]
    params, mean, scale, trace = train(ctx, tr, steps=args.steps)
    coefs = fit_cost_model(tr)
    whole = lambda rs_: [r for r in rs_ if r["part"] == "all"]
    ev = lambda sel: evaluate(ctx, params, mean, scale, coefs, sel)
    report = {"held_out": ev(whole(te)),
              "held_out_grid_50k_1m": ev([r for r in whole(te) if family(r) == "grid"]),
              "held_out_small_1k_50k": ev([r for r in whole(te) if family(r) == "small"]),
              "held_out_rs": ev([r for r in whole(te) if family(r) == "rs"]),
              "held_out_partitions": ev(te),
              "train": evaluate(ctx, params, mean, scale, coefs, whole(tr)),
              "final_loss": float(trace[-1]) if len(trace) else None, "first_loss": float(trace[0])}
    os.makedirs(args.out, exist_ok=True)
    with open(os.path.join(args.out, "selector_weights.json"), "w") as f:
        json.dump({"params": params.tolist(), "mean": mean.tolist(), "scale": scale.tolist(),
                   "cost": coefs.ravel().tolist(), "techniques": TECHNIQUES,
                   "trained_on": args.train + args.small_train + args.rs_train,
                   "held_out": nb - args.train + ns - args.small_train + args.rs - args.rs_train,
                   "report": report}, f)
    with open(os.path.join(args.out, "selector_samples.json"), "w") as f:
        json.dump(rows, f)
    print(json.dumps(report, indent=1))


if __name__ == "__main__":
    main()

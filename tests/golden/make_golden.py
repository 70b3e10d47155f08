"""Generates the golden fixtures in this directory from the REFERENCE itself.

Each fixture is a small collection in the reference's text format plus the
pairs that the reference's own hyset::algorithms::host::allpairs (whole
collection, as src/cpu_single.cu runs it) and host::ppjoin (per length-filtered
block pair, as src/queue.cu runs it) emit on it.  The reference code runs
through oracle/_ref/ref_join (built by `make -C oracle ref` from the reference
headers, see oracle/ref_driver.cu); both runs must agree before a fixture is
written.  The reference only implements jaccard.

    python tests/golden/make_golden.py       # needs oracle/_ref/ref_join

Fixture layout (<name>.sets.txt, <name>.json):
    sets.txt   one set per line, ascending tokens, lines ordered by size
    json       {"results": {"<tau>": {"count": N, "pairs": [[probe, indexed], ...]}}}
               pairs sorted by (probe, indexed)
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from hyset_gb300 import synth  # noqa: E402


def write_sets(path, sets):
    with open(path, "w") as f:
        for s in sets:
            f.write(" ".join(map(str, s)) + "\n")


def collection_sets(c):
    return [c.set(i).tolist() for i in range(c.n)]


def edge_sets(tau: float, seed: int):
    """Pairs whose overlap equals the exact rational threshold at sizes where the
    reference's double minoverlap rounds up (so the reference rejects them), and
    pairs one token above it (accepted)."""
    rng = np.random.default_rng(seed)
    sums = []
    for s in range(4, 400):
        exact_num = s * round(tau * 100)
        den = round((1 + tau) * 100)
        if exact_num % den == 0:
            k = exact_num // den
            if math.ceil(float(s) * tau / (1 + tau)) != k:
                sums.append((s, k))
    sets, next_tok = [], 1
    for s, k in sums[:12]:
        l1 = s // 2
        l2 = s - l1
        for extra in (0, 1):
            ov = min(k + extra, l1)
            common = list(range(next_tok, next_tok + ov))
            next_tok += ov
            a = common + list(range(next_tok, next_tok + l1 - ov)); next_tok += l1 - ov
            b = common + list(range(next_tok, next_tok + l2 - ov)); next_tok += l2 - ov
            sets.append(sorted(a))
            sets.append(sorted(b))
    # duplicates and subsets
    base = sorted(rng.choice(np.arange(next_tok, next_tok + 500), 20, replace=False).tolist())
    sets += [base, list(base), base[:-1], base[:-2] + [next_tok + 600]]
    sets.sort(key=lambda x: (len(x), x))
    return sets, sums


DATASETS = {
    "toy": (lambda: [[1, 2, 3], [1, 2, 3], [1, 2, 3, 4], [2, 3, 4, 5, 6]], [0.5, 0.7]),
    "c1_small": (lambda: collection_sets(synth.generate(synth.C1, n_sets=1500, universe=2500, dup_frac=0.05,
                                                        dup_edit_lo=0.0, dup_edit_hi=0.3, seed=11)),
                 [0.5, 0.6, 0.7, 0.75, 0.8, 0.85, 0.9, 0.95]),
    "zipf_long": (lambda: collection_sets(synth.generate(synth.C3, n_sets=800, universe=20000, size_a=4.2,
                                                         size_b=0.6, size_max=400, dup_frac=0.1, seed=12)),
                  [0.6, 0.8, 0.9]),
    "edge_080": (lambda: edge_sets(0.8, 13)[0], [0.8]),
    "edge_090": (lambda: edge_sets(0.9, 14)[0], [0.9]),
}


def main():
    if not oracle.ref_available():
        sys.exit("oracle/_ref/ref_join is missing: run `make -C oracle ref` where the reference sources exist")
    for name, (make, taus) in DATASETS.items():
        sets = make()
        path = os.path.join(HERE, f"{name}.sets.txt")
        write_sets(path, sets)
        results = {}
        for tau in taus:
            a = oracle.ref_join(path, tau, "allpairs", "whole")
            b = oracle.ref_join(path, tau, "ppjoin", "blocks", 97)
            if oracle.as_set(a) != oracle.as_set(b) or len(a) != len(oracle.as_set(a)):
                raise SystemExit(f"{name} tau={tau}: reference allpairs and ppjoin disagree")
            p = sorted(oracle.as_set(a))
            results[repr(tau)] = {"count": len(p), "pairs": [list(x) for x in p]}
            print(f"{name:10s} tau={tau}: {len(p)} pairs")
        with open(os.path.join(HERE, f"{name}.json"), "w") as f:
            json.dump({"source": "reference host::allpairs (whole) == host::ppjoin (blocks of 97)",
                       "results": results}, f, separators=(",", ":"))


if __name__ == "__main__":
    main()

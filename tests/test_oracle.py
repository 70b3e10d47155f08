"""The CPU oracle pinned against the reference's own outputs (CPU only)."""
import math
import os
import tempfile

import numpy as np
import pytest

import oracle
from conftest import GOLDEN_SETS, load_golden
from hyset_gb300 import similarity, synth


@pytest.mark.parametrize("name", GOLDEN_SETS)
def test_oracle_matches_reference_golden(name):
    tokens, starts, sizes, results = load_golden(name)
    for tau, want in results.items():
        exp = {tuple(p) for p in want["pairs"]}
        assert len(exp) == want["count"]
        for algo in ("allpairs", "ppjoin"):
            got = oracle.join(tokens, starts, sizes, tau, algorithm=algo)
            assert len(got) == want["count"], (name, tau, algo)
            assert oracle.as_set(got) == exp, (name, tau, algo)
        assert oracle.as_set(oracle.brute(tokens, starts, sizes, tau)) == exp, (name, tau, "brute")
        assert oracle.as_set(oracle.join_multi(tokens, starts, sizes, tau, 3)) == exp, (name, tau, "multi")


def test_toy_counts():
    tokens, starts, sizes, results = load_golden("toy")
    assert results[0.7]["count"] == 3 and results[0.5]["count"] == 4


def test_edge_fixture_exercises_double_rounding():
    """The edge fixture holds pairs at sizes where the reference's double
    minoverlap is one above the exact rational bound; the reference rejects
    them and so must every path."""
    tokens, starts, sizes, results = load_golden("edge_080")
    bumped = 0
    for i in range(len(sizes)):
        for j in range(i):
            a = set(tokens[starts[i]:starts[i] + sizes[i]].tolist())
            b = set(tokens[starts[j]:starts[j] + sizes[j]].tolist())
            o = len(a & b)
            s = int(sizes[i] + sizes[j])
            exact = -(-s * 80 // 180)  # ceil(s * 0.8 / 1.8) in integers
            if o == exact and similarity.minoverlap("jaccard", int(sizes[i]), int(sizes[j]), 0.8) == exact + 1:
                bumped += 1
                assert (i, j) not in {tuple(p) for p in results[0.8]["pairs"]}
    assert bumped >= 3


@pytest.mark.skipif(not oracle.ref_available(), reason="reference build (oracle/_ref) not present")
@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_matches_live_reference(seed):
    c = synth.generate(synth.C1, n_sets=1200, universe=1500, dup_frac=0.08, dup_edit_lo=0.0, dup_edit_hi=0.3,
                       seed=seed)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "c.txt")
        c.write_text(path)
        for tau in (0.55, 0.8, 0.9):
            ref = oracle.ref_join(path, tau, "allpairs")
            got = oracle.join(c.tokens, c.starts, c.sizes, tau)
            assert oracle.as_set(ref) == oracle.as_set(got)


@pytest.mark.parametrize("sim", ["jaccard", "cosine", "dice"])
def test_host_bounds_match_oracle(sim):
    for tau in (0.5, 0.61, 0.7, 0.8, 0.85, 0.9, 0.95, 1.0):
        for l in list(range(1, 300)) + [997, 1999, 2000]:
            b = oracle.bounds(sim, tau, l)
            assert similarity.minsize(sim, l, tau) == b["minsize"]
            assert similarity.maxsize(sim, l, tau) == b["maxsize"]
            assert similarity.maxprefix(sim, l, tau) == b["maxprefix"]
            assert similarity.midprefix(sim, l, tau) == b["midprefix"]
        for l1 in range(1, 120, 7):
            for l2 in range(1, 120, 5):
                assert similarity.minoverlap(sim, l1, l2, tau) == oracle.minoverlap(sim, l1, l2, tau)


@pytest.mark.parametrize("sim", ["jaccard", "cosine", "dice"])
@pytest.mark.parametrize("tau", [0.5, 0.7, 0.8, 0.9, 0.95])
def test_prefix_filter_is_complete_for_bounds(sim, tau):
    """Prefix filtering never drops a pair the exact predicate accepts: for every
    length-compatible (big, small), minoverlap(big, small) >= minsize(big)
    (probe maxprefix) and >= minoverlap(small, small) (indexed midprefix), and
    for R-S joins >= minsize(small) (both sides index maxprefix)."""
    for big in range(1, 700):
        ms = similarity.minsize(sim, big, tau)
        for small in range(max(ms, 1), big + 1):
            mo = similarity.minoverlap(sim, big, small, tau)
            assert mo >= ms
            assert mo >= similarity.minoverlap(sim, small, small, tau)
            assert mo >= similarity.minsize(sim, small, tau)


def test_oracle_cosine_dice_allpairs_vs_brute():
    c = synth.generate(synth.C1, n_sets=900, universe=900, dup_frac=0.1, dup_edit_lo=0.0, dup_edit_hi=0.3, seed=5)
    for sim in ("cosine", "dice"):
        for tau in (0.6, 0.8, 0.9):
            a = oracle.join(c.tokens, c.starts, c.sizes, tau, sim=sim)
            b = oracle.brute(c.tokens, c.starts, c.sizes, tau, sim=sim)
            assert oracle.as_set(a) == oracle.as_set(b)

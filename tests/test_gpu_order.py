"""Deterministic output and batch lifetimes on the GPU.

`sort_pairs` orders a result by (probe id, indexed id) with a device radix
sort, so the pair list is the same array on every run (the reference's append
order is nondeterministic: each pair takes the next slot of an atomicAdd,
include/hyset/verification.hpp:125-130).  The batch
tests check that a captured batch stays correct when later joins grow the
context's scratch memory, and that freeing a collection drops a captured batch
that reads it."""
import numpy as np
import pytest

import oracle
from hyset_gb300 import synth

pytestmark = pytest.mark.gpu


class _DevicePairs:
    """A (n, 2) int32 view of device memory for torch.as_tensor."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n, 2), "typestr": "<i4", "data": (ptr, False), "version": 2}


def _read_device_pairs(r):
    torch = pytest.importorskip("torch")
    if r.count == 0:
        return np.zeros((0, 2), np.uint32)
    t = torch.as_tensor(_DevicePairs(r.device_pairs, r.count), device="cuda")
    return t.cpu().numpy().astype(np.uint32)


def _lexsorted(p):
    p = np.asarray(p, dtype=np.uint64)
    key = (p[:, 0] << np.uint64(32)) | p[:, 1]
    return bool(np.all(key[1:] > key[:-1]))


@pytest.mark.parametrize("kw", [dict(technique="fgss", probe_major=True), dict(technique="fgss"),
                                dict(technique="bitmap", bitmap=128), dict(technique="auto")])
def test_sorted_pairs_are_the_oracle_pairs_in_order(ctx, kw):
    c = synth.generate(synth.C2, n_sets=20000, seed=41)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    want = oracle.join(c.tokens, c.starts, c.sizes, 0.6)
    exp = want[np.lexsort((want[:, 1], want[:, 0]))]
    r1 = ctx.self_join(coll, threshold=0.6, sort_pairs=True, **kw)
    r2 = ctx.self_join(coll, threshold=0.6, sort_pairs=True, **kw)
    assert r1.count == len(exp) > 100
    assert _lexsorted(r1.pairs)
    np.testing.assert_array_equal(r1.pairs, exp)
    np.testing.assert_array_equal(r2.pairs, exp)


def _split(c, frac, seed):
    """Two collections from one (near-duplicates land on both sides)."""
    side = np.random.default_rng(seed).random(c.n) < frac
    out = []
    for mask in (side, ~side):
        ids = np.nonzero(mask)[0]
        sizes = c.sizes[ids]
        starts = np.zeros(len(ids), np.uint32)
        starts[1:] = np.cumsum(sizes[:-1])
        tokens = np.concatenate([c.tokens[c.starts[i]:c.starts[i] + c.sizes[i]] for i in ids])
        out.append((tokens, starts, sizes))
    return out


def test_sorted_device_pairs_rs_join(ctx):
    R, S = _split(synth.generate(synth.C2, n_sets=16000, seed=42), 0.55, 43)
    cr = ctx.upload(R[0], R[2], R[1])
    cs = ctx.upload(S[0], S[2], S[1])
    r = ctx.rs_join(cr, cs, threshold=0.5, sort_pairs=True, device_pairs=True)
    got = _read_device_pairs(r)
    exp = oracle.brute_rs(R, S, 0.5)
    assert r.count == len(exp) > 0
    assert _lexsorted(got)
    assert oracle.as_set(got) == oracle.as_set(exp)


def test_batch_sorted_pairs(ctx):
    colls = [synth.generate(synth.C2, n_sets=n, seed=50 + n) for n in (3000, 5000, 8000)]
    ups = [ctx.upload(c.tokens, c.sizes, c.starts) for c in colls]
    joins = [(u, None, dict(threshold=0.6, sort_pairs=True)) for u in ups]
    for attempt in range(2):
        res = ctx.batch_join(joins)
        for c, r in zip(colls, res):
            want = oracle.join(c.tokens, c.starts, c.sizes, 0.6)
            exp = want[np.lexsort((want[:, 1], want[:, 0]))]
            np.testing.assert_array_equal(r.pairs, exp)


def test_batch_replay_survives_scratch_growth(ctx):
    small = [synth.generate(synth.C2, n_sets=2000 + 500 * k, seed=60 + k) for k in range(4)]
    ups = [ctx.upload(c.tokens, c.sizes, c.starts) for c in small]
    joins = [(u, None, dict(threshold=0.7, technique="fgss")) for u in ups]
    exp = [oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.7)) for c in small]
    first = ctx.batch_join(joins)
    assert [oracle.as_set(r.pairs) for r in first] == exp
    big = synth.generate(synth.C3, n_sets=60000, universe=300000, seed=61)  # grows the index scratch
    cb = ctx.upload(big.tokens, big.sizes, big.starts)
    ctx.self_join(cb, threshold=0.8, technique="fgss", probe_major=True, count_only=True)
    again = ctx.batch_join(joins)  # same batch: replays the captured graph
    assert [oracle.as_set(r.pairs) for r in again] == exp


def test_freeing_a_collection_drops_its_captured_batch(ctx):
    a = synth.generate(synth.C2, n_sets=4000, seed=70)
    b = synth.generate(synth.C2, n_sets=4000, seed=71)
    ua = ctx.upload(a.tokens, a.sizes, a.starts)
    res = ctx.batch_join([(ua, None, dict(threshold=0.6))])
    assert oracle.as_set(res[0].pairs) == oracle.as_set(oracle.join(a.tokens, a.starts, a.sizes, 0.6))
    ua.free()
    ub = ctx.upload(b.tokens, b.sizes, b.starts)  # may reuse the freed handle's address
    res = ctx.batch_join([(ub, None, dict(threshold=0.6))])
    assert oracle.as_set(res[0].pairs) == oracle.as_set(oracle.join(b.tokens, b.starts, b.sizes, 0.6))


@pytest.mark.parametrize("frac", [0.85, 0.15])
@pytest.mark.parametrize("sim,tau", [("jaccard", 0.6), ("cosine", 0.7), ("dice", 0.65)])
def test_rs_orientation_gives_the_same_pairs(ctx, frac, sim, tau):
    """Indexing either collection of an R-S join yields the same (probe, indexed)
    pairs; `auto` indexes the smaller one."""
    R, S = _split(synth.generate(synth.C2, n_sets=16000, seed=44), frac, 45)
    cr = ctx.upload(R[0], R[2], R[1])
    cs = ctx.upload(S[0], S[2], S[1])
    exp = oracle.brute_rs(R, S, tau, sim=sim)
    exp = exp[np.lexsort((exp[:, 1], exp[:, 0]))]
    assert len(exp) > 0
    for orient in ("auto", "as_given", "swapped"):
        for kw in (dict(technique="fgss", probe_major=True), dict(technique="bitmap", bitmap=128),
                   dict(technique="fgss")):
            r = ctx.rs_join(cr, cs, threshold=tau, sim=sim, orientation=orient, sort_pairs=True, **kw)
            np.testing.assert_array_equal(r.pairs, exp, err_msg=f"{orient} {kw}")

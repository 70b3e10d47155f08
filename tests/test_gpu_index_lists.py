"""How the prefix index's lists are built on the GPU.

The lists must hold their entries in set-id order (the join bisects them by
candidate id).  When every list has at most 64 entries the build fills them
with one atomic per entry and a warp puts 32 lists back in order (insertion
sort in shared memory, or in global memory when the 32 lists exceed the stage);
a longer list sends the whole build through the stable radix passes.  The
choice is made on the device from the longest list, so both sides of the bound
are checked here against the oracle, with a token planted in the prefix of
exactly 64 and 65 sets.  Lists of at most 32 entries in a collection the
library owns become token records for the single-join kernel (31 and 32)."""
import numpy as np
import pytest

import oracle
from hyset_gb300 import similarity, synth

pytestmark = pytest.mark.gpu


def _longest_list(c, tau):
    mid = similarity.midprefix_array("jaccard", c.sizes, tau)
    idx = np.concatenate([c.tokens[s:s + m] for s, m in zip(c.starts, mid)])
    return int(np.bincount(idx).max())


def _plant_many(c, n_tokens, per_token, seed):
    """Tokens 0..n_tokens-1 (below every other token) each added to per_token
    distinct sets, one planted token per set; sets re-sorted by size."""
    rng = np.random.default_rng(seed)
    shift = n_tokens
    sets = [c.tokens[s:s + l].astype(np.uint32) + shift for s, l in zip(c.starts, c.sizes)]
    chosen = rng.choice(len(sets), size=n_tokens * per_token, replace=False)
    for q, i in enumerate(chosen):
        sets[i] = np.concatenate([[q % n_tokens], sets[i]]).astype(np.uint32)
    order = sorted(range(len(sets)), key=lambda i: len(sets[i]))
    sets = [sets[i] for i in order]
    sizes = np.array([len(s) for s in sets], np.uint32)
    starts = np.concatenate([[0], np.cumsum(sizes[:-1], dtype=np.uint64)]).astype(np.uint32)
    return synth.Collection(np.concatenate(sets).astype(np.uint32), starts, sizes)


def _plant(c, k, seed):
    """Token 0 (below every other token, so inside every prefix) added to k
    random sets; the sets are re-sorted by size (stable)."""
    rng = np.random.default_rng(seed)
    sets = [c.tokens[s:s + l].astype(np.uint32) + 1 for s, l in zip(c.starts, c.sizes)]
    for i in rng.choice(len(sets), size=k, replace=False):
        sets[i] = np.concatenate([[0], sets[i]]).astype(np.uint32)
    order = sorted(range(len(sets)), key=lambda i: len(sets[i]))
    sets = [sets[i] for i in order]
    sizes = np.array([len(s) for s in sets], np.uint32)
    starts = np.concatenate([[0], np.cumsum(sizes[:-1], dtype=np.uint64)]).astype(np.uint32)
    return synth.Collection(np.concatenate(sets).astype(np.uint32), starts, sizes)


@pytest.mark.parametrize("k", [64, 65])
def test_lists_on_both_sides_of_the_bound(ctx, k):
    c = _plant(synth.generate(synth.C2, n_sets=20000, seed=61), k, seed=k)
    assert _longest_list(c, 0.8) == k
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.8))
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    for kw in (dict(technique="fgss", probe_major=True, bitmap=0), dict(technique="fgss", probe_major=True,
                                                                         bitmap=256, verify_mode=2)):
        r = ctx.self_join(coll, threshold=0.8, **kw)
        assert r.count == len(exp) and oracle.as_set(r.pairs) == exp, kw
    # the host-input join builds its index the same way
    r = ctx.self_join_host(c.tokens, c.sizes, c.starts, threshold=0.8, technique="fgss", probe_major=True,
                           bitmap=256)
    assert oracle.as_set(r.pairs) == exp


@pytest.mark.parametrize("k", [31, 32])
def test_token_records_on_both_sides_of_their_bound(ctx, k):
    """Lists of at most 31 entries become fixed 32-word token records (a
    length word and the entries): the collection's first build converts its
    sorted lists, later builds emit the records directly (an atomic slot per
    entry, then each record ordered).  A planted token in exactly 31 and 32
    prefixes puts the collection on either side; every join of the sequence
    must give the oracle's pairs."""
    c = _plant(synth.generate(synth.C2, n_sets=20000, seed=64), k, seed=k)
    assert _longest_list(c, 0.8) == k
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.8))
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    for kw in (dict(bitmap=0), dict(bitmap=256), dict(bitmap=512, verify_mode=2), dict(bitmap=0, fgss_batch=1)):
        r = ctx.self_join(coll, threshold=0.8, technique="fgss", probe_major=True, **kw)
        assert r.count == len(exp) and oracle.as_set(r.pairs) == exp, kw


@pytest.mark.parametrize("n,tau", [(10000, 0.5), (200000, 0.6), (200000, 0.8)])
def test_natural_lists(ctx, n, tau):
    """Longest lists 63 (short-list path), 141 (radix path) and 25."""
    c = synth.generate(synth.C2 if n > 10000 else synth.C1, n_sets=n, seed=7)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, tau))
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    r = ctx.self_join(coll, threshold=tau, technique="fgss", probe_major=True, sort_pairs=True)
    assert oracle.as_set(r.pairs) == exp
    p = np.asarray(r.pairs, np.uint64)
    key = (p[:, 0] << np.uint64(32)) | p[:, 1]
    assert bool(np.all(key[1:] > key[:-1]))


def test_short_lists_beyond_one_warp_stage(ctx):
    """32 consecutive lists of 40 entries (1,280 together, more than a warp
    stages in shared memory): the short-list path orders them in global memory."""
    c = _plant_many(synth.generate(synth.C2, n_sets=20000, seed=62), 32, 40, seed=5)
    assert _longest_list(c, 0.8) == 40
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.8))
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    r = ctx.self_join(coll, threshold=0.8, technique="fgss", probe_major=True, bitmap=256, sort_pairs=True)
    assert r.count == len(exp) and oracle.as_set(r.pairs) == exp


def test_remembered_short_path_with_lists_grown_in_place(ctx):
    """The list path is read back once per collection and prefix table.  A
    collection over caller memory can change afterwards: here token 0 is put
    at the head of 1,500 sets in place (tokens stay sorted, the universe the
    same), so one list far exceeds the short-list bound while the remembered
    path is the short one; the lists must still come out in order."""
    torch = pytest.importorskip("torch")
    c = synth.generate(synth.C2, n_sets=20000, seed=63)
    assert c.tokens.min() >= 1
    dt = torch.from_numpy(c.tokens.view(np.int32)).cuda()
    ds = torch.from_numpy(c.starts.view(np.int32)).cuda()
    dz = torch.from_numpy(c.sizes.view(np.int32)).cuda()
    coll = ctx.from_device(dt.data_ptr(), c.tokens.size, ds.data_ptr(), dz.data_ptr(), c.n, keep=(dt, ds, dz))
    kw = dict(technique="fgss", probe_major=True, bitmap=256)
    r = ctx.self_join(coll, threshold=0.8, **kw)
    assert oracle.as_set(r.pairs) == oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.8))
    grown = c.tokens.copy()
    chosen = np.random.default_rng(9).choice(c.n, size=1500, replace=False)
    grown[c.starts[chosen]] = 0
    assert _longest_list(synth.Collection(grown, c.starts, c.sizes), 0.8) == 1500
    dt.copy_(torch.from_numpy(grown.view(np.int32)).cuda())
    torch.cuda.synchronize()
    r = ctx.self_join(coll, threshold=0.8, **kw)
    assert oracle.as_set(r.pairs) == oracle.as_set(oracle.join(grown, c.starts, c.sizes, 0.8))
    coll.free()

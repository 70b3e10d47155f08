"""hyset_self_join_host: upload and self-join from host arrays in one call, the
copy chunked and overlapped with the checks and the index build.  It must give
exactly what hyset_collection_upload + hyset_self_join give, on both of its
paths (the pipelined one and the plain sequence it falls back to), and reject
the same invalid inputs."""
import numpy as np
import pytest

import hyset_gb300 as hs
import oracle
from conftest import GOLDEN_SETS, load_golden
from hyset_gb300 import synth

pytestmark = pytest.mark.gpu

PIPELINED = dict(technique="fgss", probe_major=True, bitmap=256)


@pytest.mark.parametrize("name", GOLDEN_SETS)
def test_host_join_matches_the_golden_pairs(ctx, name):
    tokens, starts, sizes, results = load_golden(name)
    for tau, want in results.items():
        for kw in (PIPELINED, dict(technique="fgss", probe_major=True, bitmap=0), {}):
            r = ctx.self_join_host(tokens, sizes, starts, threshold=tau, **kw)
            assert r.count == want["count"], (name, tau, kw)
            assert oracle.as_set(r.pairs) == {tuple(p) for p in want["pairs"]}, (name, tau, kw)


def test_host_join_across_copy_chunks(ctx):
    """About 22 M tokens: two 16 M-token copy chunks, sets straddling the cut."""
    c = synth.generate(synth.C3, n_sets=200000, seed=97)
    assert c.tokens.size > (16 << 20)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.8))
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    ref = ctx.self_join(coll, threshold=0.8, **PIPELINED)
    assert oracle.as_set(ref.pairs) == exp
    for kw in (PIPELINED, {}, {}):  # AUTO: the first call chooses (plain path), the next reuses the choice
        r = ctx.self_join_host(c.tokens, c.sizes, c.starts, threshold=0.8, **kw)
        assert r.count == len(exp) and oracle.as_set(r.pairs) == exp, kw
    r2 = ctx.self_join_host(c.tokens, c.sizes, None, threshold=0.8, sort_pairs=True, **PIPELINED)
    want = np.array(sorted(exp), dtype=np.uint32)
    np.testing.assert_array_equal(r2.pairs, want)


def test_host_join_keeps_the_collection(ctx):
    c = synth.generate(synth.C2, n_sets=20000, seed=98)
    r, coll = ctx.self_join_host(c.tokens, c.sizes, c.starts, threshold=0.6, keep_collection=True, **PIPELINED)
    again = ctx.self_join(coll, threshold=0.6, **PIPELINED)
    assert oracle.as_set(again.pairs) == oracle.as_set(r.pairs) == oracle.as_set(
        oracle.join(c.tokens, c.starts, c.sizes, 0.6))


def test_host_join_with_gaps_between_sets(ctx):
    """Starts that leave gaps: the plain sequence, same pairs."""
    c = synth.generate(synth.C2, n_sets=5000, seed=99)
    gap = 3
    starts = (c.starts.astype(np.int64) + gap * np.arange(c.n)).astype(np.uint32)
    tokens = np.zeros(int(starts[-1]) + int(c.sizes[-1]), np.uint32)
    for i in range(c.n):
        tokens[starts[i]:starts[i] + c.sizes[i]] = c.tokens[c.starts[i]:c.starts[i] + c.sizes[i]]
    r = ctx.self_join_host(tokens, c.sizes, starts, threshold=0.6, **PIPELINED)
    assert oracle.as_set(r.pairs) == oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.6))


@pytest.mark.parametrize("case", ["unsorted_tokens", "unsorted_sizes", "reserved_token", "past_end", "empty_set"])
def test_host_join_rejects_what_upload_rejects(ctx, case):
    c = synth.generate(synth.C2, n_sets=3000, seed=100)
    tokens, sizes, starts = c.tokens.copy(), c.sizes.copy(), c.starts.copy()
    n_tokens = None
    if case == "unsorted_tokens":
        i = int(np.argmax(sizes >= 3))
        s0 = int(starts[i])
        tokens[s0], tokens[s0 + 1] = tokens[s0 + 1], tokens[s0]
    elif case == "unsorted_sizes":
        sizes[0], sizes[-1] = sizes[-1], sizes[0]
        starts = None
    elif case == "reserved_token":
        tokens[int(starts[-1]) + int(sizes[-1]) - 1] = 0xFFFFFFFF
    elif case == "past_end":
        starts[-1] += 10
    elif case == "empty_set":
        sizes = np.concatenate([[0], sizes]).astype(np.uint32)
        starts = np.concatenate([[0], starts]).astype(np.uint32)
    with pytest.raises(hs.HysetError):
        ctx.self_join_host(tokens, sizes, starts, threshold=0.7, **PIPELINED)
    # the context stays usable
    r = ctx.self_join_host(c.tokens, c.sizes, c.starts, threshold=0.7, **PIPELINED)
    assert r.count == len(oracle.join(c.tokens, c.starts, c.sizes, 0.7))


def test_host_join_with_a_reused_size_profile(ctx):
    """Collections with the same sizes but different token ranges: the second
    call assumes the first one's universe (too small, then too large) and must
    still return the exact pairs."""
    c = synth.generate(synth.C2, n_sets=30000, seed=101)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.6))
    shifted = (c.tokens.astype(np.int64) + 3_000_000).astype(np.uint32)  # same pairs, larger tokens
    for toks in (c.tokens, shifted, c.tokens, shifted):
        r = ctx.self_join_host(toks, c.sizes, c.starts, threshold=0.6, **PIPELINED)
        assert oracle.as_set(r.pairs) == exp
    bad = shifted.copy()
    bad[int(c.starts[-1])] = 0xFFFFFFFF if c.sizes[-1] == 1 else bad[int(c.starts[-1])]
    bad[int(c.starts[-1]) + int(c.sizes[-1]) - 1] = 0xFFFFFFFF  # reserved token, profile seen before
    with pytest.raises(hs.HysetError):
        ctx.self_join_host(bad, c.sizes, c.starts, threshold=0.6, **PIPELINED)


def test_host_join_records_and_a_list_that_outgrows_them(ctx):
    """Once a join with a size profile and threshold saw every index list at
    most 31 long, later host-input joins with that profile put the prefix
    entries straight into token records while the chunks land.  A collection
    with the same sizes whose token 0 heads the prefixes of 40 sets overflows
    one record: the ordering pass flags it and the join runs again over lists.
    Every call must return the oracle's pairs."""
    c = synth.generate(synth.C2, n_sets=20000, seed=103)
    assert c.tokens.min() >= 1
    grown = c.tokens.copy()
    grown[c.starts[np.random.default_rng(5).choice(c.n, size=40, replace=False)]] = 0
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.8))
    exp_grown = oracle.as_set(oracle.join(grown, c.starts, c.sizes, 0.8))
    for toks, want in ((c.tokens, exp), (c.tokens, exp), (grown, exp_grown), (c.tokens, exp), (c.tokens, exp)):
        r = ctx.self_join_host(toks, c.sizes, c.starts, threshold=0.8, **PIPELINED)
        assert r.count == len(want) and oracle.as_set(r.pairs) == want


def test_host_join_chunk_by_chunk(ctx):
    """A repeat of a size profile whose index lists fit token records, in more
    than one copy chunk: each chunk's probes are joined as soon as its entries
    are in the records and ordered, beside the copies of the later chunks.
    Every call must return the oracle's pairs: plain repeats, a pair buffer
    too small (the join runs again with room), a list that outgrows its record
    and a token past the assumed universe (both run again over lists), count
    only and work counters."""
    c = synth.generate(synth.C3, n_sets=200000, seed=131)
    assert c.tokens.size > (16 << 20)
    base = (c.tokens.astype(np.int64) + 1).astype(np.uint32)  # token 0 unused: same pairs
    exp = oracle.as_set(oracle.join(base, c.starts, c.sizes, 0.8))
    grown = base.copy()
    grown[c.starts[np.random.default_rng(7).choice(c.n, size=40, replace=False)]] = 0  # 40 prefixes share token 0
    exp_grown = oracle.as_set(oracle.join(grown, c.starts, c.sizes, 0.8))
    shifted = (base.astype(np.int64) + 2_000_000).astype(np.uint32)
    calls = [(base, exp, {}), (base, exp, {}), (base, exp, {}), (base, exp, dict(pair_capacity=64)),
             (grown, exp_grown, {}), (base, exp, {}), (base, exp, {}), (shifted, exp, {}), (base, exp, {}),
             (base, exp, {}), (base, exp, {})]
    for i, (toks, want, kw) in enumerate(calls):
        r = ctx.self_join_host(toks, c.sizes, c.starts, threshold=0.8, **PIPELINED, **kw)
        assert r.count == len(want) and oracle.as_set(r.pairs) == want, (i, kw)
    r = ctx.self_join_host(base, c.sizes, c.starts, threshold=0.8, count_only=True, **PIPELINED)
    assert r.count == len(exp)
    r = ctx.self_join_host(base, c.sizes, None, threshold=0.8, collect_stats=True, **PIPELINED)
    assert r.count == len(exp) and oracle.as_set(r.pairs) == exp
    assert r.stats[0] > 0 and r.stats[3] > 0  # filter items, index entries

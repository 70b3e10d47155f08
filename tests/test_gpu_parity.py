"""GPU parity: the CUDA path through the C ABI against the reference's golden
pairs and the CPU oracle.  Integer work, so the bar is exact equality of the
pair sets (and no duplicates)."""
import numpy as np
import pytest

import hyset_gb300 as hs
import oracle
from conftest import GOLDEN_SETS, load_golden
from hyset_gb300 import synth
from hyset_gb300.handlers import BitmapHandler, DeviceHandler, FgssHandler

pytestmark = pytest.mark.gpu

TECHS = [
    dict(technique="fgss"),                                     # token-major (default FGSS kernel)
    dict(technique="fgss", bitmap=256),
    dict(technique="fgss", bitmap=64),
    dict(technique="fgss", probe_major=True, verify_mode=1),    # probe-major kernel, sorted index
    dict(technique="fgss", probe_major=True, verify_mode=2, bitmap=256),
    dict(technique="bitmap", bitmap=64, verify_mode=1),
    dict(technique="bitmap", bitmap=256, verify_mode=2),
    dict(technique="bitmap", bitmap=512, verify_mode=1),
    dict(technique="fgss", probe_major=True, bitmap=1024, verify_mode=1),  # 1024-bit signatures
    dict(technique="direct", verify_mode=1),
]
TECH_IDS = ["-".join(f"{k}{v}" for k, v in t.items()) for t in TECHS]


def as_set_checked(pairs):
    s = oracle.as_set(pairs)
    assert len(s) == len(pairs), "duplicate pairs emitted"
    return s


@pytest.mark.parametrize("name", GOLDEN_SETS)
@pytest.mark.parametrize("kw", TECHS, ids=TECH_IDS)
def test_self_join_matches_reference_golden(ctx, name, kw):
    tokens, starts, sizes, results = load_golden(name)
    coll = ctx.upload(tokens, sizes, starts)
    for tau, want in results.items():
        r = ctx.self_join(coll, threshold=tau, **kw)
        assert r.count == want["count"], (name, tau)
        assert as_set_checked(r.pairs) == {tuple(p) for p in want["pairs"]}, (name, tau)
        rc = ctx.self_join(coll, threshold=tau, count_only=True, **kw)
        assert rc.count == want["count"] and rc.pairs is None


SCALED = [
    ("c1", synth.C1, {}, [0.5, 0.8, 0.95]),
    ("c2", synth.C2, {"n_sets": 30000}, [0.5, 0.7, 0.9]),
    ("c3", synth.C3, {"n_sets": 20000, "universe": 200000}, [0.8]),
]


@pytest.mark.parametrize("label,spec,kw,taus", SCALED, ids=[s[0] for s in SCALED])
@pytest.mark.parametrize("sim", ["jaccard", "cosine", "dice"])
def test_self_join_matches_oracle_on_workloads(ctx, label, spec, kw, taus, sim):
    c = synth.generate(spec, **kw)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    for tau in taus:
        exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, tau, sim=sim))
        for kw in (dict(technique="fgss"), dict(technique="fgss", bitmap=128),
                   dict(technique="fgss", probe_major=True, verify_mode=2),
                   dict(technique="fgss", probe_major=True, bitmap=128, verify_mode=1),
                   dict(technique="fgss", probe_major=True, bitmap=1024, verify_mode=1),
                   dict(technique="bitmap", bitmap=256, verify_mode=2)):
            r = ctx.self_join(coll, threshold=tau, sim=sim, **kw)
            assert as_set_checked(r.pairs) == exp, (label, sim, tau, kw)


@pytest.mark.parametrize("sim", ["jaccard", "cosine", "dice"])
def test_rs_join_matches_brute_force(ctx, sim):
    R = synth.generate(synth.C1, n_sets=1500, universe=1200, dup_frac=0.0, seed=21)
    S = synth.generate(synth.C1, n_sets=1200, universe=1200, seed=22)
    # plant near-copies of some R sets into S (same universe numbering is not
    # guaranteed across generations, so copy tokens directly)
    sets = [S.set(i).tolist() for i in range(S.n)] + [R.set(i).tolist() for i in range(0, R.n, 7)]
    sets.sort(key=lambda x: (len(x), x))
    s_sizes = np.array([len(x) for x in sets], np.uint32)
    s_tok = np.array([t for x in sets for t in x], np.uint32)
    s_st = np.concatenate([[0], np.cumsum(s_sizes[:-1])]).astype(np.uint32)
    cr = ctx.upload(R.tokens, R.sizes, R.starts)
    cs = ctx.upload(s_tok, s_sizes, s_st)
    for tau in (0.6, 0.85):
        exp = oracle.as_set(oracle.brute_rs((R.tokens, R.starts, R.sizes), (s_tok, s_st, s_sizes), tau, sim=sim))
        assert len(exp) > 0
        for kw in (dict(technique="fgss"), dict(technique="fgss", bitmap=64),
                   dict(technique="fgss", probe_major=True), dict(technique="bitmap", bitmap=128),
                   dict(technique="fgss", probe_major=True, bitmap=1024), dict(technique="direct")):
            r = ctx.rs_join(cr, cs, threshold=tau, sim=sim, **kw)
            assert as_set_checked(r.pairs) == exp, (sim, tau, kw)


@pytest.mark.parametrize("tech", ["bitmap", "fgss"])
@pytest.mark.parametrize("aggregate", [False, True])
def test_reference_handlers_partition_join(ctx, tech, aggregate):
    c = synth.generate(synth.C2, n_sets=12000)
    hc = hs.from_arrays(c.tokens, c.sizes, 2500, 0.7)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    if tech == "bitmap":
        h = BitmapHandler(ctx, hc, coll, 64, 2500, aggregate, 0.7)
    else:
        h = FgssHandler(ctx, hc, coll, 2500, aggregate, 0.7)
    out = hs.CountHandler() if aggregate else hs.PairsHandler()
    h.set_output_handler(out)
    part = hs.Partition(0, hc.blocks)
    h.join(part, part)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.7))
    if aggregate:
        assert out.get_count() == len(exp)
    else:
        assert as_set_checked(out.pairs) == exp


def test_reference_handler_block_pairs(ctx):
    c = synth.generate(synth.C1, n_sets=6000, universe=3000, dup_frac=0.05, dup_edit_hi=0.2)
    hc = hs.from_arrays(c.tokens, c.sizes, 1000, 0.8)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    h = FgssHandler(ctx, hc, coll, 1000, False, 0.8)
    out = hs.PairsHandler()
    h.set_output_handler(out)
    for first in hc.blocks:
        for second in hc.blocks:
            if second.id >= first.id:
                h.join(first, second)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.8))
    assert as_set_checked(out.pairs) == exp


@pytest.mark.parametrize("scenario", [1, 2])
def test_device_handler_verifies_candidates(ctx, scenario):
    c = synth.generate(synth.C1, n_sets=2000, universe=1500, dup_frac=0.05, dup_edit_hi=0.3, seed=9)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    tau = 0.7
    dh = DeviceHandler(ctx, coll, coll, 32, scenario, False, 64, 5000, tau)
    out = hs.PairsHandler()
    dh.set_output_handler(out)
    from hyset_gb300 import similarity
    for p in range(c.n):
        ms = similarity.minsize("jaccard", int(c.sizes[p]), tau)
        lo = int(np.searchsorted(c.sizes, ms, side="left"))
        cands = np.arange(lo, p, dtype=np.uint32)
        if cands.size:
            dh.add_candidates(p, cands)
    dh.flush()
    exp = oracle.as_set(oracle.brute(c.tokens, c.starts, c.sizes, tau))
    assert as_set_checked(out.pairs) == exp


def test_edge_cases(ctx):
    # one set; identical sets; singletons; tau = 1.0
    one = ctx.upload(np.array([1, 2, 3], np.uint32), np.array([3], np.uint32))
    assert ctx.self_join(one, threshold=0.5).count == 0
    same = ctx.upload(np.tile(np.array([2, 5, 9], np.uint32), 40), np.full(40, 3, np.uint32))
    for kw in (dict(technique="fgss"), dict(technique="fgss", probe_major=True), dict(technique="bitmap"),
               dict(technique="direct")):
        r = ctx.self_join(same, threshold=1.0, **kw)
        assert r.count == 40 * 39 // 2, kw
    singles = ctx.upload(np.array([1, 1, 2, 3, 3], np.uint32), np.ones(5, np.uint32))
    r = ctx.self_join(singles, threshold=0.9, technique="fgss", sort_pairs=True)
    assert r.pairs.tolist() == [[1, 0], [4, 3]]
    empty = ctx.upload(np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    assert ctx.self_join(empty, threshold=0.8).count == 0


def test_probe_ranges_shard_a_join(ctx):
    c = synth.generate(synth.C2, n_sets=20000)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.7))
    got = set()
    for lo, hi in ((0, 7000), (7000, 15000), (15000, 20000)):
        r = ctx.self_join(coll, threshold=0.7, technique="fgss", probe_major=True, probe_range=(lo, hi))
        got |= as_set_checked(r.pairs)
    assert got == exp
    with pytest.raises(hs.HysetError):
        ctx.self_join(coll, threshold=0.7, technique="fgss", probe_range=(0, 10))  # token-major: whole joins


def test_invalid_inputs_fail_loudly(ctx):
    with pytest.raises(hs.HysetError):
        ctx.upload(np.array([3, 2, 1], np.uint32), np.array([3], np.uint32))  # unsorted set
    with pytest.raises(hs.HysetError):
        ctx.upload(np.array([1, 2, 3], np.uint32), np.array([2, 1], np.uint32))  # sizes decrease
    coll = ctx.upload(np.array([1, 2], np.uint32), np.array([2], np.uint32))
    with pytest.raises(hs.HysetError):
        ctx.self_join(coll, threshold=1.5)
    with pytest.raises(hs.HysetError):
        ctx.self_join(coll, threshold=0.8, bitmap=96)


def test_pair_buffer_growth(ctx):
    # 300 identical sets -> 44850 pairs with a 16-pair initial buffer
    coll = ctx.upload(np.tile(np.arange(1, 9, dtype=np.uint32), 300), np.full(300, 8, np.uint32))
    for pm in (False, True):
        r = ctx.self_join(coll, threshold=0.9, technique="fgss", pair_capacity=16, probe_major=pm)
        assert r.count == 300 * 299 // 2 and len(oracle.as_set(r.pairs)) == r.count


def _mixed_batch(ctx, seed=5, n_joins=18):
    """Independent joins of uneven sizes, similarity functions, thresholds and
    techniques (self-joins and R-S joins)."""
    rng = np.random.default_rng(seed)
    joins, colls = [], []
    sims = ["jaccard", "cosine", "dice"]
    for j in range(n_joins):
        nr = int(rng.integers(300, 6000))
        mean = float(np.exp(rng.uniform(np.log(8), np.log(120))))
        spec = dict(n_sets=nr, universe=int(rng.integers(3000, 40000)), zipf_s=float(rng.uniform(0.7, 1.3)),
                    size_dist=synth.LOGNORMAL, size_a=float(np.log(mean)), size_b=0.5, size_min=2,
                    size_max=600, dup_frac=0.05, dup_edit_lo=0.0, dup_edit_hi=0.2, seed=1000 + j)
        R = synth.generate(synth.C2, **spec)
        cr = ctx.upload(R.tokens, R.sizes, R.starts)
        colls.append(cr)
        kw = dict(threshold=float(rng.uniform(0.5, 0.95)), sim=sims[j % 3])
        if j % 4 == 1:
            kw.update(technique="bitmap", bitmap=128)
        elif j % 4 == 2:
            kw.update(technique="direct") if nr < 1500 else kw.update(technique="fgss", probe_major=True)
        if j % 2 == 0:
            joins.append((cr, None, kw))  # self-join
        else:
            spec2 = dict(spec, n_sets=int(rng.integers(300, 4000)), seed=2000 + j)
            S = synth.generate(synth.C2, **spec2)
            cs = ctx.upload(S.tokens, S.sizes, S.starts)
            colls.append(cs)
            joins.append((cr, cs, kw))
    return joins, colls


def test_batch_join_matches_joins_run_one_at_a_time(ctx):
    joins, colls = _mixed_batch(ctx)
    single = []
    for R, S, kw in joins:
        r = ctx.self_join(R, **kw) if S is None else ctx.rs_join(R, S, **kw)
        single.append(as_set_checked(r.pairs))
    assert sum(len(x) for x in single) > 0
    for attempt in range(2):  # first call captures the batch graph, the second replays it
        res = ctx.batch_join(joins)
        for k, (r, exp) in enumerate(zip(res, single)):
            assert r.count == len(exp), (attempt, k, joins[k][2])
            assert as_set_checked(r.pairs) == exp, (attempt, k, joins[k][2])


@pytest.mark.parametrize("tau", [0.6, 0.9])
def test_autotuned_join_keeps_the_pairs(ctx, tau):
    """AUTO with bitmap 0 on 80,000 probes: the autotuner times samples and
    picks the signature width and the verification mode (a lane or the warp
    per candidate); the choice is reported, reused from the context's cache
    (also by the host-input join) and never changes the pairs."""
    c = synth.generate(synth.C2, n_sets=80000, seed=71)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, tau))
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    r1 = ctx.self_join(coll, threshold=tau)
    r2 = ctx.self_join(coll, threshold=tau)
    assert r1.bitmap_bits in (0, 128, 256, 512, 1024) and r1.verify_mode in (1, 2), (r1.bitmap_bits, r1.verify_mode)
    assert (r2.bitmap_bits, r2.verify_mode) == (r1.bitmap_bits, r1.verify_mode)
    assert as_set_checked(r1.pairs) == exp and as_set_checked(r2.pairs) == exp
    r3 = ctx.self_join_host(c.tokens, c.sizes, c.starts, threshold=tau)
    assert oracle.as_set(r3.pairs) == exp
    for vm in (1, 2):
        r = ctx.self_join(coll, threshold=tau, verify_mode=vm)
        assert r.verify_mode == vm and as_set_checked(r.pairs) == exp

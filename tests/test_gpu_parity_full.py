"""GPU parity at the full sizes of the benchmark workloads.

The scaled-down workloads of test_gpu_parity.py run every kernel variant; this
file runs the workloads themselves, at the sizes the benchmark times them:

- the 200,000-set short-set collection at Jaccard 0.5, 0.7 and 0.9 with the
  reference's two GPU techniques (64-bit and 256-bit bitmap signatures, the
  prefix filter, token-major and probe-major) and AUTO;
- the 1,000,000-set long-set collection at Jaccard, cosine and dice 0.8, AUTO
  and explicit prefix-filter configurations (warp verification, 512-bit
  signatures);
- the 256-join batch in one persistent launch, against the same joins run one
  call at a time, and against the oracle's self-join of R ∪ S for every join
  small enough for the CPU.

Expected pair sets come from the CPU oracle's restatement of the reference's
host::allpairs (cpu_multi split over the host cores).  Integer work: the bar
is equality of the pair sets, with no duplicates."""
import os

import numpy as np
import pytest

import oracle
from hyset_gb300 import synth

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def pair_keys(pairs):
    """Sorted 64-bit keys of a pair list; asserts no pair appears twice."""
    p = np.asarray(pairs, np.uint64).reshape(-1, 2)
    k = np.sort((p[:, 0] << np.uint64(32)) | p[:, 1])
    assert k.size == 0 or np.all(k[1:] != k[:-1]), "duplicate pairs emitted"
    return k


@pytest.fixture(scope="module")
def c2():
    return synth.generate(synth.C2)


@pytest.fixture(scope="module")
def c3():
    return synth.generate(synth.C3)


C2_TECHS = [dict(technique="bitmap", bitmap=64), dict(technique="bitmap", bitmap=256),
            dict(technique="fgss"), dict(technique="fgss", probe_major=True),
            dict(technique="fgss", probe_major=True, bitmap=256, verify_mode=2), dict(technique="auto")]


@pytest.mark.parametrize("tau", [0.5, 0.7, 0.9])
def test_c2_full_size_matches_oracle(ctx, c2, tau):
    assert c2.n == 200_000
    exp = pair_keys(oracle.join_multi(c2.tokens, c2.starts, c2.sizes, tau, THREADS))
    assert exp.size > 0
    coll = ctx.upload(c2.tokens, c2.sizes, c2.starts)
    for kw in C2_TECHS:
        r = ctx.self_join(coll, threshold=tau, **kw)
        assert r.count == exp.size, (tau, kw)
        assert np.array_equal(pair_keys(r.pairs), exp), (tau, kw)
    coll.free()


@pytest.mark.parametrize("sim", ["jaccard", "cosine", "dice"])
def test_c3_full_size_matches_oracle(ctx, c3, sim):
    assert c3.n == 1_000_000
    exp = pair_keys(oracle.join_multi(c3.tokens, c3.starts, c3.sizes, 0.8, THREADS, sim=sim))
    assert exp.size > 0
    coll = ctx.upload(c3.tokens, c3.sizes, c3.starts)
    for kw in (dict(technique="auto"), dict(technique="fgss", probe_major=True, verify_mode=2),
               dict(technique="fgss", probe_major=True, bitmap=512, verify_mode=1),
               dict(technique="fgss", probe_major=True, bitmap=1024, verify_mode=1),
               dict(technique="fgss", probe_major=True, verify_mode=1, sort_pairs=True)):
        r = ctx.self_join(coll, threshold=0.8, sim=sim, **kw)
        assert r.count == exp.size, (sim, kw)
        assert np.array_equal(pair_keys(r.pairs), exp), (sim, kw)
    # the host-input call (upload and join in one) returns the same set
    r = ctx.self_join_host(c3.tokens, c3.sizes, c3.starts, threshold=0.8, sim=sim)
    assert np.array_equal(pair_keys(r.pairs), exp), sim
    coll.free()


def _union_oracle(R, S, tau, sim):
    """R-S pairs (s, r) from the oracle's self-join of R ∪ S: the R-S predicate is
    the self-join predicate applied across the two collections, so the cross
    pairs of the union's self-join, mapped back to their collections, are the
    R-S join."""
    (rt, rs, rz), (st, ss, sz) = R, S
    nr = rz.size
    sets = [(int(rz[i]), rt[int(rs[i]):int(rs[i]) + int(rz[i])], i) for i in range(nr)]
    sets += [(int(sz[i]), st[int(ss[i]):int(ss[i]) + int(sz[i])], nr + i) for i in range(sz.size)]
    sets.sort(key=lambda x: (x[0], x[1].tolist()))
    sizes = np.array([x[0] for x in sets], np.uint32)
    tokens = np.concatenate([x[1] for x in sets]).astype(np.uint32)
    starts = np.concatenate([[0], np.cumsum(sizes[:-1], dtype=np.uint64)]).astype(np.uint32)
    origin = np.array([x[2] for x in sets], np.int64)
    p = oracle.join_multi(tokens, starts, sizes, tau, THREADS, sim=sim).astype(np.int64)
    a, b = origin[p[:, 0]], origin[p[:, 1]]
    cross = (a < nr) != (b < nr)
    a, b = a[cross], b[cross]
    s_id = np.where(a >= nr, a - nr, b - nr)
    r_id = np.where(a >= nr, b, a)
    return np.stack([s_id, r_id], 1)


def test_c4_full_batch_matches_joins_one_at_a_time(ctx):
    work = synth.batch_workload(256)
    colls, joins = [], []
    for (rt, rs, rz), (st, ss, sz), kw in work:
        R = ctx.upload(rt, rz, rs)
        S = ctx.upload(st, sz, ss)
        colls += [R, S]
        joins.append((R, S, kw))
    res = ctx.batch_join(joins)
    assert len(res) == 256
    total, checked = 0, 0
    for k, ((R, S, kw), r) in enumerate(zip(joins, res)):
        one = ctx.rs_join(R, S, **kw)
        got = pair_keys(r.pairs)
        assert r.count == one.count, (k, kw)
        assert np.array_equal(got, pair_keys(one.pairs)), (k, kw)
        total += r.count
        (rt, rs, rz), (st, ss, sz), _ = work[k]
        if rz.size + sz.size <= 30_000:  # small enough for the CPU oracle
            exp = pair_keys(_union_oracle((rt, rs, rz), (st, ss, sz), kw["threshold"], kw["sim"]))
            assert np.array_equal(got, exp), (k, kw)
            checked += 1
    assert total > 0 and checked >= 8, (total, checked)
    for c in colls:
        c.free()

"""hyset_verify_device: device-resident candidate lists verified by the
candidate verifier (one warp or one lane per candidate, with or without the
XOR-signature bound before the merges) against the oracle's restatement of
hybrid::device_handler's verification."""
import numpy as np
import pytest

import oracle
from hyset_gb300 import synth

pytestmark = pytest.mark.gpu


def _lists(c, tau, sim, seed):
    """Random length-window candidates plus every result pair of the join (so
    both outcomes occur), grouped by probe."""
    rng = np.random.default_rng(seed)
    pairs = oracle.join(c.tokens, c.starts, c.sizes, tau, sim=sim)
    n = c.n
    probes = rng.choice(np.arange(1, n), size=min(n - 1, 2000), replace=False)
    extra = [(int(p), int(x)) for p in probes for x in rng.integers(0, p, size=8)]
    allp = sorted({(int(a), int(b)) for a, b in pairs} | set(extra))
    pr, off, ca = [], [], []
    for p, x in allp:
        if not pr or pr[-1] != p:
            pr.append(p)
            off.append(len(ca))
        ca.append(x)
    ends = off[1:] + [len(ca)]
    return (np.array(pr, np.uint32), np.array(ends, np.uint32), np.array(ca, np.uint32))


SIG = [dict(technique="direct"), dict(technique="auto"), dict(technique="bitmap", bitmap=64),
       dict(technique="bitmap", bitmap=512)]


@pytest.mark.parametrize("sig", SIG, ids=["direct", "auto", "bits64", "bits512"])
@pytest.mark.parametrize("sim,tau", [("jaccard", 0.7), ("cosine", 0.8), ("dice", 0.75)])
@pytest.mark.parametrize("vm", [1, 2, 3])
def test_verify_device_matches_the_oracle(ctx, sim, tau, vm, sig):
    torch = pytest.importorskip("torch")
    c = synth.generate(synth.C2, n_sets=15000, seed=120)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    probes, ends, cands = _lists(c, tau, sim, 121)
    exp, _ = oracle.verify_csr((c.tokens, c.starts, c.sizes), probes, ends, cands, tau, sim=sim)
    assert len(exp) > 0
    dp, de, dc = (torch.from_numpy(a.view(np.int32)).cuda() for a in (probes, ends, cands))
    r = ctx.verify_device(coll, dp.data_ptr(), de.data_ptr(), dc.data_ptr(), probes.size, threshold=tau, sim=sim,
                          verify_mode=vm, **sig)
    assert r.count == len(exp)
    assert r.bitmap_bits == (0 if sig["technique"] == "direct" else sig.get("bitmap", 128))
    assert oracle.as_set(r.pairs) == oracle.as_set(exp)
    rc = ctx.verify_device(coll, dp.data_ptr(), de.data_ptr(), dc.data_ptr(), probes.size, threshold=tau, sim=sim,
                           verify_mode=vm, count_only=True, **sig)
    assert rc.count == len(exp) and rc.pairs is None


def test_verify_device_rs_with_signatures(ctx):
    """R-S lists (probes of S, candidates of R): each side's own signatures.
    S holds near-copies of every third R set (one token dropped), each listed
    with its source and 23 random R sets as candidates."""
    torch = pytest.importorskip("torch")
    R = synth.generate(synth.C2, n_sets=6000, seed=131)
    rng = np.random.default_rng(133)
    src = np.arange(0, R.n, 3)
    sets = []
    for i in src:
        x = R.set(int(i)).tolist()
        if len(x) > 3:
            x.pop(int(rng.integers(len(x))))
        sets.append((len(x), x, int(i)))
    sets.sort(key=lambda e: (e[0], e[1]))
    s_sizes = np.array([e[0] for e in sets], np.uint32)
    s_tok = np.array([t for e in sets for t in e[1]], np.uint32)
    s_st = np.concatenate([[0], np.cumsum(s_sizes[:-1])]).astype(np.uint32)
    cr = ctx.upload(R.tokens, R.sizes, R.starts)
    cs = ctx.upload(s_tok, s_sizes, s_st)
    probes = np.arange(len(sets), dtype=np.uint32)
    cands = np.concatenate([[e[2]] + rng.integers(0, R.n, size=23).tolist() for e in sets]).astype(np.uint32)
    ends = (np.arange(1, probes.size + 1) * 24).astype(np.uint32)
    exp, _ = oracle.verify_csr((R.tokens, R.starts, R.sizes), probes, ends, cands, 0.7,
                               probe=(s_tok, s_st, s_sizes))
    assert len(exp) > len(sets) // 2
    dp, de, dc = (torch.from_numpy(a.view(np.int32)).cuda() for a in (probes, ends, cands))
    for sig in SIG:
        r = ctx.verify_device(cr, dp.data_ptr(), de.data_ptr(), dc.data_ptr(), probes.size, probe=cs, threshold=0.7,
                              **sig)
        assert oracle.as_set(r.pairs) == oracle.as_set(exp), sig

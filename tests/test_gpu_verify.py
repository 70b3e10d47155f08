"""hyset_verify_device: device-resident candidate lists verified by the
candidate verifier (one warp or one lane per candidate) against the oracle's
restatement of hybrid::device_handler's verification."""
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


@pytest.mark.parametrize("sim,tau", [("jaccard", 0.7), ("cosine", 0.8), ("dice", 0.75)])
@pytest.mark.parametrize("vm", [1, 2, 3])
def test_verify_device_matches_the_oracle(ctx, sim, tau, vm):
    torch = pytest.importorskip("torch")
    c = synth.generate(synth.C2, n_sets=15000, seed=120)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    probes, ends, cands = _lists(c, tau, sim, 121)
    exp, _ = oracle.verify_csr((c.tokens, c.starts, c.sizes), probes, ends, cands, tau, sim=sim)
    assert len(exp) > 0
    dp, de, dc = (torch.from_numpy(a.view(np.int32)).cuda() for a in (probes, ends, cands))
    r = ctx.verify_device(coll, dp.data_ptr(), de.data_ptr(), dc.data_ptr(), probes.size, threshold=tau, sim=sim,
                          verify_mode=vm)
    assert r.count == len(exp)
    assert oracle.as_set(r.pairs) == oracle.as_set(exp)
    rc = ctx.verify_device(coll, dp.data_ptr(), de.data_ptr(), dc.data_ptr(), probes.size, threshold=tau, sim=sim,
                           verify_mode=vm, count_only=True)
    assert rc.count == len(exp) and rc.pairs is None

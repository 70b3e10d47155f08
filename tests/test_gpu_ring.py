"""The candidate ring behind hybrid::device_handler (hyset_verifier_*).

Candidates stream through device-resident rings that a persistent kernel
verifies as the host publishes them.  These tests drive the rings through
their edge cases: rings of a few slots (wrap-around on every lap, waits for
space, pair-buffer drains), candidate sets larger than the ring (split into
several records), count-only output, a join on the same context while the
verifier kernel is live, and the bounded wait: with no producer the kernel
gives up after its wait limit and reports HYSET_E_TIMEOUT, and the next
publication starts it again.  Expected pairs come from the CPU oracle's
candidate verifier (the reference's verify_pair on every listed pair)."""
import time

import numpy as np
import pytest

import hyset_gb300 as hs
import oracle
from hyset_gb300 import similarity, synth
from hyset_gb300.handlers import DeviceHandler

pytestmark = pytest.mark.gpu

E_TIMEOUT = 5


@pytest.fixture(scope="module")
def coll_data():
    return synth.generate(synth.C1, n_sets=2500, universe=1800, dup_frac=0.06, dup_edit_hi=0.3, seed=61)


def _lists(c, tau, stride=1):
    """Length-compatible candidate lists of a self-join (every `stride`-th probe)."""
    probes, cands = [], []
    for p in range(1, c.n, stride):
        lo = int(np.searchsorted(c.sizes, similarity.minsize("jaccard", int(c.sizes[p]), tau), side="left"))
        if lo < p:
            probes.append(p)
            cands.append(np.arange(lo, p, dtype=np.uint32))
    return probes, cands


def _expected(c, probes, cands, tau):
    ends = np.cumsum([len(x) for x in cands]).astype(np.uint32)
    pairs, _ = oracle.verify_csr((c.tokens, c.starts, c.sizes), np.array(probes, np.uint32), ends,
                                 np.concatenate(cands), tau)
    return oracle.as_set(pairs)


@pytest.mark.parametrize("scenario", [1, 2])
@pytest.mark.parametrize("max_probes,max_candidates", [(8, 300), (64, 5000), (4096, 1 << 20)])
def test_ring_streams_candidates(ctx, coll_data, scenario, max_probes, max_candidates):
    c = coll_data
    tau = 0.7
    probes, cands = _lists(c, tau)
    exp = _expected(c, probes, cands, tau)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    for aggregate in (False, True):
        dh = DeviceHandler(ctx, coll, coll, 32, scenario, aggregate, max_probes, max_candidates, tau)
        out = hs.CountHandler() if aggregate else hs.PairsHandler()
        dh.set_output_handler(out)
        half = len(probes) // 2
        for p, cs in zip(probes[:half], cands[:half]):
            dh.add_candidates(p, cs)
        dh.flush()  # a flush in the middle: the stream continues after it
        for p, cs in zip(probes[half:], cands[half:]):
            dh.add_candidates(p, cs)
        dh.flush()
        if aggregate:
            assert out.get_count() == len(exp)
        else:
            got = oracle.as_set(out.pairs)
            assert len(got) == len(out.pairs) and got == exp
        dh.close()
    coll.free()


def test_ring_splits_a_candidate_set_larger_than_the_ring(ctx, coll_data):
    c = coll_data
    tau = 0.6
    p = c.n - 1
    cands = np.arange(0, p, dtype=np.uint32)  # every smaller set, far more than the ring holds
    exp = _expected(c, [p], [cands], tau)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    dh = DeviceHandler(ctx, coll, coll, 32, 1, False, 16, 1000, tau)
    out = hs.PairsHandler()
    dh.set_output_handler(out)
    dh.add_candidates(p, cands)
    dh.flush()
    assert oracle.as_set(out.pairs) == exp
    dh.close()
    coll.free()


def test_ring_runs_beside_a_join_on_the_same_context(ctx, coll_data):
    c = coll_data
    tau = 0.7
    probes, cands = _lists(c, tau, stride=3)
    exp = _expected(c, probes, cands, tau)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    dh = DeviceHandler(ctx, coll, coll, 32, 2, False, 256, 20000, tau)
    out = hs.PairsHandler()
    dh.set_output_handler(out)
    join_exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, tau))
    for k, (p, cs) in enumerate(zip(probes, cands)):
        dh.add_candidates(p, cs)
        if k % 200 == 0:  # the verifier kernel is live meanwhile
            assert oracle.as_set(ctx.self_join(coll, threshold=tau, technique="fgss", probe_major=True).pairs) \
                == join_exp
    dh.flush()
    assert oracle.as_set(out.pairs) == exp
    dh.close()
    coll.free()


def test_ring_wait_is_bounded_and_restarts(ctx, coll_data):
    """No producer: the verifier kernel started at creation gives up after its
    wait limit (100 ms) and the status says so; the next publication starts
    a new kernel, with the shorter limit set meanwhile."""
    c = coll_data
    tau = 0.8
    probes, cands = _lists(c, tau, stride=5)
    exp = _expected(c, probes, cands, tau)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    dh = DeviceHandler(ctx, coll, coll, 32, 1, False, 128, 50000, tau)
    out = hs.PairsHandler()
    dh.set_output_handler(out)
    time.sleep(0.5)
    assert dh.status() == E_TIMEOUT
    dh.set_wait_limit(2000)  # 2 ms from the next start on
    half = len(probes) // 2
    for p, cs in zip(probes[:half], cands[:half]):
        dh.add_candidates(p, cs)
    dh.flush()
    time.sleep(0.1)
    assert dh.status() == E_TIMEOUT  # the restarted kernel gave up again, after 2 ms
    for p, cs in zip(probes[half:], cands[half:]):
        dh.add_candidates(p, cs)
    dh.flush()
    assert oracle.as_set(out.pairs) == exp
    dh.close()
    coll.free()

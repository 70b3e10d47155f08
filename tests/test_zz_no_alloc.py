"""hyset_verify_candidates_noalloc: verification for callers that cannot allocate.

Engines that own all device memory through their own pool, and
latency-critical paths that cannot take cudaMalloc's implicit
synchronisation, use this entry point: it keeps its scratch in a fixed device
array inside the library and writes only to the buffers the caller passes.
This test drives it through the C ABI with device buffers the test owns and
checks, on two calls in a row (the second reusing the scratch the first left
behind), that it returns exactly the pairs of the allocating verifier
(hyset_verifier_*), for Jaccard and dice, self-joins and R-S joins.  The pair sets are integer results, so the
comparison is exact.

Kept in a file that pytest collects last so a failure here never hides the
results of the other GPU tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _candidates(probe_sizes, indexed_sizes, tau, sim, self_join):
    """Length-compatible (probe, candidate) lists as CSR: for a self-join the
    smaller ids whose size is at least minsize(|probe|), for an R-S join every
    indexed set with a size in [minsize(|probe|), maxsize(|probe|)]."""
    from hyset_gb300 import similarity
    probes, ends, cands = [], [], []
    total = 0
    for p in range(len(probe_sizes)):
        lp = int(probe_sizes[p])
        lo = int(np.searchsorted(indexed_sizes, similarity.minsize(sim, lp, tau), side="left"))
        hi = p if self_join else int(np.searchsorted(indexed_sizes, similarity.maxsize(sim, lp, tau), side="right"))
        if lo < hi:
            cands.append(np.arange(lo, hi, dtype=np.uint32))
            total += hi - lo
            probes.append(p)
            ends.append(total)
    return (np.array(probes, np.uint32), np.array(ends, np.uint32),
            np.concatenate(cands) if cands else np.zeros(0, np.uint32))


def _reference_verifier(ctx, indexed, probe, probes, ends, cands, tau, scenario, sim):
    import hyset_gb300 as hs
    from hyset_gb300.handlers import DeviceHandler
    dh = DeviceHandler(ctx, indexed, probe, 32, scenario, False, 4096, 1 << 22, tau, sim=sim)
    out = hs.PairsHandler()
    dh.set_output_handler(out)
    start = 0
    for p, e in zip(probes.tolist(), ends.tolist()):
        dh.add_candidates(p, cands[start:e])
        start = e
    dh.flush()
    dh.close()
    return out.pairs


def _collections(self_join):
    """R (indexed) and S (probe): one C1-like collection for a self-join; for
    an R-S join a second collection holding near-copies of every fifth R set."""
    from hyset_gb300 import synth
    R = synth.generate(synth.C1, n_sets=1500, universe=1200, dup_frac=0.06, dup_edit_hi=0.3, seed=31)
    if self_join:
        return (R.tokens, R.starts, R.sizes), (R.tokens, R.starts, R.sizes)
    S = synth.generate(synth.C1, n_sets=900, universe=1200, dup_frac=0.0, seed=32)
    rng = np.random.default_rng(33)
    sets = [S.set(i).tolist() for i in range(S.n)]
    for i in range(0, R.n, 5):
        x = R.set(i).tolist()
        if len(x) > 8 and rng.random() < 0.5:  # drop one token: a near-copy
            x.pop(int(rng.integers(len(x))))
        sets.append(x)
    sets.sort(key=lambda x: (len(x), x))
    sizes = np.array([len(x) for x in sets], np.uint32)
    tokens = np.array([t for x in sets for t in x], np.uint32)
    starts = np.concatenate([[0], np.cumsum(sizes[:-1])]).astype(np.uint32)
    return (R.tokens, R.starts, R.sizes), (tokens, starts, sizes)


CASES = [("jaccard", True), ("dice", True), ("jaccard", False), ("dice", False)]


@pytest.mark.parametrize("scenario", [1, 2])
@pytest.mark.parametrize("sim,self_join", CASES, ids=[f"{s}-{'self' if j else 'rs'}" for s, j in CASES])
def test_noalloc_matches_allocating_verifier_twice(scenario, sim, self_join):
    torch = pytest.importorskip("torch")
    import hyset_gb300 as hs
    from hyset_gb300 import _lib

    lib = _lib.load()
    (rt, rs, rz), (st_, ss, sz) = _collections(self_join)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    on_dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).astype(np.int32)).to(dev)
    d_rt, d_rs, d_rz = on_dev(rt), on_dev(rs), on_dev(rz)
    d_st, d_ss, d_sz = (d_rt, d_rs, d_rz) if self_join else (on_dev(st_), on_dev(ss), on_dev(sz))
    max_len = int(max(rz.max(), sz.max()))
    with hs.Context(0) as ctx:
        cr = ctx.upload(rt, rz, rs)
        cs = cr if self_join else ctx.upload(st_, sz, ss)
        for tau in (0.6, 0.8):  # two calls in a row on the shared scratch
            probes, ends, cands = _candidates(sz, rz, tau, sim, self_join)
            expected = _reference_verifier(ctx, cr, cs, probes, ends, cands, tau, scenario, sim)
            assert len(expected) > 0
            d_pr, d_en, d_ca = on_dev(probes), on_dev(ends), on_dev(cands)
            cap = len(cands)
            d_pairs = torch.zeros((max(cap, 1), 2), dtype=torch.int32, device=dev)
            d_count = torch.zeros(1, dtype=torch.int64, device=dev)
            d_skip = torch.zeros(1, dtype=torch.int32, device=dev)
            stream = torch.cuda.current_stream(dev)
            ptr = lambda t: C.c_void_p(t.data_ptr())
            st = lib.hyset_verify_candidates_noalloc(
                ptr(d_rt), ptr(d_rs), ptr(d_rz), ptr(d_st), ptr(d_ss), ptr(d_sz), max_len,
                ptr(d_pr), ptr(d_en), ptr(d_ca), len(probes), _lib.SIM[sim], tau, scenario,
                ptr(d_pairs), cap, ptr(d_count), ptr(d_skip), C.c_void_p(stream.cuda_stream))
            assert st == 0
            torch.cuda.synchronize()
            n = int(d_count.item())
            assert int(d_skip.item()) == 0
            got = d_pairs[:n].cpu().numpy().astype(np.uint32)
            assert n == len(expected)
            assert {tuple(x) for x in got.tolist()} == {tuple(x) for x in expected.tolist()}
            assert len({tuple(x) for x in got.tolist()}) == n


def test_noalloc_rejects_sizes_beyond_its_table():
    from hyset_gb300 import _lib
    lib = _lib.load()
    one = C.c_void_p(16)  # never dereferenced: the size check fails first
    st = lib.hyset_verify_candidates_noalloc(one, one, one, one, one, one, 4097, one, one, one, 1,
                                             _lib.SIM["jaccard"], 0.8, 1, one, 1, one, None, None)
    assert st == 6  # HYSET_E_UNSUPPORTED
    st = lib.hyset_verify_candidates_noalloc(one, one, one, one, one, one, 100, one, one, one, 1,
                                             _lib.SIM["cosine"], 0.8, 1, one, 1, one, None, None)
    assert st == 6

"""hyset_verify_candidates_noalloc: verification for callers that cannot allocate.

Engines that own all device memory, code running while a stream is captured
into a CUDA graph, and latency-critical paths that cannot take cudaMalloc's
implicit synchronisation use this entry point: it keeps its scratch in a fixed
device array inside the library and writes only to the buffers the caller
passes.  This test drives it through the C ABI with device buffers the test
owns and checks, on two calls in a row (the second reusing the scratch the
first left behind), that it returns exactly the pairs of the allocating
verifier (hyset_verifier_*).  The pair sets are integer results, so the
comparison is exact.

Kept in a file that pytest collects last so a failure here never hides the
results of the other GPU tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _candidates(sizes, tau):
    """All length-compatible (probe, candidate) lists of a self-join, as CSR."""
    from hyset_gb300 import similarity
    probes, ends, cands = [], [], []
    for p in range(len(sizes)):
        ms = similarity.minsize("jaccard", int(sizes[p]), tau)
        lo = int(np.searchsorted(sizes, ms, side="left"))
        if lo < p:
            cands.append(np.arange(lo, p, dtype=np.uint32))
            probes.append(p)
            ends.append(sum(len(x) for x in cands))
    return (np.array(probes, np.uint32), np.array(ends, np.uint32),
            np.concatenate(cands) if cands else np.zeros(0, np.uint32))


def _reference_verifier(ctx, coll, probes, ends, cands, tau, scenario):
    import hyset_gb300 as hs
    from hyset_gb300.handlers import DeviceHandler
    dh = DeviceHandler(ctx, coll, coll, 32, scenario, False, 4096, 1 << 22, tau)
    out = hs.PairsHandler()
    dh.set_output_handler(out)
    start = 0
    for p, e in zip(probes.tolist(), ends.tolist()):
        dh.add_candidates(p, cands[start:e])
        start = e
    dh.flush()
    dh.close()
    return out.pairs


@pytest.mark.parametrize("scenario", [1, 2])
def test_noalloc_matches_allocating_verifier_twice(scenario):
    torch = pytest.importorskip("torch")
    import hyset_gb300 as hs
    from hyset_gb300 import _lib, synth

    lib = _lib.load()
    c = synth.generate(synth.C1, n_sets=1500, universe=1200, dup_frac=0.06, dup_edit_hi=0.3, seed=31)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    d_tok = torch.from_numpy(c.tokens.astype(np.int32)).to(dev)
    d_st = torch.from_numpy(c.starts.astype(np.int32)).to(dev)
    d_sz = torch.from_numpy(c.sizes.astype(np.int32)).to(dev)
    with hs.Context(0) as ctx:
        coll = ctx.upload(c.tokens, c.sizes, c.starts)
        for tau in (0.6, 0.8):  # two calls in a row on the shared scratch
            probes, ends, cands = _candidates(c.sizes, tau)
            expected = _reference_verifier(ctx, coll, probes, ends, cands, tau, scenario)
            d_pr = torch.from_numpy(probes.astype(np.int32)).to(dev)
            d_en = torch.from_numpy(ends.astype(np.int32)).to(dev)
            d_ca = torch.from_numpy(cands.astype(np.int32)).to(dev)
            cap = len(cands)
            d_pairs = torch.zeros((max(cap, 1), 2), dtype=torch.int32, device=dev)
            d_count = torch.zeros(1, dtype=torch.int64, device=dev)
            d_skip = torch.zeros(1, dtype=torch.int32, device=dev)
            stream = torch.cuda.current_stream(dev)
            ptr = lambda t: C.c_void_p(t.data_ptr())
            st = lib.hyset_verify_candidates_noalloc(
                ptr(d_tok), ptr(d_st), ptr(d_sz), ptr(d_tok), ptr(d_st), ptr(d_sz), int(c.sizes.max()),
                ptr(d_pr), ptr(d_en), ptr(d_ca), len(probes), _lib.SIM["jaccard"], tau, scenario,
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

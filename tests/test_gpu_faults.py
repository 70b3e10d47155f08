"""Host-side failure injection: allocation failures and truncated inputs.

The library reports failures as status codes.  Every device allocation goes
through one buffer type whose failure a test can force: while the environment
variable HYSET_FAULT_ALLOC holds N, the N-th allocation counted from when the
value was set fails as an out-of-memory error, before cudaMallocAsync is
called (no GPU fault is involved).  For each public operation the test forces
the first, second, third, ... allocation to fail until the operation needs no
more; every forced failure must surface as HYSET_E_NOMEM, the same context must
then run the operation correctly, and once the objects are released the
library must hold exactly the device memory it held before
(hyset_device_bytes)."""
import os

import numpy as np
import pytest

import hyset_gb300 as hs
import oracle
from hyset_gb300 import _lib, synth
from hyset_gb300.handlers import DeviceHandler, FgssHandler

pytestmark = pytest.mark.gpu

E_INVALID, E_NOMEM = 1, 3


@pytest.fixture(scope="module")
def data():
    c = synth.generate(synth.C1, n_sets=3000, universe=2000, dup_frac=0.05, dup_edit_hi=0.2, seed=77)
    s = synth.generate(synth.C1, n_sets=2000, universe=2000, dup_frac=0.05, dup_edit_hi=0.2, seed=78)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.7))
    exp_rs = oracle.as_set(oracle.brute_rs((c.tokens, c.starts, c.sizes), (s.tokens, s.starts, s.sizes), 0.7))
    return c, s, exp, exp_rs


def _self_join(ctx, d, **kw):
    c, _, exp, _ = d
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    try:
        return oracle.as_set(ctx.self_join(coll, threshold=0.7, **kw).pairs) == exp
    finally:
        coll.free()


def _host_join(ctx, d):
    c, _, exp, _ = d
    r = ctx.self_join_host(c.tokens, c.sizes, c.starts, threshold=0.7, technique="fgss", probe_major=True)
    return oracle.as_set(r.pairs) == exp


def _rs_join(ctx, d):
    c, s, _, exp_rs = d
    R = ctx.upload(c.tokens, c.sizes, c.starts)
    S = ctx.upload(s.tokens, s.sizes, s.starts)
    try:
        return oracle.as_set(ctx.rs_join(R, S, threshold=0.7, technique="fgss", probe_major=True).pairs) == exp_rs
    finally:
        R.free()
        S.free()


def _batch(ctx, d):
    c, s, exp, exp_rs = d
    R = ctx.upload(c.tokens, c.sizes, c.starts)
    S = ctx.upload(s.tokens, s.sizes, s.starts)
    try:
        res = ctx.batch_join([(R, None, dict(threshold=0.7)), (R, S, dict(threshold=0.7))])
        return oracle.as_set(res[0].pairs) == exp and oracle.as_set(res[1].pairs) == exp_rs
    finally:
        R.free()  # also drops the captured batch that reads it
        S.free()


def _parse(ctx, d):
    c = d[0]
    text = synth.format_text(c.tokens, c.starts, c.sizes).tobytes()
    coll = ctx.parse(text)
    try:
        tk, _, sz = coll.download()
        return np.array_equal(tk, c.tokens) and np.array_equal(sz, c.sizes)
    finally:
        coll.free()


def _verifier(ctx, d):
    c, _, _, _ = d
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    dh = None
    try:
        dh = DeviceHandler(ctx, coll, coll, 32, 1, False, 64, 4096, 0.7)
        out = hs.PairsHandler()
        dh.set_output_handler(out)
        for p in range(1, 400):
            dh.add_candidates(p, np.arange(0, p, dtype=np.uint32))
        dh.flush()
        exp = oracle.as_set(oracle.verify_csr((c.tokens, c.starts, c.sizes),
                                              np.arange(1, 400, dtype=np.uint32),
                                              np.cumsum(np.arange(1, 400)).astype(np.uint32),
                                              np.concatenate([np.arange(0, p, dtype=np.uint32)
                                                              for p in range(1, 400)]), 0.7)[0])
        return oracle.as_set(out.pairs) == exp
    finally:
        if dh is not None:
            dh.close()
        coll.free()


def _handler(ctx, d):
    c, _, exp, _ = d
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    hc = hs.from_arrays(c.tokens, c.sizes, 1000, 0.7)
    h = None
    try:
        h = FgssHandler(ctx, hc, coll, 1000, False, 0.7)
        out = hs.PairsHandler()
        h.set_output_handler(out)
        h.join(hs.Partition(0, hc.blocks), hs.Partition(0, hc.blocks))
        return oracle.as_set(out.pairs) == exp
    finally:
        if h is not None:
            h.close()
        coll.free()


OPS = {
    "self_join_auto": lambda ctx, d: _self_join(ctx, d),
    "self_join_token_major": lambda ctx, d: _self_join(ctx, d, technique="fgss"),
    "self_join_bitmap_sorted": lambda ctx, d: _self_join(ctx, d, technique="bitmap", bitmap=128, sort_pairs=True),
    "self_join_host": _host_join,
    "rs_join": _rs_join,
    "batch_join": _batch,
    "parse": _parse,
    "verifier": _verifier,
    "handler": _handler,
}


@pytest.mark.parametrize("name", list(OPS))
def test_forced_allocation_failures_are_clean(data, name):
    op = OPS[name]
    lib = _lib.load()
    base = lib.hyset_device_bytes()
    failures = 0
    for n in range(1, 500):
        ctx = hs.Context(0)  # the selector's weights are allocated before the fault is armed
        os.environ["HYSET_FAULT_ALLOC"] = str(n)
        try:
            ok = op(ctx, data)
            completed = True
        except hs.HysetError as e:
            assert e.status == E_NOMEM, (name, n, str(e))
            completed = False
        finally:
            os.environ.pop("HYSET_FAULT_ALLOC", None)
        if not completed:
            failures += 1
            ok = op(ctx, data)  # the same context recovers
        assert ok, (name, n)
        ctx.close()
        assert lib.hyset_device_bytes() == base, (name, n, lib.hyset_device_bytes(), base)
        if completed:
            break
    else:
        pytest.fail(f"{name}: still allocating after 500 forced failures")
    assert failures >= 1, name


def test_truncated_and_inconsistent_inputs_are_rejected(data):
    c = data[0]
    lib = _lib.load()
    base = lib.hyset_device_bytes()
    with hs.Context(0) as ctx:
        short = c.tokens[: c.tokens.size // 2]
        with pytest.raises(hs.HysetError) as e:  # sizes sum past the token array
            ctx.upload(short, c.sizes)
        assert e.value.status == E_INVALID
        with pytest.raises(hs.HysetError) as e:  # a set that reaches past the end
            ctx.upload(short, c.sizes, c.starts)
        assert e.value.status == E_INVALID
        with pytest.raises(hs.HysetError) as e:
            ctx.self_join_host(short, c.sizes, None, threshold=0.7)
        assert e.value.status == E_INVALID
        text = synth.format_text(c.tokens, c.starts, c.sizes).tobytes()
        cut = text[: len(text) // 2]
        cut = cut[: cut.rfind(b" ") + 1] + b" 12\n"  # an empty item (two spaces) where the text was cut
        with pytest.raises(hs.HysetError) as e:
            ctx.parse(cut)
        assert e.value.status == E_INVALID
        coll = ctx.parse(text[: text.rfind(b"\n", 0, len(text) // 2) + 1])  # cut at a line end: valid prefix
        assert coll.n > 0
        coll.free()
    assert lib.hyset_device_bytes() == base

"""The reference's collection text format parsed on the GPU
(hyset_collection_parse) against the CPU restatement of the reference reader
(oracle/reader.py, read_collection at include/hyset/collection.hpp:93-177).

CPU tests pin the restatement to the golden fixtures (the files the
reference's own reader parsed to produce the golden pairs).  GPU tests check
the parser byte for byte against the restatement, through joins against the
golden pairs, and on the malformed inputs the parser rejects."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, GOLDEN_SETS, load_golden
from oracle.reader import read_text, write_text

VALID = {
    "plain": b"1 2 3\n4 5 6\n",
    "no_final_newline": b"1 2 3\n4 5 6",
    "crlf": b"1 2 3\r\n4 5 6\r\n",
    "empty_lines": b"\n\n1 2\n\n\n3 4 5\n\n",
    "trailing_space": b"1 2 \n3 4 5 \n",
    "single_token_lines": b"7\n8\n9\n",
    "large_values": b"4294967290 4294967294\n",
    "leading_zeros": b"007 0010\n",
    "empty": b"",
    "only_newlines": b"\n\n\n",
}

# inputs the reference reads with a token 0 from an empty or non-numeric item
ZERO_ITEMS = {
    "double_space": b"1  2\n",
    "leading_space": b" 1 2\n",
    "space_before_cr": b"1 2 \r\n",
    "cr_line": b"1 2\n\r\n3 4\n",
}
OTHER_BAD = {
    "letter": b"1 2 x\n",
    "tab": b"1\t2\n",
    "lone_cr": b"1 2\r3 4\n",
    "eleven_digits": b"1 12345678901\n",
    "too_large": b"4294967296\n",
}


@pytest.mark.parametrize("name", GOLDEN_SETS)
def test_reader_restatement_reads_the_golden_files(name):
    tokens, starts, sizes, _ = load_golden(name)
    with open(os.path.join(GOLDEN, f"{name}.sets.txt"), "rb") as f:
        t, z, empty = read_text(f.read())
    assert empty == 0
    np.testing.assert_array_equal(t, tokens)
    np.testing.assert_array_equal(z, sizes)


def test_reader_restatement_edge_cases():
    t, z, e = read_text(VALID["trailing_space"])
    assert t.tolist() == [1, 2, 3, 4, 5] and z.tolist() == [2, 3] and e == 0
    t, z, e = read_text(VALID["empty_lines"])
    assert z.tolist() == [2, 3] and e == 0
    for name, text in ZERO_ITEMS.items():
        t, z, e = read_text(text)
        assert e > 0 and 0 in t.tolist(), name


def test_c_and_python_restatements_agree():
    cases = list(VALID.values()) + list(ZERO_ITEMS.values()) + [b"-5 +7\n", b" \n", b"  \n", b"1 2\r"]
    for name in GOLDEN_SETS:
        with open(os.path.join(GOLDEN, f"{name}.sets.txt"), "rb") as f:
            cases.append(f.read())
    for text in cases:
        a, b = oracle.read_text(text), read_text(text)
        assert a[0].tolist() == b[0].tolist() and a[1].tolist() == b[1].tolist() and a[2] == b[2], text[:40]


def test_format_text_matches_the_writer():
    from hyset_gb300 import synth
    c = synth.generate(synth.C2, n_sets=3000, seed=92)
    buf = synth.format_text(c.tokens, c.starts, c.sizes)
    assert buf.tobytes() == write_text(c.tokens, c.starts, c.sizes)


def test_write_text_round_trips():
    tokens, starts, sizes, _ = load_golden("c1_small")
    t, z, _ = read_text(write_text(tokens, starts, sizes))
    np.testing.assert_array_equal(t, tokens)
    np.testing.assert_array_equal(z, sizes)


@pytest.mark.gpu
@pytest.mark.parametrize("name", GOLDEN_SETS)
def test_gpu_parse_of_golden_files_joins_to_the_golden_pairs(ctx, name):
    tokens, starts, sizes, results = load_golden(name)
    coll = ctx.parse(os.path.join(GOLDEN, f"{name}.sets.txt"))
    t, st, z = coll.download()
    np.testing.assert_array_equal(t, tokens)
    np.testing.assert_array_equal(z, sizes)
    np.testing.assert_array_equal(st, starts)
    for tau, want in results.items():
        r = ctx.self_join(coll, threshold=tau)
        assert oracle.as_set(r.pairs) == {tuple(p) for p in want["pairs"]}, (name, tau)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(VALID))
def test_gpu_parse_matches_reader_on_valid_inputs(ctx, name):
    text = VALID[name]
    t, z, _ = read_text(text)
    coll = ctx.parse(text)
    gt, gs, gz = coll.download()
    np.testing.assert_array_equal(gt, t)
    np.testing.assert_array_equal(gz, z)
    if len(z):
        np.testing.assert_array_equal(gs, np.concatenate([[0], np.cumsum(z[:-1])]).astype(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(ZERO_ITEMS) + sorted(OTHER_BAD))
def test_gpu_parse_rejects_malformed_text(ctx, name):
    import hyset_gb300 as hs
    text = ZERO_ITEMS.get(name, OTHER_BAD.get(name))
    with pytest.raises(hs.HysetError, match="parse error at byte"):
        ctx.parse(text)


@pytest.mark.gpu
@pytest.mark.parametrize("crlf", [False, True])
def test_gpu_parse_large_synthetic_text(ctx, crlf):
    """Many 4 KiB tiles: numbers and lines cross tile boundaries."""
    from hyset_gb300 import synth
    c = synth.generate(synth.C2, n_sets=20000, seed=91)
    text = write_text(c.tokens, c.starts, c.sizes, crlf=crlf)
    assert len(text) > 100 * 4096
    coll = ctx.parse(text)
    gt, gs, gz = coll.download()
    np.testing.assert_array_equal(gt, c.tokens)
    np.testing.assert_array_equal(gz, c.sizes)
    np.testing.assert_array_equal(gs, c.starts)
    # texts ending near tile boundaries, with and without a final line end
    for target in (4090, 4095, 4096, 4097, 8190):
        end = text.index(b"\n", target) + 1
        for part in (text[:end], text[:end - 1], text[:end - (2 if crlf else 1)]):
            t, z, e = read_text(part)
            assert e == 0
            pt, _, pz = ctx.parse(part).download()
            np.testing.assert_array_equal(pt, t)
            np.testing.assert_array_equal(pz, z)


@pytest.mark.gpu
def test_gpu_parse_from_device_memory(ctx):
    torch = pytest.importorskip("torch")
    tokens, starts, sizes, _ = load_golden("c1_small")
    text = write_text(tokens, starts, sizes)
    d = torch.frombuffer(bytearray(text), dtype=torch.uint8).to("cuda")
    coll = ctx.parse((d.data_ptr(), d.numel()))
    gt, _, gz = coll.download()
    np.testing.assert_array_equal(gt, tokens)
    np.testing.assert_array_equal(gz, sizes)
    # an odd device offset (unaligned start) is copied to an aligned buffer first
    d2 = torch.frombuffer(bytearray(b"x" + text), dtype=torch.uint8).to("cuda")
    coll2 = ctx.parse((d2.data_ptr() + 1, d2.numel() - 1))
    gt2, _, _ = coll2.download()
    np.testing.assert_array_equal(gt2, tokens)


def _at_tile_edge(number: bytes, offset: int) -> bytes:
    """A valid collection whose one-token line `number` starts `offset` bytes
    before the first 4 KiB tile boundary (one-token lines before it, a
    two-token line after it: sizes stay sorted)."""
    p = 4096 - offset
    head = b"1\n" * (p // 2) if p % 2 == 0 else b"11\n" + b"1\n" * ((p - 3) // 2)
    assert len(head) == p
    return head + number + b"\n7 8\n"


@pytest.mark.gpu
@pytest.mark.parametrize("offset", range(1, 12))
def test_gpu_parse_numbers_across_the_tile_edge(ctx, offset):
    """A ten-digit number split by the tile boundary at every offset; an
    eleven-digit one and one of 2^32 must be rejected wherever they are cut."""
    import hyset_gb300 as hs
    text = _at_tile_edge(b"4294967294", offset)  # 0xFFFFFFFF is reserved
    t, z, _ = read_text(text)
    gt, _, gz = ctx.parse(text).download()
    np.testing.assert_array_equal(gt, t)
    np.testing.assert_array_equal(gz, z)
    assert 4294967294 in gt.tolist()
    with pytest.raises(hs.HysetError, match="parse error at byte"):
        ctx.parse(_at_tile_edge(b"12345678901", offset))
    with pytest.raises(hs.HysetError, match="parse error at byte"):
        ctx.parse(_at_tile_edge(b"4294967296", offset))


@pytest.mark.gpu
@pytest.mark.parametrize("digits", [9, 10, 11, 16, 17, 40])
def test_gpu_parse_digit_runs_across_chunks(ctx, digits):
    """Runs of 9 to 40 digits placed across the 16-byte chunk boundaries of a
    tile: up to ten digits parse (1111111111 is below 2^32), longer runs are
    rejected."""
    import hyset_gb300 as hs
    for lead in range(0, 17, 3):
        text = b"1\n" * lead + b"1" * digits + b"\n3 4\n"
        if digits <= 10:
            t, _, _ = read_text(text)
            np.testing.assert_array_equal(ctx.parse(text).download()[0], t)
        else:
            with pytest.raises(hs.HysetError, match="parse error at byte"):
                ctx.parse(text)


@pytest.mark.gpu
def test_gpu_parse_text_denser_after_the_first_chunk(ctx):
    """Host text is emitted chunk by chunk into buffers sized from the first
    64 MB; here the rest is five times denser, so the estimate overflows and the
    parse falls back to an exact second emission.  Same result as the reader."""
    sparse = b"1000000000\n" * ((64 << 20) // 11 + 7)
    dense = b"1 2\n" * (20 << 20)
    text = sparse + dense
    t, z, _ = oracle.read_text(text)
    gt, gs, gz = ctx.parse(text).download()
    np.testing.assert_array_equal(gt, t)
    np.testing.assert_array_equal(gz, z)
    np.testing.assert_array_equal(gs, np.concatenate([[0], np.cumsum(z[:-1])]).astype(np.uint32))

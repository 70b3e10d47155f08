"""Host-side logic: generator invariants, collection/blocks, partitioners (CPU only)."""
import numpy as np
import pytest

import hyset_gb300 as hs
from conftest import GOLDEN
from hyset_gb300 import partitioner, similarity, synth


def test_synth_deterministic_and_thread_independent():
    a = synth.generate(synth.C2, n_sets=5000, threads=1)
    b = synth.generate(synth.C2, n_sets=5000, threads=7)
    assert np.array_equal(a.tokens, b.tokens) and np.array_equal(a.sizes, b.sizes)


@pytest.mark.parametrize("spec", [synth.C1, synth.C2, synth.C3])
def test_synth_contract(spec):
    c = synth.generate(spec, n_sets=3000)
    assert c.tokens.min() >= 1  # token 0 is undefined in the reference
    assert np.all(np.diff(c.sizes.astype(np.int64)) >= 0)
    assert c.sizes.min() >= spec.size_min and c.sizes.max() <= spec.size_max
    for i in range(0, c.n, 97):
        s = c.set(i)
        assert np.all(np.diff(s.astype(np.int64)) > 0)


def test_synth_frequency_renumbering():
    c = synth.generate(synth.C1, n_sets=4000)
    freq = np.bincount(c.tokens)
    nz = freq[1:int(c.tokens.max()) + 1]
    assert np.all(np.diff(nz) >= 0)  # token ids ascend with global frequency


def test_read_collection_blocks_match_reference_layout(tmp_path):
    p = tmp_path / "c.txt"
    p.write_text("1 2 3\n\n1 2 3\n1 2 3 4\n2 3 4 5 6\n")
    hc = hs.read_collection(str(p), block_size=3, threshold=0.7)
    assert hc.n == 4 and hc.universe_size == 7
    assert [(b.start_id, b.end_id) for b in hc.blocks] == [(0, 2), (3, 3)]
    pre = [similarity.midprefix("jaccard", int(s), 0.7) for s in hc.sizes]
    assert hc.blocks[0].first_entry_position == 0
    assert hc.blocks[0].last_entry_position == sum(pre[:3])
    assert hc.blocks[1].last_entry_position == sum(pre)
    assert hc.max_entries == max(b.entries for b in hc.blocks)


def test_partitioners():
    c = synth.generate(synth.C1, n_sets=1000)
    hc = hs.from_arrays(c.tokens, c.sizes, 100, 0.8)
    parts = partitioner.even(hc.blocks, 3)
    assert [len(p.blocks) for p in parts] == [4, 4, 2]
    comp, small, large = partitioner.dichotomize(hc.blocks, 40)
    assert len(comp.blocks) == 10 and len(small.blocks) == 4 and len(large.blocks) == 6


def test_output_handlers(tmp_path):
    ph = hs.PairsHandler()
    ph.add_pairs(np.array([[3, 1], [2, 0]], np.uint32))
    ch = hs.CountHandler()
    ch.add_count(5)
    assert hs.count([ph, ch]) == 7
    out = tmp_path / "o.txt"
    assert hs.write_to_file([ph], str(out))
    assert out.read_text() == "3 1\n2 0\n"

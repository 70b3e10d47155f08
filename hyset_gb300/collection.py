"""Host collection and blocks, mirroring include/hyset/collection.hpp and structs.hpp.

read_collection parses the reference's text format (one set per line,
space-separated ascending tokens, lines ordered by set size) into CSR arrays,
the per-set prefix starts (midprefix tokens, collection.hpp:128-142) and
fixed-size blocks of `block_size` consecutive sets (collection.hpp:147-171).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import similarity


@dataclass
class Block:
    """hyset::structs::block (structs.hpp:10-54)."""
    id: int
    start_id: int
    end_id: int
    first_entry_position: int
    last_entry_position: int
    num_tokens: int

    @property
    def size(self) -> int:
        return self.end_id - self.start_id + 1

    @property
    def entries(self) -> int:
        return self.last_entry_position - self.first_entry_position


@dataclass
class Partition:
    """hyset::structs::partition (structs.hpp:105-148), block-based form."""
    id: int
    blocks: List[Block] = field(default_factory=list)

    def start_id(self) -> int:
        return self.blocks[0].start_id

    def end_id(self) -> int:
        return self.blocks[-1].end_id

    def size(self) -> int:
        return self.end_id() - self.start_id() + 1


@dataclass
class HostCollection:
    tokens: np.ndarray         # uint32 [T]
    starts: np.ndarray         # uint32 [n]
    sizes: np.ndarray          # uint32 [n]
    prefix_starts: np.ndarray  # uint64 [n]
    universe_size: int         # max token + 1
    max_entries: int           # largest block's prefix-entry count
    blocks: List[Block]

    @property
    def n(self) -> int:
        return int(self.sizes.shape[0])

    def set(self, i: int) -> np.ndarray:
        s = int(self.starts[i])
        return self.tokens[s:s + int(self.sizes[i])]


def from_arrays(tokens, sizes, block_size: int, threshold: float, sim: str = "jaccard") -> HostCollection:
    tokens = np.ascontiguousarray(tokens, dtype=np.uint32)
    sizes = np.ascontiguousarray(sizes, dtype=np.uint32)
    n = int(sizes.size)
    starts = np.zeros(n, dtype=np.uint64)
    if n:
        np.cumsum(sizes[:-1], out=starts[1:])
    if n and starts[-1] + sizes[-1] >= (1 << 32):
        raise ValueError("more than 2^32 tokens")
    prefix = similarity.midprefix_array(sim, sizes, threshold)
    prefix_starts = np.zeros(n, dtype=np.uint64)
    if n:
        np.cumsum(prefix[:-1], out=prefix_starts[1:])
    total_prefix = int(prefix.sum()) if n else 0
    blocks: List[Block] = []
    max_entries = 0
    for b, lo in enumerate(range(0, n, block_size)):
        hi = min(n, lo + block_size) - 1
        first = int(prefix_starts[lo])
        last = int(prefix_starts[hi + 1]) if hi + 1 < n else total_prefix
        ntok = int(sizes[lo:hi + 1].sum())
        blk = Block(b, lo, hi, first, last, ntok)
        max_entries = max(max_entries, blk.entries)
        blocks.append(blk)
    universe = int(tokens.max()) + 1 if tokens.size else 1
    return HostCollection(tokens, starts.astype(np.uint32), sizes, prefix_starts, universe, max_entries, blocks)


def read_collection(path: str, block_size: int, threshold: float, sim: str = "jaccard") -> HostCollection:
    """read_collection<Similarity> (collection.hpp:93-177): empty lines are skipped."""
    toks, sizes = [], []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line:
                continue
            row = np.array(line.split(), dtype=np.uint32)
            toks.append(row)
            sizes.append(row.size)
    tokens = np.concatenate(toks) if toks else np.zeros(0, np.uint32)
    return from_arrays(tokens, np.array(sizes, dtype=np.uint32), block_size, threshold, sim)


def one_partition(hc: HostCollection) -> Partition:
    return Partition(0, list(hc.blocks))

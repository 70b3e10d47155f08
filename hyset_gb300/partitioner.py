"""Block partitioners, mirroring include/hyset/partitioner.hpp."""
from __future__ import annotations

import math
from typing import List

from .collection import Block, Partition


def even(blocks: List[Block], num_partitions: int) -> List[Partition]:
    """partitioner::even (partitioner.hpp:11-30)."""
    size = int(math.ceil(len(blocks) / float(num_partitions)))
    parts = []
    for pid, i in enumerate(range(0, len(blocks), max(size, 1))):
        parts.append(Partition(pid, list(blocks[i:min(len(blocks), i + size)])))
    return parts


def dichotomize(blocks: List[Block], split: float) -> List[Partition]:
    """partitioner::dichotomize (partitioner.hpp:32-68): [complete, small, large]."""
    portion = int(math.ceil((split / 100.0) * len(blocks)))
    return [Partition(0, list(blocks)), Partition(1, list(blocks[:portion])), Partition(2, list(blocks[portion:]))]

"""Result sinks, mirroring include/hyset/output.hpp."""
from __future__ import annotations

from typing import Iterable, List

import numpy as np


class OutputHandler:
    def add_pairs(self, pairs: np.ndarray) -> None:  # pragma: no cover - interface
        raise NotImplementedError

    def add_count(self, count: int) -> None:  # pragma: no cover - interface
        raise NotImplementedError

    def get_count(self) -> int:  # pragma: no cover - interface
        raise NotImplementedError


class CountHandler(OutputHandler):
    """output::count_handler (output.hpp:19-26)."""

    def __init__(self):
        self.count = 0

    def add_pairs(self, pairs: np.ndarray) -> None:
        self.count += int(np.asarray(pairs).reshape(-1, 2).shape[0])

    def add_count(self, count: int) -> None:
        self.count += int(count)

    def get_count(self) -> int:
        return self.count


class PairsHandler(OutputHandler):
    """output::pairs_handler (output.hpp:28-37); pairs are (first, second) rows."""

    def __init__(self):
        self._chunks: List[np.ndarray] = []

    def add_pairs(self, pairs: np.ndarray) -> None:
        p = np.asarray(pairs, dtype=np.uint32).reshape(-1, 2)
        if p.shape[0]:
            self._chunks.append(p.copy())

    def add_count(self, count: int) -> None:
        raise TypeError("a pairs handler needs the pairs, not a count")

    @property
    def pairs(self) -> np.ndarray:
        if not self._chunks:
            return np.zeros((0, 2), np.uint32)
        if len(self._chunks) > 1:
            self._chunks = [np.concatenate(self._chunks)]
        return self._chunks[0]

    def get_count(self) -> int:
        return int(sum(c.shape[0] for c in self._chunks))


def write_to_file(handlers: Iterable[OutputHandler], path: str) -> bool:
    """output::write_to_file (output.hpp:40-76): one "first second" line per pair."""
    try:
        with open(path, "w") as f:
            for h in handlers:
                for a, b in np.asarray(h.pairs).tolist():
                    f.write(f"{a} {b}\n")
        return True
    except OSError:
        return False


def count(handlers: Iterable[OutputHandler]) -> int:
    """output::count (output.hpp:78-93)."""
    return sum(h.get_count() for h in handlers)

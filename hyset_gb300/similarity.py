"""Similarity bounds on the host, in the reference's double expressions.

Restates include/hyset/similarity.hpp:11-54 (jaccard) and adds cosine and dice
in the same style (the reference has only jaccard).  Python floats are IEEE
doubles and math.ceil/int() match C's ceil and truncation, so these values are
the ones the reference computes.  The device never evaluates them: the library
uploads host-computed tables.
"""
from __future__ import annotations

import math

import numpy as np


def _imin(a: int, b: int) -> int:  # hyset::min(int, int), helpers.hpp:41-44
    return b if a > b else a


def sim_minoverlap(sim: str, l1: int, l2: int, t: float) -> int:
    if sim == "cosine":
        return int(math.ceil(t * math.sqrt(float(l1) * float(l2))))
    if sim == "dice":
        return int(math.ceil(t * float(l1 + l2) / 2.0))
    return int(math.ceil(float(l1 + l2) * t / (1 + t)))


def minsize(sim: str, l: int, t: float) -> int:
    if sim == "cosine":
        return int(math.ceil(t * t * float(l)))
    if sim == "dice":
        return int(math.ceil(t * float(l) / (2.0 - t)))
    return int(math.ceil(t * float(l)))


def maxsize(sim: str, l: int, t: float) -> int:
    if sim == "cosine":
        return int(float(l) / (t * t))
    if sim == "dice":
        return int((2.0 - t) * float(l) / t)
    return int(float(l) / t)


def minoverlap(sim: str, l1: int, l2: int, t: float) -> int:
    return _imin(l2, _imin(l1, sim_minoverlap(sim, l1, l2, t)))


def maxprefix(sim: str, l: int, t: float) -> int:
    return _imin(l, l - minsize(sim, l, t) + 1)


def midprefix(sim: str, l: int, t: float) -> int:
    return _imin(l, l - minoverlap(sim, l, l, t) + 1)


def midprefix_array(sim: str, sizes: np.ndarray, t: float) -> np.ndarray:
    """midprefix for every size (vectorised through a table of distinct sizes)."""
    sizes = np.asarray(sizes, dtype=np.int64)
    if sizes.size == 0:
        return np.zeros(0, np.int64)
    top = int(sizes.max())
    tab = np.array([midprefix(sim, l, t) if l else 0 for l in range(top + 1)], dtype=np.int64)
    return tab[sizes]

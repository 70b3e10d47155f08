"""Reference-shaped join handlers over the C ABI.

    BitmapHandler  ~ hyset::algorithms::device::bitmap::handler   (device_algorithms.hpp:120-260)
    FgssHandler    ~ hyset::algorithms::device::fgssjoin::handler (device_algorithms.hpp:305-446)
    DeviceHandler  ~ hyset::algorithms::hybrid::device_handler    (hybrid_algorithms.hpp:16-205)

Same constructor arguments (minus the timer), same setOutputHandler / join
calls, same result semantics: pairs (probe id, indexed id) appended to the
output handler, or the count added to a count handler when `aggregate`.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence, Union

import numpy as np

from . import _lib
from ._lib import SIM, TECH, Block as CBlock, U32P, check
from .api import Context, DeviceCollection
from .collection import Block, HostCollection, Partition
from .output import OutputHandler


def _cblock(b: Block) -> CBlock:
    return CBlock(b.id, b.start_id, b.end_id, b.first_entry_position, b.last_entry_position, b.num_tokens,
                  b.entries, b.size)


def _cblocks(blocks: Sequence[Block]):
    arr = (CBlock * max(len(blocks), 1))()
    for i, b in enumerate(blocks):
        arr[i] = _cblock(b)
    return arr


class _BlockHandler:
    _technique = "fgss"

    def __init__(self, ctx: Context, host_collection: HostCollection, device_collection: DeviceCollection,
                 bitmap_size: int, block_size: int, aggregate: bool, threshold: float, sim: str = "jaccard"):
        self._ctx = ctx
        self._lib = _lib.load()
        self.host_collection = host_collection
        self.block_size = block_size
        self.aggregate = bool(aggregate)
        self.threshold = threshold
        self.output: OutputHandler = None
        h = C.c_void_p()
        check(self._lib.hyset_handler_create(ctx.handle, device_collection.handle, TECH[self._technique], SIM[sim],
                                             int(bitmap_size), int(block_size), int(self.aggregate),
                                             float(threshold), C.byref(h)), ctx.handle)
        self.handle = h
        self._coll = device_collection

    def set_output_handler(self, output: OutputHandler) -> None:
        self.output = output

    def join(self, first: Union[Block, Partition], second: Union[Block, Partition]) -> None:
        if isinstance(first, Partition):
            a, b = _cblocks(first.blocks), _cblocks(second.blocks)
            check(self._lib.hyset_handler_join_partitions(self.handle, a, len(first.blocks), b, len(second.blocks)),
                  self._ctx.handle)
        else:
            a, b = _cblock(first), _cblock(second)
            check(self._lib.hyset_handler_join_blocks(self.handle, C.byref(a), C.byref(b)), self._ctx.handle)
        self._drain()

    def _drain(self) -> None:
        cnt = C.c_uint64()
        ptr = C.c_void_p()
        check(self._lib.hyset_handler_output(self.handle, C.byref(cnt), C.byref(ptr)), self._ctx.handle)
        n = int(cnt.value)
        if self.output is not None:
            if self.aggregate:
                self.output.add_count(n)
            elif n:
                self.output.add_pairs(np.ctypeslib.as_array(C.cast(ptr, U32P), (2 * n,)).reshape(n, 2))
        check(self._lib.hyset_handler_clear_output(self.handle), self._ctx.handle)

    def close(self) -> None:
        if self.handle:
            self._lib.hyset_handler_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BitmapHandler(_BlockHandler):
    _technique = "bitmap"

    def __init__(self, ctx, host_collection, device_collection, bitmap_size: int, block_size: int,
                 aggregate: bool, threshold: float, sim: str = "jaccard"):
        super().__init__(ctx, host_collection, device_collection, bitmap_size, block_size, aggregate, threshold, sim)


class FgssHandler(_BlockHandler):
    _technique = "fgss"

    def __init__(self, ctx, host_collection, device_collection, block_size: int, aggregate: bool,
                 threshold: float, sim: str = "jaccard"):
        super().__init__(ctx, host_collection, device_collection, 0, block_size, aggregate, threshold, sim)


class DeviceHandler:
    """Verifies explicit candidate lists on the GPU (scenario 1: lane per
    candidate, scenario 2: warp per candidate with merge-path steps)."""

    def __init__(self, ctx: Context, indexed: DeviceCollection, probe: DeviceCollection, threads: int,
                 scenario: int, aggregate: bool, max_probes: int, max_candidates: int, threshold: float,
                 sim: str = "jaccard"):
        self._ctx = ctx
        self._lib = _lib.load()
        self.aggregate = bool(aggregate)
        self.output: OutputHandler = None
        h = C.c_void_p()
        check(self._lib.hyset_verifier_create(ctx.handle, indexed.handle, probe.handle, SIM[sim], int(threads),
                                              int(scenario), int(self.aggregate), int(max_probes),
                                              int(max_candidates), float(threshold), C.byref(h)), ctx.handle)
        self.handle = h

    def set_max_set_size(self, size: int) -> None:
        """Kept for interface parity; probes longer than the shared-memory stage are read from HBM."""

    def set_wait_limit(self, microseconds: int) -> None:
        """How long the persistent verifier kernel waits for published
        candidates before it ends (the next publication starts it again)."""
        check(self._lib.hyset_verifier_set_wait(self.handle, int(microseconds)), self._ctx.handle)

    def status(self) -> int:
        """0, or 5 (HYSET_E_TIMEOUT) when the last verifier kernel ended
        because no candidates arrived within the wait limit."""
        return int(self._lib.hyset_verifier_status(self.handle))

    def set_output_handler(self, output: OutputHandler) -> None:
        self.output = output

    def add_candidates(self, probe_id: int, candidates) -> None:
        c = np.ascontiguousarray(candidates, dtype=np.uint32)
        check(self._lib.hyset_verifier_add_candidates(self.handle, int(probe_id), c.ctypes.data_as(U32P), c.size),
              self._ctx.handle)

    def flush(self) -> None:
        check(self._lib.hyset_verifier_flush(self.handle), self._ctx.handle)
        cnt = C.c_uint64()
        ptr = C.c_void_p()
        check(self._lib.hyset_verifier_output(self.handle, C.byref(cnt), C.byref(ptr)), self._ctx.handle)
        n = int(cnt.value)
        if self.output is not None:
            if self.aggregate:
                self.output.add_count(n - getattr(self, "_reported", 0))
            elif n > getattr(self, "_reported", 0):
                arr = np.ctypeslib.as_array(C.cast(ptr, U32P), (2 * n,)).reshape(n, 2)
                self.output.add_pairs(arr[getattr(self, "_reported", 0):])
        self._reported = n

    join = flush

    def close(self) -> None:
        if self.handle:
            self._lib.hyset_verifier_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

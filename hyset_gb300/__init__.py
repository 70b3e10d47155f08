"""hyset_gb300 — GB300-native (sm_103a) exact set-similarity join.

A from-scratch CUDA implementation of chribell/hyset's GPU join path behind a
C ABI (include/hyset_gb300.h).  This package is the Python host side: ctypes
bindings, the reference-shaped handlers, and the host collection model.
"""
from .api import Context, DeviceCollection, JoinResult, make_opts, sorted_pairs  # noqa: F401
from .collection import Block, HostCollection, Partition, from_arrays, read_collection  # noqa: F401
from .output import CountHandler, PairsHandler, count, write_to_file  # noqa: F401
from ._lib import HysetError, HysetLibraryError, LIB_PATH  # noqa: F401

__all__ = ["Context", "DeviceCollection", "JoinResult", "make_opts", "sorted_pairs", "Block", "HostCollection",
           "Partition", "from_arrays", "read_collection", "CountHandler", "PairsHandler", "count", "write_to_file",
           "HysetError", "HysetLibraryError", "LIB_PATH"]

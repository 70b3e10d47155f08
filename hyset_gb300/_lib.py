"""ctypes binding of libhyset_gb300.so (include/hyset_gb300.h).

The product path has no CPU fallback: if the shared library is missing or
cannot be loaded, importing anything that needs it raises HysetLibraryError.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libhyset_gb300.so")

U32P = C.POINTER(C.c_uint32)


class HysetLibraryError(RuntimeError):
    """libhyset_gb300.so is missing or failed to load."""


class HysetError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"hyset status {status} ({STATUS_NAMES.get(status, '?')}): {message}")
        self.status = status


STATUS_NAMES = {0: "OK", 1: "E_INVALID", 2: "E_CUDA", 3: "E_NOMEM", 4: "E_OVERFLOW", 5: "E_TIMEOUT",
                6: "E_UNSUPPORTED", 7: "E_NODEVICE"}
SIM = {"jaccard": 0, "cosine": 1, "dice": 2}
TECH = {"auto": 0, "bitmap": 1, "fgss": 2, "direct": 3}
TECH_NAMES = {v: k for k, v in TECH.items()}
SELECTOR_NAMES = {-1: "explicit", 0: "rules", 1: "cost_model", 2: "mlp"}
N_FEATURES, MLP_PARAMS, COST_TERMS = 12, 5187, 9


class JoinOpts(C.Structure):
    _fields_ = [("sim", C.c_int), ("threshold", C.c_double), ("technique", C.c_int), ("bitmap_bits", C.c_uint32),
                ("count_only", C.c_uint32), ("verify_mode", C.c_uint32), ("sort_pairs", C.c_uint32),
                ("pair_capacity", C.c_uint64), ("device_pairs", C.c_uint32), ("collect_stats", C.c_uint32),
                ("probe_begin", C.c_uint32), ("probe_end", C.c_uint32), ("probe_major", C.c_uint32),
                ("fgss_batch", C.c_uint32), ("orientation", C.c_uint32)]


class Block(C.Structure):
    """hyset::structs::block (include/hyset/structs.hpp:10-54)."""
    _fields_ = [("id", C.c_uint32), ("start_id", C.c_uint32), ("end_id", C.c_uint32),
                ("first_entry_position", C.c_uint32), ("last_entry_position", C.c_uint32),
                ("num_tokens", C.c_uint32), ("entries", C.c_uint32), ("size", C.c_uint32)]


class JoinDesc(C.Structure):
    _fields_ = [("indexed", C.c_void_p), ("probe", C.c_void_p), ("opts", JoinOpts)]


# every exported symbol of include/hyset_gb300.h: name -> (restype, argtypes)
PROTOTYPES = {
    "hyset_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "hyset_destroy": (None, [C.c_void_p]),
    "hyset_last_error": (C.c_char_p, [C.c_void_p]),
    "hyset_default_opts": (None, [C.POINTER(JoinOpts)]),
    "hyset_device_bytes": (C.c_uint64, []),
    "hyset_collection_upload": (C.c_int, [C.c_void_p, U32P, C.c_uint64, U32P, U32P, C.c_uint32,
                                          C.POINTER(C.c_void_p)]),
    "hyset_collection_from_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                               C.c_uint32, C.POINTER(C.c_void_p)]),
    "hyset_verify_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_uint32, C.c_void_p, C.POINTER(C.c_void_p)]),
    "hyset_self_join_host": (C.c_int, [C.c_void_p, U32P, C.c_uint64, U32P, U32P, C.c_uint32, C.c_void_p,
                                       C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "hyset_collection_parse": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "hyset_collection_free": (None, [C.c_void_p, C.c_void_p]),
    "hyset_collection_num_sets": (C.c_uint32, [C.c_void_p]),
    "hyset_collection_num_tokens": (C.c_uint64, [C.c_void_p]),
    "hyset_collection_download": (C.c_int, [C.c_void_p, C.c_void_p, U32P, U32P, U32P]),
    "hyset_self_join": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(JoinOpts), C.POINTER(C.c_void_p)]),
    "hyset_rs_join": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(JoinOpts), C.POINTER(C.c_void_p)]),
    "hyset_batch_join": (C.c_int, [C.c_void_p, C.POINTER(JoinDesc), C.c_uint32, C.POINTER(C.c_void_p)]),
    "hyset_result_count": (C.c_uint64, [C.c_void_p]),
    "hyset_result_pairs": (C.c_void_p, [C.c_void_p]),
    "hyset_result_technique": (C.c_int, [C.c_void_p]),
    "hyset_result_bitmap_bits": (C.c_uint32, [C.c_void_p]),
    "hyset_result_verify_mode": (C.c_uint32, [C.c_void_p]),
    "hyset_result_probe_batch": (C.c_uint32, [C.c_void_p]),
    "hyset_result_split": (C.c_uint32, [C.c_void_p, C.POINTER(C.c_int)]),
    "hyset_result_device_ms": (C.c_double, [C.c_void_p]),
    "hyset_result_kernel_ms": (C.c_double, [C.c_void_p]),
    "hyset_result_device_pairs": (C.c_void_p, [C.c_void_p]),
    "hyset_result_stats": (C.c_uint32, [C.c_void_p, C.POINTER(C.c_uint64), C.c_uint32]),
    "hyset_result_launches": (C.c_uint64, [C.c_void_p]),
    "hyset_result_free": (None, [C.c_void_p]),
    "hyset_handler_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_int,
                                       C.c_double, C.POINTER(C.c_void_p)]),
    "hyset_handler_join_blocks": (C.c_int, [C.c_void_p, C.POINTER(Block), C.POINTER(Block)]),
    "hyset_handler_join_partitions": (C.c_int, [C.c_void_p, C.POINTER(Block), C.c_uint32, C.POINTER(Block),
                                                C.c_uint32]),
    "hyset_handler_output": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_void_p)]),
    "hyset_handler_clear_output": (C.c_int, [C.c_void_p]),
    "hyset_handler_destroy": (None, [C.c_void_p]),
    "hyset_verifier_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_uint32, C.c_uint32,
                                        C.c_int, C.c_uint32, C.c_uint32, C.c_double, C.POINTER(C.c_void_p)]),
    "hyset_verifier_add_candidates": (C.c_int, [C.c_void_p, C.c_uint32, U32P, C.c_uint32]),
    "hyset_verifier_flush": (C.c_int, [C.c_void_p]),
    "hyset_verifier_set_wait": (C.c_int, [C.c_void_p, C.c_uint64]),
    "hyset_verifier_status": (C.c_int, [C.c_void_p]),
    "hyset_verifier_output": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_void_p)]),
    "hyset_verifier_destroy": (None, [C.c_void_p]),
    "hyset_join_features": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(JoinOpts),
                                      C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "hyset_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "hyset_mlp_grad": (C.c_int, [C.c_void_p] * 5 + [C.c_uint32, C.c_void_p, C.c_void_p]),
    "hyset_mlp_train": (C.c_int, [C.c_void_p] * 5 + [C.c_uint32, C.c_uint32, C.c_float, C.c_float, C.c_void_p]),
    "hyset_selector_set": (C.c_int, [C.c_void_p] * 5),
    "hyset_width_selector_set": (C.c_int, [C.c_void_p] * 4),
    "hyset_result_selector": (C.c_int, [C.c_void_p]),
    "hyset_verify_candidates_noalloc": (C.c_int, [C.c_void_p] * 6 + [C.c_uint32] + [C.c_void_p] * 3 +
                                        [C.c_uint32, C.c_int, C.c_double, C.c_uint32, C.c_void_p, C.c_uint64,
                                         C.c_void_p, C.c_void_p, C.c_void_p]),
}

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise HysetLibraryError(f"{path} not found: run `python -c 'import __graft_entry__ as g; g.build()'`")
    try:
        lib = C.CDLL(path)
    except OSError as e:  # pragma: no cover - depends on the machine
        raise HysetLibraryError(f"cannot load {path}: {e}") from e
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, ctx=None) -> None:
    if status != 0:
        msg = load().hyset_last_error(ctx).decode() if ctx else ""
        raise HysetError(status, msg)

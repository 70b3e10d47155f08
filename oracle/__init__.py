"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py, always as the checker or the timed CPU
reference, never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")
REF_JOIN = os.path.join(_HERE, "_ref", "ref_join")
SIM = {"jaccard": 0, "cosine": 1, "dice": 2}
U32P = C.POINTER(C.c_uint32)

_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            subprocess.run(["make", "-C", _HERE, "liboracle.so"], check=True, capture_output=True)
        lib = C.CDLL(LIB_PATH)
        for name in ("oracle_minoverlap",):
            getattr(lib, name).argtypes = [C.c_int, C.c_uint32, C.c_uint32, C.c_double]
            getattr(lib, name).restype = C.c_uint32
        for name in ("oracle_minsize", "oracle_maxsize", "oracle_maxprefix", "oracle_midprefix"):
            getattr(lib, name).argtypes = [C.c_int, C.c_uint32, C.c_double]
            getattr(lib, name).restype = C.c_uint32
        lib.oracle_join.argtypes = [U32P, U32P, U32P, C.c_uint32, C.c_uint32, C.c_int, C.c_double, C.c_int,
                                    C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
        lib.oracle_join.restype = C.c_void_p
        lib.oracle_join_multi.argtypes = [U32P, U32P, U32P, C.c_uint32, C.c_uint32, C.c_int, C.c_double, C.c_int,
                                          C.c_int]
        lib.oracle_join_multi.restype = C.c_void_p
        lib.oracle_join_multi_range.argtypes = [U32P, U32P, U32P, C.c_uint32, C.c_uint32, C.c_int, C.c_double,
                                                C.c_int, C.c_int, C.c_uint32, C.c_uint32]
        lib.oracle_join_multi_range.restype = C.c_void_p
        for name in ("oracle_last_timing", "oracle_last_multi_timing"):
            getattr(lib, name).argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
            getattr(lib, name).restype = None
        lib.oracle_brute.argtypes = [U32P, U32P, U32P, C.c_uint32, C.c_int, C.c_double]
        lib.oracle_brute.restype = C.c_void_p
        lib.oracle_brute_rs.argtypes = [U32P, U32P, U32P, C.c_uint32, U32P, U32P, U32P, C.c_uint32, C.c_int,
                                        C.c_double]
        lib.oracle_brute_rs.restype = C.c_void_p
        lib.oracle_pairs_count.argtypes = [C.c_void_p]
        lib.oracle_pairs_count.restype = C.c_uint64
        lib.oracle_pairs_data.argtypes = [C.c_void_p]
        lib.oracle_pairs_data.restype = U32P
        lib.oracle_pairs_free.argtypes = [C.c_void_p]
        lib.oracle_pairs_free.restype = None
        _lib = lib
    return _lib


def _p(a: np.ndarray):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    return a, a.ctypes.data_as(U32P)


def _take(h) -> np.ndarray:
    lib = _load()
    if not h:
        raise RuntimeError("oracle failed (allocation or bad range)")
    try:
        n = lib.oracle_pairs_count(h)
        if n == 0:
            return np.zeros((0, 2), np.uint32)
        return np.ctypeslib.as_array(lib.oracle_pairs_data(h), (2 * n,)).reshape(n, 2).copy()
    finally:
        lib.oracle_pairs_free(h)


def universe_of(tokens: np.ndarray) -> int:
    return int(tokens.max()) + 1 if tokens.size else 1


def join(tokens, starts, sizes, threshold, sim="jaccard", algorithm="allpairs", index_range=None,
         probe_range=None) -> np.ndarray:
    """AllPairs / PPJoin restated from include/hyset/host_algorithms.hpp; pairs (probe, indexed)."""
    lib = _load()
    t, tp = _p(tokens)
    s, sp = _p(starts)
    z, zp = _p(sizes)
    n = len(z)
    if n == 0:
        return np.zeros((0, 2), np.uint32)
    ilo, ihi = index_range if index_range else (0, n - 1)
    plo, phi = probe_range if probe_range else (0, n - 1)
    return _take(lib.oracle_join(tp, sp, zp, n, universe_of(t), SIM[sim], float(threshold),
                                 1 if algorithm == "ppjoin" else 0, ilo, ihi, plo, phi))


def join_multi(tokens, starts, sizes, threshold, threads, sim="jaccard", algorithm="allpairs") -> np.ndarray:
    """cpu_multi semantics (src/cpu_multi.cu): sqrt-balanced probe ranges on `threads` threads."""
    lib = _load()
    t, tp = _p(tokens)
    s, sp = _p(starts)
    z, zp = _p(sizes)
    return _take(lib.oracle_join_multi(tp, sp, zp, len(z), universe_of(t), SIM[sim], float(threshold),
                                       1 if algorithm == "ppjoin" else 0, int(threads)))


def join_multi_range(tokens, starts, sizes, threshold, threads, probe_range, sim="jaccard",
                     algorithm="allpairs") -> np.ndarray:
    """cpu_multi semantics restricted to probes [lo, hi] (a bounded sample)."""
    lib = _load()
    t, tp = _p(tokens)
    s, sp = _p(starts)
    z, zp = _p(sizes)
    lo, hi = probe_range
    return _take(lib.oracle_join_multi_range(tp, sp, zp, len(z), universe_of(t), SIM[sim], float(threshold),
                                             1 if algorithm == "ppjoin" else 0, int(threads), int(lo), int(hi)))


def last_timing(multi: bool = False):
    """(index seconds, join seconds) of the last oracle join on this thread (or the last multi join)."""
    a, b = C.c_double(), C.c_double()
    (_load().oracle_last_multi_timing if multi else _load().oracle_last_timing)(C.byref(a), C.byref(b))
    return a.value, b.value


def brute(tokens, starts, sizes, threshold, sim="jaccard") -> np.ndarray:
    lib = _load()
    t, tp = _p(tokens)
    s, sp = _p(starts)
    z, zp = _p(sizes)
    return _take(lib.oracle_brute(tp, sp, zp, len(z), SIM[sim], float(threshold)))


def brute_rs(r, s, threshold, sim="jaccard") -> np.ndarray:
    """r, s: (tokens, starts, sizes) triples.  Pairs (probe s, indexed r)."""
    lib = _load()
    rt, rtp = _p(r[0]); rs_, rsp = _p(r[1]); rz, rzp = _p(r[2])
    st, stp = _p(s[0]); ss_, ssp = _p(s[1]); sz, szp = _p(s[2])
    return _take(lib.oracle_brute_rs(rtp, rsp, rzp, len(rz), stp, ssp, szp, len(sz), SIM[sim], float(threshold)))


def bounds(sim: str, threshold: float, length: int):
    lib = _load()
    k = SIM[sim]
    return dict(minsize=lib.oracle_minsize(k, length, threshold), maxsize=lib.oracle_maxsize(k, length, threshold),
                maxprefix=lib.oracle_maxprefix(k, length, threshold),
                midprefix=lib.oracle_midprefix(k, length, threshold))


def minoverlap(sim: str, l1: int, l2: int, threshold: float) -> int:
    return int(_load().oracle_minoverlap(SIM[sim], l1, l2, threshold))


def ref_available() -> bool:
    return os.path.exists(REF_JOIN)


def ref_join(path: str, threshold: float, algorithm="allpairs", mode="whole", block=10000) -> np.ndarray:
    """Runs the reference's own host join (oracle/_ref/ref_join) on a text collection."""
    out = subprocess.run([REF_JOIN, path, repr(float(threshold)), algorithm, mode, str(block)],
                         capture_output=True, text=True, check=True).stdout.splitlines()
    rows = [tuple(map(int, l.split())) for l in out if l and not l.startswith("#")]
    return np.array(rows, dtype=np.uint32).reshape(-1, 2)


def as_set(pairs: np.ndarray) -> set:
    return set(map(tuple, np.asarray(pairs).reshape(-1, 2).tolist()))


def read_text(text: bytes):
    """(tokens, sizes, empty_items) as the reference's reader reads the text
    (C restatement, oracle_read_text)."""
    lib = _load()
    fn = lib.oracle_read_text
    fn.restype = C.c_uint64
    fn.argtypes = [C.c_char_p, C.c_uint64, U32P, C.c_uint64, U32P, C.c_uint64, C.POINTER(C.c_uint64),
                   C.POINTER(C.c_uint64)]
    cap = len(text) // 2 + 2
    tok = np.empty(cap, np.uint32)
    siz = np.empty(cap, np.uint32)
    nt, ne = C.c_uint64(), C.c_uint64()
    ns = fn(text, len(text), tok.ctypes.data_as(U32P), cap, siz.ctypes.data_as(U32P), cap, C.byref(nt), C.byref(ne))
    return tok[:nt.value].copy(), siz[:ns].copy(), int(ne.value)


def verify_csr(coll, probes, offsets, cands, threshold, sim="jaccard", probe=None):
    """(pairs, tokens read) of explicit candidate lists, verified as
    hybrid::device_handler's kernels do: probes of `probe` (default: coll)
    against candidates of coll, each a (tokens, starts, sizes) triple."""
    lib = _load()
    fn = lib.oracle_verify_csr
    fn.restype = C.c_void_p
    fn.argtypes = [U32P] * 9 + [C.c_uint32, C.c_int, C.c_double, C.POINTER(C.c_uint64)]
    t, tp = _p(coll[0]); s_, sp = _p(coll[1]); z, zp = _p(coll[2])
    pc = probe if probe is not None else coll
    t2, tp2 = _p(pc[0]); s2, sp2 = _p(pc[1]); z2, zp2 = _p(pc[2])
    pr, prp = _p(probes); of, ofp = _p(offsets); ca, cap = _p(cands)
    read = C.c_uint64()
    out = _take(fn(tp, sp, zp, tp2, sp2, zp2, prp, ofp, cap, len(pr), SIM[sim], float(threshold), C.byref(read)))
    return out, int(read.value)

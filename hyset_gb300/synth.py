"""Seeded synthetic collections (wraps libhyset_synth.so, include/hyset_gb300_synth.h).

Workload presets follow the benchmark configurations of this project: Zipf
tokens drawn without replacement, tokens renumbered 1..U by ascending global
frequency, sets sorted, collection sorted by (size, tokens).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
SYNTH_PATH = os.path.join(_HERE, "libhyset_synth.so")

UNIFORM, LOGNORMAL = 0, 1


class _Params(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_sets", C.c_uint32), ("universe", C.c_uint32), ("zipf_s", C.c_double),
                ("size_dist", C.c_int), ("size_a", C.c_double), ("size_b", C.c_double), ("size_min", C.c_uint32),
                ("size_max", C.c_uint32), ("dup_frac", C.c_double), ("dup_edit_lo", C.c_double),
                ("dup_edit_hi", C.c_double), ("threads", C.c_int)]


@dataclass
class SynthSpec:
    n_sets: int
    universe: int
    zipf_s: float
    size_dist: int
    size_a: float
    size_b: float
    size_min: int
    size_max: int
    dup_frac: float = 0.0
    dup_edit_lo: float = 0.0
    dup_edit_hi: float = 0.0
    seed: int = 0x5E7


# The benchmark configurations (sizes, universes, Zipf exponents, planted duplicates).
C1 = SynthSpec(10_000, 5_000, 1.0, UNIFORM, 5, 50, 5, 50)
C2 = SynthSpec(200_000, 100_000, 1.1, LOGNORMAL, 3.2, 0.6, 2, 500, 0.03, 0.10, 0.10)
C3 = SynthSpec(1_000_000, 1_000_000, 0.9, LOGNORMAL, 4.4, 0.8, 10, 2000, 0.05, 0.05, 0.15)


@dataclass
class Collection:
    """CSR collection in the reference's input contract (sorted sets, size-sorted)."""
    tokens: np.ndarray  # uint32 [T]
    starts: np.ndarray  # uint32 [n]
    sizes: np.ndarray   # uint32 [n]

    @property
    def n(self) -> int:
        return int(self.sizes.shape[0])

    def set(self, i: int) -> np.ndarray:
        s = int(self.starts[i])
        return self.tokens[s:s + int(self.sizes[i])]

    def write_text(self, path: str) -> None:
        with open(path, "w") as f:
            for i in range(self.n):
                f.write(" ".join(map(str, self.set(i).tolist())) + "\n")


_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(SYNTH_PATH):
            raise RuntimeError(f"{SYNTH_PATH} missing: build with hyset_gb300._build")
        lib = C.CDLL(SYNTH_PATH)
        lib.hyset_synth_generate.argtypes = [C.POINTER(_Params), C.POINTER(C.c_void_p)]
        lib.hyset_synth_generate.restype = C.c_int
        for name, res in (("num_sets", C.c_uint32), ("num_tokens", C.c_uint64), ("max_token", C.c_uint32)):
            fn = getattr(lib, "hyset_synth_" + name)
            fn.argtypes = [C.c_void_p]
            fn.restype = res
        for name in ("tokens", "sizes", "starts"):
            fn = getattr(lib, "hyset_synth_" + name)
            fn.argtypes = [C.c_void_p]
            fn.restype = C.POINTER(C.c_uint32)
        lib.hyset_synth_free.argtypes = [C.c_void_p]
        lib.hyset_synth_free.restype = None
        U32 = C.POINTER(C.c_uint32)
        lib.hyset_format_text.argtypes = [U32, U32, U32, C.c_uint32, C.c_void_p, C.c_uint64]
        lib.hyset_format_text.restype = C.c_uint64
        _lib = lib
    return _lib


def format_text(tokens, starts, sizes, out=None) -> np.ndarray:
    """The reference's text format of a collection as a uint8 array (written
    into `out`, e.g. pinned memory, when it is large enough)."""
    lib = _load()
    U32 = C.POINTER(C.c_uint32)
    t = np.ascontiguousarray(tokens, np.uint32)
    st = np.ascontiguousarray(starts, np.uint32)
    sz = np.ascontiguousarray(sizes, np.uint32)
    args = (t.ctypes.data_as(U32), st.ctypes.data_as(U32), sz.ctypes.data_as(U32), sz.size)
    n = int(lib.hyset_format_text(*args, None, 0))
    buf = out[:n] if out is not None and out.size >= n else np.empty(n, np.uint8)
    lib.hyset_format_text(*args, buf.ctypes.data_as(C.c_void_p), n)
    return buf


def generate(spec: SynthSpec, threads: int = 0, **overrides) -> Collection:
    fields = dict(spec.__dict__)
    fields.update(overrides)
    lib = _load()
    p = _Params(int(fields["seed"]), int(fields["n_sets"]), int(fields["universe"]), float(fields["zipf_s"]),
                int(fields["size_dist"]), float(fields["size_a"]), float(fields["size_b"]), int(fields["size_min"]),
                int(fields["size_max"]), float(fields["dup_frac"]), float(fields["dup_edit_lo"]),
                float(fields["dup_edit_hi"]), int(threads))
    h = C.c_void_p()
    if lib.hyset_synth_generate(C.byref(p), C.byref(h)) != 0:
        raise ValueError(f"invalid synthetic spec {fields}")
    try:
        n = lib.hyset_synth_num_sets(h)
        T = lib.hyset_synth_num_tokens(h)
        tok = np.ctypeslib.as_array(lib.hyset_synth_tokens(h), (T,)).copy() if T else np.zeros(0, np.uint32)
        sz = np.ctypeslib.as_array(lib.hyset_synth_sizes(h), (n,)).copy()
        st = np.ctypeslib.as_array(lib.hyset_synth_starts(h), (n,)).copy()
    finally:
        lib.hyset_synth_free(h)
    return Collection(tok, st, sz)


def batch_workload(n_joins: int = 256, seed: int = 0x5E7B):
    """The batched workload: `n_joins` independent R-S joins of uneven sizes:
    |R|, |S| log-uniform in [1e3, 2e5], Zipf s in [0.7, 1.3], mean set size
    log-uniform in [8, 300], universe 5e4..5e5,
    threshold in [0.5, 0.95], similarity Jaccard / cosine / dice in turn.  R and
    S of a join are a random split of one generated collection, so near-duplicate
    sets fall on both sides.  Returns [((r_tokens, r_starts, r_sizes),
    (s_tokens, s_starts, s_sizes), {"threshold": t, "sim": name}), ...]."""
    import math
    rng = np.random.default_rng(seed)
    sims = ["jaccard", "cosine", "dice"]
    out = []
    for j in range(n_joins):
        nr = int(math.exp(rng.uniform(math.log(1e3), math.log(2e5))))
        ns = int(math.exp(rng.uniform(math.log(1e3), math.log(2e5))))
        mean = math.exp(rng.uniform(math.log(8), math.log(300)))
        c = generate(C2, n_sets=nr + ns, universe=int(rng.uniform(5e4, 5e5)),
                     zipf_s=float(rng.uniform(0.7, 1.3)), size_dist=LOGNORMAL,
                     size_a=math.log(mean) - 0.125, size_b=0.5, size_min=2,
                     size_max=min(2000, max(16, int(mean * 6))), dup_frac=0.05, dup_edit_lo=0.02,
                     dup_edit_hi=0.12, seed=int(rng.integers(1, 2**31)))
        side = rng.random(c.n) < nr / (nr + ns)
        parts = []
        for mask in (side, ~side):
            ids = np.nonzero(mask)[0]
            sizes = c.sizes[ids]
            starts = np.zeros(len(ids), np.uint32)
            if len(ids):
                starts[1:] = np.cumsum(sizes[:-1])
            sz64 = sizes.astype(np.int64)
            src = np.repeat(c.starts[ids].astype(np.int64) - starts.astype(np.int64), sz64) + np.arange(sz64.sum())
            parts.append((c.tokens[src], starts, sizes))
        out.append((parts[0], parts[1], dict(threshold=float(rng.uniform(0.5, 0.95)), sim=sims[j % 3])))
    return out

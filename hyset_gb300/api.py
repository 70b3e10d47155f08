"""Python host API over the C ABI: contexts, device collections, joins.

    ctx = Context()                      # one CUDA stream on one GB300
    coll = ctx.upload(tokens, sizes)     # device_collection (collection.hpp:54-71)
    res = ctx.self_join(coll, threshold=0.8)            # R join R
    res = ctx.rs_join(indexed, probe, threshold=0.8)    # R join S
    res.pairs  # (count, 2) uint32 (probe id, indexed id); res.count
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import (COST_TERMS, MLP_PARAMS, N_FEATURES, SELECTOR_NAMES, SIM, TECH, TECH_NAMES, JoinDesc, JoinOpts,
                   U32P, check, load)


@dataclass
class JoinResult:
    count: int
    pairs: Optional[np.ndarray]  # None when count_only or device_pairs
    technique: str
    device_ms: float
    kernel_ms: float = 0.0
    stats: Optional[list] = None
    device_pairs: int = 0  # device address when device_pairs was requested
    launches: int = 0      # kernel launches the join issued
    selector: str = "explicit"  # which selector chose the technique
    bitmap_bits: int = 0        # signature width the join ran with
    split_at: int = 0           # partition split: first probe id of the high range (0 = none)
    split_low: str = ""         # the low range's technique when split
    verify_mode: int = 0        # 1 lane per candidate, 2 warp per candidate, 3 staged (candidate lists)
    probe_batch: int = 0        # probes per warp batch of the probe-major prefix kernel (0: another kernel)


# R-S joins: which collection is indexed (hyset_join_opts.orientation)
ORIENTATION = {"auto": 0, "as_given": 1, "swapped": 2}


def make_opts(threshold: float = 0.8, sim: str = "jaccard", technique: str = "auto", bitmap: int = 0,
              count_only: bool = False, verify_mode: int = 0, sort_pairs: bool = False,
              pair_capacity: int = 0, device_pairs: bool = False, collect_stats: bool = False,
              probe_range=None, probe_major: bool = False, fgss_batch: int = 0,
              orientation: str = "auto") -> JoinOpts:
    if sim not in SIM:
        raise ValueError(f"unknown similarity {sim!r}")
    if technique not in TECH:
        raise ValueError(f"unknown technique {technique!r}")
    if orientation not in ORIENTATION:
        raise ValueError(f"unknown orientation {orientation!r}")
    return JoinOpts(SIM[sim], float(threshold), TECH[technique], int(bitmap), int(bool(count_only)),
                    int(verify_mode), int(bool(sort_pairs)), int(pair_capacity), int(bool(device_pairs)),
                    int(bool(collect_stats)), int(probe_range[0]) if probe_range else 0,
                    int(probe_range[1]) if probe_range else 0, int(bool(probe_major)), int(fgss_batch),
                    ORIENTATION[orientation])


def _split(lib, r):
    low = C.c_int(0)
    at = int(lib.hyset_result_split(r, C.byref(low)))
    return at, (TECH_NAMES.get(low.value, "?") if at else "")


def _take_result(lib, r) -> JoinResult:
    try:
        n = lib.hyset_result_count(r)
        ptr = lib.hyset_result_pairs(r)
        pairs = None
        if ptr:
            pairs = (np.ctypeslib.as_array(C.cast(ptr, U32P), (2 * n,)).reshape(n, 2).copy() if n
                     else np.zeros((0, 2), np.uint32))
        st = (C.c_uint64 * 8)()
        k = lib.hyset_result_stats(r, st, 8)
        return JoinResult(int(n), pairs, TECH_NAMES.get(lib.hyset_result_technique(r), "?"),
                          float(lib.hyset_result_device_ms(r)), float(lib.hyset_result_kernel_ms(r)),
                          [int(st[i]) for i in range(k)], int(lib.hyset_result_device_pairs(r) or 0),
                          int(lib.hyset_result_launches(r)), SELECTOR_NAMES.get(lib.hyset_result_selector(r), "?"),
                          int(lib.hyset_result_bitmap_bits(r)), *_split(lib, r),
                          int(lib.hyset_result_verify_mode(r)), int(lib.hyset_result_probe_batch(r)))
    finally:
        lib.hyset_result_free(r)


class DeviceCollection:
    """A size-sorted collection resident in HBM (the reference's device_collection)."""

    def __init__(self, ctx: "Context", handle: C.c_void_p, n: int, keep=None):
        self._ctx = ctx
        self.handle = handle
        self.n = n
        self._keep = keep  # host/device arrays that must outlive the handle

    def free(self):
        if self.handle:
            load().hyset_collection_free(self._ctx.handle, self.handle)
            self.handle = None

    @property
    def num_tokens(self) -> int:
        return int(load().hyset_collection_num_tokens(self.handle))

    def download(self):
        """(tokens, starts, sizes) copied to host numpy arrays."""
        lib = load()
        tok = np.empty(self.num_tokens, np.uint32)
        st = np.empty(self.n, np.uint32)
        sz = np.empty(self.n, np.uint32)
        check(lib.hyset_collection_download(self._ctx.handle, self.handle, tok.ctypes.data_as(U32P),
                                            st.ctypes.data_as(U32P), sz.ctypes.data_as(U32P)), self._ctx.handle)
        return tok, st, sz

    def __del__(self):
        try:
            if self._ctx.handle:
                self.free()
        except Exception:
            pass


def _fptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Context:
    def __init__(self, device: int = 0, selector: bool = True, width: bool = True):
        """selector: install the shipped technique selector (learned network
        and analytic cost model) for technique AUTO, if it is present.
        width: install the shipped signature-width network, if present."""
        self._lib = load()
        h = C.c_void_p()
        check(self._lib.hyset_create(device, C.byref(h)))
        self.handle = h
        self.selector_info = None
        self.width_info = None
        if selector or width:
            from . import selector as _sel
            from . import width_selector as _wsel
            try:
                if selector:
                    self.selector_info = _sel.install_shipped(self)
                if width:
                    self.width_info = _wsel.install_shipped(self)
            except Exception:
                self.close()
                raise

    def close(self):
        if self.handle:
            self._lib.hyset_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self) -> str:
        return self._lib.hyset_last_error(self.handle).decode()

    # ---- collections
    def upload(self, tokens, sizes, starts=None) -> DeviceCollection:
        tok = np.ascontiguousarray(tokens, dtype=np.uint32)
        sz = np.ascontiguousarray(sizes, dtype=np.uint32)
        st = None if starts is None else np.ascontiguousarray(starts, dtype=np.uint32)
        h = C.c_void_p()
        check(self._lib.hyset_collection_upload(
            self.handle, tok.ctypes.data_as(U32P), tok.size, None if st is None else st.ctypes.data_as(U32P),
            sz.ctypes.data_as(U32P), sz.size, C.byref(h)), self.handle)
        return DeviceCollection(self, h, int(sz.size))

    def parse(self, text) -> DeviceCollection:
        """Parses the reference's text format on the GPU (read_collection,
        include/hyset/collection.hpp:93-177).  text: bytes, a path, or an
        object exposing a device pointer (int address, n_bytes) pair."""
        if isinstance(text, tuple):
            ptr, n = int(text[0]), int(text[1])
            keep = None
        else:
            if isinstance(text, str):
                with open(text, "rb") as f:
                    text = f.read()
            buf = np.frombuffer(text, dtype=np.uint8)
            ptr, n, keep = buf.ctypes.data, buf.size, buf
        h = C.c_void_p()
        check(self._lib.hyset_collection_parse(self.handle, C.c_void_p(ptr), n, C.byref(h)), self.handle)
        del keep
        return DeviceCollection(self, h, int(self._lib.hyset_collection_num_sets(h)))

    def from_device(self, d_tokens: int, n_tokens: int, d_starts: int, d_sizes: int, n_sets: int,
                    keep=None) -> DeviceCollection:
        """Wraps CSR arrays already in device memory (raw device pointers)."""
        h = C.c_void_p()
        check(self._lib.hyset_collection_from_device(self.handle, C.c_void_p(d_tokens), n_tokens,
                                                     C.c_void_p(d_starts), C.c_void_p(d_sizes), n_sets,
                                                     C.byref(h)), self.handle)
        return DeviceCollection(self, h, n_sets, keep)

    # ---- joins
    def self_join(self, coll: DeviceCollection, threshold: float = 0.8, **kw) -> JoinResult:
        o = make_opts(threshold, **kw)
        r = C.c_void_p()
        check(self._lib.hyset_self_join(self.handle, coll.handle, C.byref(o), C.byref(r)), self.handle)
        return _take_result(self._lib, r)

    def self_join_host(self, tokens, sizes, starts=None, threshold: float = 0.8, keep_collection: bool = False,
                       **kw):
        """Upload and self-join in one call from host arrays (hyset_self_join_host):
        the copy overlaps the checks and the index build.  Returns the result, or
        (result, DeviceCollection) with keep_collection."""
        tok = np.ascontiguousarray(tokens, dtype=np.uint32)
        sz = np.ascontiguousarray(sizes, dtype=np.uint32)
        st = None if starts is None else np.ascontiguousarray(starts, dtype=np.uint32)
        o = make_opts(threshold, **kw)
        r = C.c_void_p()
        h = C.c_void_p()
        check(self._lib.hyset_self_join_host(
            self.handle, tok.ctypes.data_as(U32P), tok.size, None if st is None else st.ctypes.data_as(U32P),
            sz.ctypes.data_as(U32P), sz.size, C.byref(o), C.byref(h) if keep_collection else None, C.byref(r)),
            self.handle)
        res = _take_result(self._lib, r)
        if keep_collection:
            return res, DeviceCollection(self, h, int(sz.size))
        return res

    def verify_device(self, indexed: DeviceCollection, d_probes: int, d_offsets: int, d_candidates: int,
                      n_probes: int, probe: Optional[DeviceCollection] = None, threshold: float = 0.8,
                      **kw) -> JoinResult:
        """Verifies device-resident candidate lists (raw device pointers to uint32
        arrays: probe ids, inclusive end offsets, candidate ids)."""
        o = make_opts(threshold, **kw)
        r = C.c_void_p()
        check(self._lib.hyset_verify_device(self.handle, indexed.handle, probe.handle if probe else None,
                                            C.c_void_p(d_probes), C.c_void_p(d_offsets), C.c_void_p(d_candidates),
                                            n_probes, C.byref(o), C.byref(r)), self.handle)
        return _take_result(self._lib, r)

    def rs_join(self, indexed: DeviceCollection, probe: DeviceCollection, threshold: float = 0.8,
                **kw) -> JoinResult:
        o = make_opts(threshold, **kw)
        r = C.c_void_p()
        check(self._lib.hyset_rs_join(self.handle, indexed.handle, probe.handle, C.byref(o), C.byref(r)),
              self.handle)
        return _take_result(self._lib, r)

    # ---- selector
    def features(self, indexed: DeviceCollection, probe: Optional[DeviceCollection] = None, **kw):
        """(features[12], base_stats[8]) of a join, computed on the GPU."""
        o = make_opts(**kw)
        f = np.zeros(N_FEATURES, np.float32)
        b = np.zeros(8, np.float64)
        check(self._lib.hyset_join_features(self.handle, indexed.handle, probe.handle if probe else None,
                                            C.byref(o), f.ctypes.data_as(C.POINTER(C.c_float)),
                                            b.ctypes.data_as(C.POINTER(C.c_double))), self.handle)
        return f, b

    def mlp_forward(self, params: np.ndarray, x: np.ndarray) -> np.ndarray:
        params = np.ascontiguousarray(params, np.float32)
        x = np.ascontiguousarray(x, np.float32).reshape(-1, N_FEATURES)
        y = np.zeros((x.shape[0], 3), np.float32)
        check(self._lib.hyset_mlp_forward(self.handle, _fptr(params), _fptr(x), x.shape[0], _fptr(y)), self.handle)
        return y

    def mlp_grad(self, params, x, t, mask):
        params = np.ascontiguousarray(params, np.float32)
        x = np.ascontiguousarray(x, np.float32).reshape(-1, N_FEATURES)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, 3)
        mask = np.ascontiguousarray(mask, np.float32).reshape(-1, 3)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        check(self._lib.hyset_mlp_grad(self.handle, _fptr(params), _fptr(x), _fptr(t), _fptr(mask), x.shape[0],
                                       _fptr(g), _fptr(loss)), self.handle)
        return g, float(loss[0])

    def mlp_train(self, params, x, t, mask, steps, lr=1e-3, weight_decay=0.0):
        p = np.array(params, dtype=np.float32, copy=True)
        x = np.ascontiguousarray(x, np.float32).reshape(-1, N_FEATURES)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, 3)
        mask = np.ascontiguousarray(mask, np.float32).reshape(-1, 3)
        trace = np.zeros(max(int(steps), 1), np.float32)
        check(self._lib.hyset_mlp_train(self.handle, _fptr(p), _fptr(x), _fptr(t), _fptr(mask), x.shape[0],
                                        int(steps), float(lr), float(weight_decay), _fptr(trace)), self.handle)
        return p, trace[:int(steps)]

    def selector_set(self, params=None, mean=None, scale=None, cost=None):
        args = []
        keep = []
        for a, dt in ((params, np.float32), (mean, np.float32), (scale, np.float32), (cost, np.float64)):
            if a is None:
                args.append(None)
            else:
                arr = np.ascontiguousarray(a, dt)
                keep.append(arr)
                args.append(_fptr(arr))
        check(self._lib.hyset_selector_set(self.handle, *args), self.handle)

    def width_selector_set(self, params=None, mean=None, scale=None):
        """Installs (or with params None removes) the signature-width network."""
        if params is None:
            check(self._lib.hyset_width_selector_set(self.handle, None, None, None), self.handle)
            return
        arrs = [np.ascontiguousarray(a, np.float32) for a in (params, mean, scale)]
        check(self._lib.hyset_width_selector_set(self.handle, *[_fptr(a) for a in arrs]), self.handle)

    def batch_join(self, joins: Sequence[tuple]) -> list:
        """joins: (indexed, probe_or_None, opts_kwargs) triples."""
        n = len(joins)
        descs = (JoinDesc * max(n, 1))()
        for i, (R, S, kw) in enumerate(joins):
            descs[i].indexed = R.handle
            descs[i].probe = S.handle if S is not None else None
            descs[i].opts = make_opts(**kw)
        res = (C.c_void_p * max(n, 1))()
        check(self._lib.hyset_batch_join(self.handle, descs, n, res), self.handle)
        return [_take_result(self._lib, C.c_void_p(res[i])) for i in range(n)]


def sorted_pairs(pairs: np.ndarray) -> np.ndarray:
    p = np.asarray(pairs, dtype=np.uint32).reshape(-1, 2)
    if p.shape[0] == 0:
        return p
    key = (p[:, 0].astype(np.uint64) << np.uint64(32)) | p[:, 1].astype(np.uint64)
    return p[np.argsort(key, kind="stable")]

"""The C-ABI library loads and exports every declared symbol (CPU only, no compute)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "hyset_gb300.h")


def declared_functions(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hyset_[a-z_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions(HEADER)
    for must in ("hyset_create", "hyset_collection_upload", "hyset_self_join", "hyset_rs_join", "hyset_batch_join",
                 "hyset_handler_create", "hyset_handler_join_blocks", "hyset_verifier_create"):
        assert must in names


def test_library_exports_every_declared_symbol():
    import hyset_gb300._lib as L
    assert os.path.exists(L.LIB_PATH), "build first: python -c 'import __graft_entry__ as g; g.build()'"
    lib = ctypes.CDLL(L.LIB_PATH)
    missing = [n for n in declared_functions(HEADER) if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes prototypes cover exactly the header
    assert sorted(L.PROTOTYPES) == declared_functions(HEADER)


def test_create_reports_no_device_without_gpu():
    import hyset_gb300._lib as L
    lib = L.load()
    h = ctypes.c_void_p()
    st = lib.hyset_create(0, ctypes.byref(h))
    if st == 0:  # a GPU is present (this suite also runs on the GPU machine)
        lib.hyset_destroy(h)
    else:
        assert st == 7  # HYSET_E_NODEVICE: no silent CPU fallback


def test_synth_header_and_library_agree():
    from hyset_gb300 import synth
    names = declared_functions(os.path.join(ROOT, "include", "hyset_gb300_synth.h"))
    lib = ctypes.CDLL(synth.SYNTH_PATH)
    assert all(hasattr(lib, n) for n in names)


def test_struct_layouts_match_header():
    import hyset_gb300._lib as L
    assert ctypes.sizeof(L.Block) == 32
    assert ctypes.sizeof(L.JoinOpts) == 80

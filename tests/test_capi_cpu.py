"""CPU checks of the drop-in boundary: libbsfh.so builds for sm_103a, loads without a GPU
and exports every entry point include/bsfh.h declares; host-only helpers behave."""
import ctypes as C
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "bsfh.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(built_lib)
    names = header_functions()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(built_lib):
    from bs45_quantum_explorer_gb300._lib import SIGNATURES
    assert set(header_functions()) <= set(SIGNATURES)


def test_strerror_and_pack_without_gpu(built_lib):
    from bs45_quantum_explorer_gb300._lib import lib
    assert lib().bs_strerror(-4) == b"device wait limit reached"
    assert lib().bs_version() >= 100
    seq = np.array([[1, -1, 1, 1], [-1, -1, -1, 1]], np.int8)
    words = np.zeros(2, np.uint64)
    assert lib().bs_pack_rows(seq.ctypes.data, 2, 4, words.ctypes.data) == 0
    assert list(words) == [0b1101, 0b1000]
    bad = np.array([[1, 0, 1, 1]], np.int8)
    assert lib().bs_pack_rows(bad.ctypes.data, 1, 4, words.ctypes.data) == -1


def test_context_refuses_without_device(built_lib):
    import torch
    if torch.cuda.is_available():
        return
    from bs45_quantum_explorer_gb300._lib import lib
    h = C.c_void_p()
    rc = lib().bs_ctx_create(42, 7, 11, 0, 0, 0, C.byref(h))
    assert rc == -7  # BS_ERR_NODEV: fails loudly, no CPU fallback
    rc = lib().bs_ctx_create(42, 7, 11, 0, 1, 0, C.byref(h))
    assert rc in (-1, -7)


def test_pack_roundtrip():
    from bs45_quantum_explorer_gb300.hall import pack, unpack
    rng = np.random.default_rng(3)
    x = rng.choice(np.array([-1, 1], np.int8), size=(100, 2, 42))
    assert (unpack(pack(x), 42) == x).all()

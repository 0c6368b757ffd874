"""The C-ABI library builds, loads and exports every symbol the header
declares; argument validation answers without touching a GPU."""
import ctypes
import os
import re

import pytest

from exptool_gb300 import _lib
from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "exptool_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xt_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert declared_symbols() == sorted(_lib.EXPORTED)


def test_library_exports_every_symbol():
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.xt_abi_version() == 1


def test_argument_errors_without_gpu():
    lib = _lib.load()
    h = ctypes.c_void_p()
    import numpy as np
    a = np.zeros(10)
    p = a.ctypes.data
    rc = lib.xt_sph_table_create(40, 4, 10, 2, 1e-3, 1.0, 1.0, p, p, p, p, p, ctypes.byref(h))
    assert rc == -1 and b"lmax" in lib.xt_last_error()
    rc = lib.xt_sph_table_create(2, 4, 2, 2, 1e-3, 1.0, 1.0, p, p, p, p, p, ctypes.byref(h))
    assert rc == -1 and b"numr" in lib.xt_last_error()
    rc = lib.xt_cyl_table_create(2, 3, 4, 4, 5, 0, 0., 1., 0., 1., 1., 1., p, None, None, None, p, None, None, None,
                                 ctypes.byref(h))
    assert rc == -1 and b"cmap" in lib.xt_last_error()
    rc = lib.xt_sph_accumulate(None, None, None, None, None, 0, 0, 0, None, None, 0, None)
    assert rc == -1
    assert lib.xt_sph_accumulate_workspace(None) == 0
    assert lib.xt_cyl_field_bytes(None, 0, 0) == 0


def test_copy_list_arguments_without_gpu():
    """xt_copy_async checks its copy list before any CUDA call: an empty list
    and zero-byte entries are no-ops, missing arrays and null addresses are
    argument errors."""
    lib = _lib.load()
    assert lib.xt_copy_async(0, None, None, None, None) == 0
    assert lib.xt_copy_async(-1, None, None, None, None) == -1
    assert lib.xt_copy_async(2, None, None, None, None) == -1
    assert b"NULL copy list" in lib.xt_last_error()
    dst = (ctypes.c_void_p * 2)(None, None)
    src = (ctypes.c_void_p * 2)(None, None)
    nb = (ctypes.c_size_t * 2)(0, 0)
    assert lib.xt_copy_async(2, dst, src, nb, None) == 0          # zero bytes: skipped
    nb[1] = 8
    assert lib.xt_copy_async(2, dst, src, nb, None) == -1
    assert b"copy 1" in lib.xt_last_error()

"""The C ABI: libgwgb.so loads, exports every symbol include/gwgb.h declares,
and rejects bad layouts/parameters before touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from _helpers import crystal
from mbsymmetry_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "gwgb.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gwgb_[A-Za-z0-9_]+)\s*\(", txt)))


def test_header_and_binding_agree():
    assert set(_declared()) == set(_abi.SIGNATURES)


def test_library_exports_every_symbol():
    lib = _abi.load()
    for name in _declared():
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.gwgb_version()


def _params(nts=62, ns=1):
    return _abi.GwgbParams(ns=ns, nts=nts, nw=nts - 2, nw_b=nts - 3, beta=50.0, precision=0, device=0,
                           nt_batch=0, flags=0)


def _create(params, layout_c):
    lib = _abi.load()
    h = ctypes.c_void_p()
    rc = lib.gwgb_create(ctypes.byref(params), ctypes.byref(layout_c), ctypes.byref(h))
    return rc, h


def test_rejects_odd_tau_count():
    cr, _ = crystal("C1")
    L, keep = cr.layout.to_c()
    rc, h = _create(_params(nts=61), L)
    assert rc == _abi.GWGB_E_INVALID
    assert b"even" in _abi.load().gwgb_last_error()


def test_rejects_bad_block_and_index_data():
    cr, _ = crystal("C1")
    lay = cr.layout
    L, keep = lay.to_c()
    # corrupt one tensor_irreps entry (points at a non-existent aux block)
    ti = np.ctypeslib.as_array(ctypes.cast(L.tensor_irreps, ctypes.POINTER(ctypes.c_int32)), shape=(3,))
    saved = ti[0]
    ti[0] = 999
    rc, h = _create(_params(), L)
    ti[0] = saved
    assert rc == _abi.GWGB_E_INVALID
    # a zero-sized block
    ao = np.ctypeslib.as_array(ctypes.cast(L.ao_sizes, ctypes.POINTER(ctypes.c_int32)), shape=(1,))
    saved = ao[0]
    ao[0] = 0
    rc, h = _create(_params(), L)
    ao[0] = saved
    assert rc == _abi.GWGB_E_UNSUPPORTED
    # irre_index out of range
    ii = np.ctypeslib.as_array(ctypes.cast(L.irre_index, ctypes.POINTER(ctypes.c_int32)), shape=(1,))
    saved = ii[0]
    ii[0] = 77
    rc, h = _create(_params(), L)
    ii[0] = saved
    assert rc == _abi.GWGB_E_INVALID


def test_null_arguments():
    lib = _abi.load()
    assert lib.gwgb_create(None, None, None) == _abi.GWGB_E_INVALID
    assert lib.gwgb_solve(None) == _abi.GWGB_E_INVALID
    assert lib.gwgb_destroy(None) == _abi.GWGB_OK

"""gwgb_create rejects bad tile-shape settings before touching the device
(host logic; runs without a GPU)."""
import ctypes

import pytest

from mbsymmetry_gb300 import _abi


@pytest.mark.parametrize("field,value", [("uvt_smem_kb", 10), ("uvt_smem_kb", 300), ("sw_npk_max", 48),
                                         ("uv_waves", 17), ("uv_waves", -1),
                                         ("oz_simt_cols", -2), ("oz_simt_cols", 2000)])
def test_bad_tune_settings_are_rejected(field, value):
    lib = _abi.load()
    p = _abi.GwgbParams(ns=1, nts=62, nw=60, nw_b=60, beta=50.0, precision=_abi.PREC_FP64, device=0,
                        nt_batch=0, flags=0)
    setattr(p, field, value)
    lay = _abi.GwgbLayout()
    h = ctypes.c_void_p()
    rc = lib.gwgb_create(ctypes.byref(p), ctypes.byref(lay), ctypes.byref(h))
    assert rc == _abi.GWGB_E_INVALID
    assert field.encode() in lib.gwgb_last_error()
    assert not h.value

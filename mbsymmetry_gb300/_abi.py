"""ctypes mirror of ``include/gwgb.h`` and the loader of ``libgwgb.so``.

The engine is the in-tree CUDA library ``mbsymmetry_gb300/csrc/libgwgb.so``
built by ``__graft_entry__.build()``; there is no other implementation behind
this module.  :func:`load` raises when the library is missing.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int32, c_int64, c_void_p

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "csrc", "libgwgb.so")

GWGB_OK = 0
GWGB_E_INVALID = 1
GWGB_E_NOMEM = 2
GWGB_E_CUDA = 3
GWGB_E_TIMEOUT = 4
GWGB_E_NUMERIC = 5
GWGB_E_STATE = 6
GWGB_E_UNSUPPORTED = 7

PREC_FP64 = 0
PREC_TF32X3 = 1
PREC_BF16X3 = 2
PREC_OZAKI = 3

PREC_NAMES = {"fp64": PREC_FP64, "tf32x3": PREC_TF32X3, "bf16x3": PREC_BF16X3, "ozaki": PREC_OZAKI}


class GwgbParams(ctypes.Structure):
    _fields_ = [
        ("ns", c_int32), ("nts", c_int32), ("nw", c_int32), ("nw_b", c_int32),
        ("beta", c_double), ("precision", c_int32), ("device", c_int32),
        ("nt_batch", c_int32), ("flags", c_int32),
        ("uvt_smem_kb", c_int32), ("sw_npk_max", c_int32), ("uv_waves", c_int32), ("uv_simt", c_int32),
        ("oz_simt_cols", c_int32),
    ]


class GwgbLayout(ctypes.Structure):
    _fields_ = [
        ("nk", c_int32), ("ink", c_int32),
        ("irre_list", c_void_p), ("index", c_void_p), ("irre_index", c_void_p),
        ("conj_index", c_void_p), ("q_ind", c_void_p), ("q_ind2", c_void_p),
        ("ao_block_ptr", c_void_p), ("ao_sizes", c_void_p),
        ("aux_block_ptr", c_void_p), ("aux_sizes", c_void_p),
        ("kpair_block_ptr", c_void_p), ("tensor_irreps", c_void_p),
        ("orep_block_ptr", c_void_p), ("orep_irreps", c_void_p),
        ("auxrep_block_ptr", c_void_p), ("auxrep_irreps", c_void_p),
    ]


class GwgbStats(ctypes.Structure):
    _fields_ = [
        ("rotate_G_ms", c_double), ("p0_ms", c_double), ("pq_ms", c_double),
        ("rotate_P_ms", c_double), ("sigma_ms", c_double), ("dyson_ms", c_double),
        ("total_ms", c_double), ("p0_flops", c_double), ("sigma_flops", c_double),
        ("leakage", c_double), ("kernel_launches", c_int64),
        ("device_bytes", c_int64), ("transform_ms", c_double), ("transform_bytes", c_double),
        ("solve_ms", c_double), ("solve_flops", c_double), ("transform_flops", c_double),
    ]


class GwgbLaunchStat(ctypes.Structure):
    _fields_ = [
        ("stage", c_int32), ("kernel", c_int32), ("tasks", c_int32), ("ran", c_int32),
        ("ms", c_double), ("flops", c_double), ("mma_flops", c_double), ("bytes", c_double),
    ]


LAUNCH_STAGES = ("Z1", "Z", "P0", "W", "U", "Sigma")
LAUNCH_KERNELS = ("oz_gemm_kernel", "oz_simt_kernel", "reduce_slices_kernel", "oz_perm_kernel")


class GwgbProxyStats(ctypes.Structure):
    _fields_ = [("p0_ms", c_double), ("sigma_ms", c_double), ("gemm_calls", c_int64), ("other_calls", c_int64)]


class GwgbMuSearch(ctypes.Structure):
    _fields_ = [
        ("n_electrons", c_double), ("mu0", c_double), ("step", c_double), ("tol", c_double),
        ("max_evals", c_int32), ("pad", c_int32),
    ]


class GwgbScRecord(ctypes.Structure):
    _fields_ = [
        ("mu", c_double), ("n_electrons", c_double), ("e_corr", c_double), ("e_one", c_double),
        ("leakage", c_double), ("mu_evals", c_int32), ("precision", c_int32),
    ]


#: every symbol include/gwgb.h declares, with (restype, argtypes)
SIGNATURES = {
    "gwgb_version": (c_char_p, []),
    "gwgb_last_error": (c_char_p, []),
    "gwgb_create": (c_int32, [POINTER(GwgbParams), POINTER(GwgbLayout), POINTER(c_void_p)]),
    "gwgb_destroy": (c_int32, [c_void_p]),
    "gwgb_set_precision": (c_int32, [c_void_p, c_int32]),
    "gwgb_upload_V": (c_int32, [c_void_p, c_void_p, c_int64]),
    "gwgb_set_reps": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_int64]),
    "gwgb_set_transforms": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p]),
    "gwgb_set_fock": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "gwgb_set_G": (c_int32, [c_void_p, c_void_p]),
    "gwgb_get_G": (c_int32, [c_void_p, c_void_p]),
    "gwgb_set_sigma": (c_int32, [c_void_p, c_void_p]),
    "gwgb_get_sigma": (c_int32, [c_void_p, c_void_p]),
    "gwgb_set_P0": (c_int32, [c_void_p, c_void_p]),
    "gwgb_get_P0": (c_int32, [c_void_p, c_void_p]),
    "gwgb_solve_P0": (c_int32, [c_void_p]),
    "gwgb_solve_Pq": (c_int32, [c_void_p]),
    "gwgb_solve_sigma": (c_int32, [c_void_p]),
    "gwgb_solve_sigma_from_P": (c_int32, [c_void_p]),
    "gwgb_hf_hartree": (c_int32, [c_void_p, c_void_p]),
    "gwgb_solve": (c_int32, [c_void_p]),
    "gwgb_dyson": (c_int32, [c_void_p, c_double]),
    "gwgb_iteration": (c_int32, [c_void_p, c_double]),
    "gwgb_get_stats": (c_int32, [c_void_p, POINTER(GwgbStats)]),
    "gwgb_set_launch_timing": (c_int32, [c_void_p, c_int32]),
    "gwgb_get_launch_stats": (c_int32, [c_void_p, POINTER(GwgbLaunchStat), c_int32, POINTER(c_int32)]),
    "gwgb_synchronize": (c_int32, [c_void_p]),
    "gwgb_refproxy_run": (c_int32, [c_void_p, c_int32, c_int32, POINTER(GwgbProxyStats)]),
    "gwgb_refproxy_get": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "gwgb_set_hcore": (c_int32, [c_void_p, c_void_p]),
    "gwgb_set_energy_matrix": (c_int32, [c_void_p, c_void_p, c_int32]),
    "gwgb_find_mu": (c_int32, [c_void_p, POINTER(GwgbMuSearch), POINTER(c_double), POINTER(c_double)]),
    "gwgb_energy": (c_int32, [c_void_p, POINTER(c_double), POINTER(c_double)]),
    "gwgb_sc_loop": (c_int32, [c_void_p, c_int32, c_double, POINTER(GwgbMuSearch), c_int32,
                               POINTER(GwgbScRecord)]),
    "gwgb_test_raise_status": (c_int32, [c_void_p, c_int32]),
    "gwgb_test_wait_timeout": (c_int32, [c_int32, c_int32]),
    "gwgb_wsolve_noalloc": (c_int32, [c_int32, c_void_p, c_void_p, c_void_p, c_void_p, c_int32, c_int32,
                                      c_void_p, c_int32, c_void_p]),
}

NOALLOC_SCRATCH_BYTES = 8 << 20
NOALLOC_MAX_BLOCKS = 64

_lib = None


class GwgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gwgb error {code}: {msg}")
        self.code = code


def load(path: str = LIB_PATH):
    """Load libgwgb.so once; raise if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} not found: the CUDA engine is not built "
            "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int):
    if code != GWGB_OK:
        msg = _lib.gwgb_last_error().decode() if _lib is not None else "?"
        raise GwgbError(code, msg)

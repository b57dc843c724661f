"""gwgb_wsolve_noalloc: the W~ solve for callers that cannot allocate device
memory while they run (a host code whose own pool owns HBM, a plugin called
where new allocations are forbidden).  The entry point keeps its work space in
a static device array and takes only caller-owned inputs and outputs; here it
is checked against the handle-based entry point gwgb_solve_Pq and against the
FP64 oracle's P~ on the same P0, on two calls in a row, on aux blocks above 16
(the CTA-per-block inverse) with a work space close to the array's size, and
its size limits are checked.

This file is named to be collected last."""
import ctypes
import os
import sys

import numpy as np
import pytest

from _helpers import crystal
from mbsymmetry_gb300 import _abi

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))

pytestmark = pytest.mark.gpu


def _mirrored_p0_and_reference(cr, tr):
    """P0 of the GPU drop-in (mirrored to all nts rows) and P~ from gwgb_solve_Pq."""
    from mbsymmetry_gb300.solver import GWSolver
    L, nts = cr.layout, tr.nts
    s = GWSolver(L, cr.ns, tr)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    s.dyson(cr.mu)
    s.solve_P0()
    P0 = s.P0_q_t_QP()
    for iq in range(L.ink):          # mirror t -> nts-1-t (all nts rows filled)
        o, sz = L.qaux_slice_offsets_irre[iq], L.qaux_slice_sizes_irre[iq]
        blk = P0[nts * o: nts * (o + sz)].reshape(nts, sz)
        blk[nts // 2:] = blk[:nts // 2][::-1]
    s.set_P0(P0)
    s.compute_Pq_from_P0q()          # the existing entry point
    P_ref = s.P0_q_t_QP()
    s.close()
    return P0, P_ref


def _oracle_p_tilde(cr, tr, P0):
    from oracle import Oracle  # the checker
    return Oracle(cr.layout, cr.ns, tr.nts).p_tilde(P0, tr)


def _call(lib, P0, L, tr, iq, dev):
    import torch
    nts = tr.nts
    q = L.irre_list[iq]
    o, sz = L.qaux_slice_offsets_irre[iq], L.qaux_slice_sizes_irre[iq]
    tnt = torch.from_numpy(tr.Tnt_BF.view(np.float64)).to(dev)
    ttn = torch.from_numpy(tr.Ttn_FB.view(np.float64)).to(dev)
    src = torch.from_numpy(P0[nts * o: nts * (o + sz)].view(np.float64).copy()).to(dev)
    out = torch.zeros_like(src)
    sizes = np.ascontiguousarray(L.aux_sizes[q], dtype=np.int32)
    torch.cuda.synchronize()
    rc = lib.gwgb_wsolve_noalloc(dev.index, ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                 ctypes.c_void_p(tnt.data_ptr()), ctypes.c_void_p(ttn.data_ptr()),
                                 nts, tr.nw_b, sizes.ctypes.data, len(sizes), None)
    _abi.check(rc)
    return out.cpu().numpy().view(np.complex128), slice(nts * o, nts * (o + sz))


def test_noalloc_wsolve_matches_solve_pq_and_oracle_twice():
    import torch
    cr, tr = crystal("C1")
    L = cr.layout
    P0, P_ref = _mirrored_p0_and_reference(cr, tr)
    P_orc = _oracle_p_tilde(cr, tr, P0)
    lib = _abi.load()
    for iq in (0, 1):                # two calls in a row on the shared scratch array
        got, sl = _call(lib, P0, L, tr, iq, torch.device("cuda:0"))
        assert np.abs(got - P_ref[sl]).max() < 1e-12, iq
        assert np.abs(got - P_orc[sl]).max() < 1e-10, iq


def test_noalloc_wsolve_large_blocks_near_the_scratch_limit():
    """C2 slices: aux blocks up to 40 (the CTA-per-block inverse, n > 16); the
    largest slice fills most of the 8 MiB array."""
    import torch
    cr, tr = crystal("C2")
    L = cr.layout
    P0, P_ref = _mirrored_p0_and_reference(cr, tr)
    P_orc = _oracle_p_tilde(cr, tr, P0)
    lib = _abi.load()
    need = [tr.nw_b * L.qaux_slice_sizes_irre[iq] * 16 for iq in range(L.ink)]
    big = max(range(L.ink), key=lambda i: need[i])
    assert need[big] > 0.5 * _abi.NOALLOC_SCRATCH_BYTES
    assert max(L.aux_sizes[L.irre_list[big]]) > 16
    for iq in (big, 0):
        got, sl = _call(lib, P0, L, tr, iq, torch.device("cuda:0"))
        assert np.abs(got - P_ref[sl]).max() < 1e-12, iq
        assert np.abs(got - P_orc[sl]).max() < 1e-10, iq


def test_noalloc_rejects_sizes_beyond_the_limit():
    lib = _abi.load()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size checks come first
    too_many = np.ones(_abi.NOALLOC_MAX_BLOCKS + 1, dtype=np.int32)
    rc = lib.gwgb_wsolve_noalloc(0, dummy, dummy, dummy, dummy, 62, 59, too_many.ctypes.data, len(too_many), None)
    assert rc == _abi.GWGB_E_UNSUPPORTED
    big = np.full(_abi.NOALLOC_MAX_BLOCKS, 64, dtype=np.int32)  # 59 * 64 * 64 * 64 * 16 B >> 8 MiB
    rc = lib.gwgb_wsolve_noalloc(0, dummy, dummy, dummy, dummy, 62, 59, big.ctypes.data, len(big), None)
    assert rc == _abi.GWGB_E_UNSUPPORTED
    assert b"scratch" in lib.gwgb_last_error()

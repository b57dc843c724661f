"""gwgb_wsolve_noalloc: the W~ solve for callers that cannot allocate device
memory while they run (a host code whose own pool owns HBM, a plugin called
where new allocations are forbidden).  The entry point keeps its work space in
a static device array and takes only caller-owned inputs and outputs; here it
is checked against the handle-based entry point gwgb_solve_Pq on the same P0,
on two calls in a row, and its size limits are checked.

This file is named to be collected last."""
import ctypes

import numpy as np
import pytest

from _helpers import crystal
from mbsymmetry_gb300 import _abi

pytestmark = pytest.mark.gpu


def _mirrored_p0_and_reference(cr, tr):
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


def test_noalloc_wsolve_matches_solve_pq_twice():
    import torch
    cr, tr = crystal("C1")
    L, nts = cr.layout, tr.nts
    P0, P_ref = _mirrored_p0_and_reference(cr, tr)
    lib = _abi.load()
    dev = torch.device("cuda:0")
    tnt = torch.from_numpy(tr.Tnt_BF.view(np.float64)).to(dev)
    ttn = torch.from_numpy(tr.Ttn_FB.view(np.float64)).to(dev)
    for iq in (0, 1):                # two calls in a row on the shared scratch array
        q = L.irre_list[iq]
        o, sz = L.qaux_slice_offsets_irre[iq], L.qaux_slice_sizes_irre[iq]
        src = torch.from_numpy(P0[nts * o: nts * (o + sz)].view(np.float64).copy()).to(dev)
        out = torch.zeros_like(src)
        sizes = np.ascontiguousarray(L.aux_sizes[q], dtype=np.int32)
        torch.cuda.synchronize()
        rc = lib.gwgb_wsolve_noalloc(0, ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                     ctypes.c_void_p(tnt.data_ptr()), ctypes.c_void_p(ttn.data_ptr()),
                                     nts, tr.nw_b, sizes.ctypes.data, len(sizes), None)
        _abi.check(rc)
        got = out.cpu().numpy().view(np.complex128)
        ref = P_ref[nts * o: nts * (o + sz)]
        assert np.abs(got - ref).max() < 1e-12, iq


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

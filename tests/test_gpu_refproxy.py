"""The reference-GPU proxy (the reference's cuBLAS call sequence replayed on
this GPU, measurement only) computes the same P0 and Sigma as the engine's
FP64 kernels: it is a faithful replay, so its timing is a fair comparison."""
import numpy as np
import pytest

from _helpers import crystal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,rotate,ns", [("C1", True, 1), ("C1", False, 2), ("C1", True, 2)])
def test_refproxy_matches_engine(name, rotate, ns):
    from mbsymmetry_gb300.solver import GWSolver
    cr, tr = crystal(name, rotate=rotate, ns=ns)
    s = GWSolver(cr.layout, cr.ns, tr)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    s.dyson(cr.mu)
    s.solve_P0()
    P0 = s.P0_q_t_QP().copy()
    s.solve()                      # P~ in the handle: the proxy's Sigma input
    Sig = s.Selfenergy()
    st = s.refproxy(nt_batch=4, nstreams=4)
    Pp, Sp = s.refproxy_results()
    s.close()
    assert st["gemm_calls"] > 0 and st["p0_ms"] > 0 and st["sigma_ms"] > 0
    assert np.abs(Pp - P0).max() < 1e-11 * max(1.0, np.abs(P0).max())
    assert np.abs(Sp - Sig).max() < 1e-11 * max(1.0, np.abs(Sig).max())

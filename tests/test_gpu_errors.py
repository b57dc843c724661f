"""Error behaviour on the GPU path: state errors, size errors and singular
blocks come back as status codes and leave the handle usable."""
import numpy as np
import pytest

from _helpers import crystal
from mbsymmetry_gb300 import _abi

pytestmark = pytest.mark.gpu


def test_state_size_and_numeric_errors():
    from mbsymmetry_gb300.solver import GWSolver
    cr, tr = crystal("C1")
    s = GWSolver(cr.layout, cr.ns, tr)
    with pytest.raises(_abi.GwgbError) as e:
        s.solve()                                   # V not uploaded yet
    assert e.value.code == _abi.GWGB_E_STATE
    with pytest.raises(_abi.GwgbError) as e:
        s.set_shared_Coulomb(cr.V[:-1])             # wrong size
    assert e.value.code == _abi.GWGB_E_INVALID
    s.set_shared_Coulomb(cr.V)
    # S = 0 and F = 0 make every Dyson block (i w + mu) S - F - Sigma singular
    zero_f = np.zeros_like(cr.F)
    s.set_fock(zero_f, zero_f)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    with pytest.raises(_abi.GwgbError) as e:
        s.dyson(0.0)
    assert e.value.code == _abi.GWGB_E_NUMERIC
    # the handle still works afterwards
    s.set_fock(cr.F, cr.S)
    s.dyson(cr.mu)
    assert np.isfinite(s.G_tau()).all()
    s.close()

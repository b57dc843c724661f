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


def test_bounded_wait_runs_out_and_reports():
    """A device-side wait on a barrier nothing arrives on gives up after its
    poll limit, records a status word, and the host turns it into
    GWGB_E_TIMEOUT; the context stays usable."""
    lib = _abi.load()
    assert lib.gwgb_test_wait_timeout(0, 100000) == _abi.GWGB_E_TIMEOUT
    assert b"ran out" in lib.gwgb_last_error()
    assert lib.gwgb_test_wait_timeout(0, 0) == _abi.GWGB_E_INVALID


def test_injected_status_words_and_nan_inputs():
    """Status words raised as kernels raise them come back as status codes and
    are cleared; NaN in the inputs ends as GWGB_E_NUMERIC, not as silent NaN."""
    from mbsymmetry_gb300.solver import GWSolver
    cr, tr = crystal("C1")
    s = GWSolver(cr.layout, cr.ns, tr)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    lib = _abi.load()
    for which, code in ((2, _abi.GWGB_E_TIMEOUT), (1, _abi.GWGB_E_NUMERIC), (0, _abi.GWGB_E_NUMERIC)):
        _abi.check(lib.gwgb_test_raise_status(s.h, which))
        with pytest.raises(_abi.GwgbError) as e:
            s.synchronize()
        assert e.value.code == code
        s.synchronize()                              # cleared
    assert lib.gwgb_test_raise_status(s.h, 3) == _abi.GWGB_E_INVALID
    bad = cr.F.copy()
    bad[0] = np.nan
    s.set_fock(bad, cr.S)
    with pytest.raises(_abi.GwgbError) as e:
        s.dyson(cr.mu)
    assert e.value.code == _abi.GWGB_E_NUMERIC
    s.set_fock(cr.F, cr.S)
    s.dyson(cr.mu)
    G0 = s.G_tau()
    assert np.isfinite(G0).all()
    s.solve()
    assert np.isfinite(s.Selfenergy()).all()
    s.close()

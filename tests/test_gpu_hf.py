"""Hartree-Fock exchange on the block engine (Sigma contraction with P =
identity, G = rho at tau = 0) against the oracle, with and without rotations."""
import numpy as np
import pytest

from _helpers import crystal
from test_hf_oracle import density, hf_exchange_oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rotate,ns", [(True, 1), (False, 2), (True, 2)])
def test_hf_exchange_matches_oracle(rotate, ns):
    from mbsymmetry_gb300.solver import GWSolver
    cr, tr = crystal("C1", rotate=rotate, ns=ns)
    rho = density(cr)
    s = GWSolver(cr.layout, cr.ns, tr)
    s.set_shared_Coulomb(cr.V)
    K = s.hf_exchange(rho)
    s.close()
    Kr = hf_exchange_oracle(cr, tr, rho)
    assert np.abs(K - Kr).max() < 1e-12 * max(1.0, np.abs(Kr).max())


@pytest.mark.parametrize("rotate,ns", [(True, 1), (False, 2)])
def test_hf_hartree_matches_numpy(rotate, ns):
    from mbsymmetry_gb300.solver import GWSolver
    from test_hf_oracle import hf_hartree_numpy
    cr, tr = crystal("C1", rotate=rotate, ns=ns)
    rho = density(cr)
    s = GWSolver(cr.layout, cr.ns, tr)
    s.set_shared_Coulomb(cr.V)
    J = s.hf_hartree(rho)
    s.close()
    Jr, _ = hf_hartree_numpy(cr, tr, rho)
    assert np.abs(J[0] - Jr).max() < 1e-12 * max(1.0, np.abs(Jr).max())
    assert np.array_equal(J[0], J[-1])

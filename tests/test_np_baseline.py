"""The numpy/BLAS restatement of the contractions (the CPU baseline's second
timed figure, oracle/np_baseline.py) against the C oracle, all tau, on the
rotated C1 crystal with one and two spins."""
import numpy as np
import pytest

import np_baseline
from _helpers import crystal
from oracle import Oracle


@pytest.mark.parametrize("ns", [1, 2])
def test_numpy_contractions_match_oracle(ns):
    cr, tr = crystal("C1", ns=ns)
    L, nts = cr.layout, tr.nts
    orc = Oracle(L, cr.ns, nts)
    zero = np.zeros(nts * cr.ns * L.flat_ao_size, np.complex128)
    G, _ = orc.dyson(zero, cr.F, cr.S, tr, cr.mu)
    Gf = orc.rotate_G(G)
    P0 = orc.p0(Gf, cr.V)
    P0n = np_baseline.p0(L, cr.ns, nts, Gf, cr.V)
    assert np.abs(P0 - P0n).max() < 1e-12 * max(1.0, np.abs(P0).max())
    Pf = orc.rotate_P(orc.p_tilde(P0, tr))
    S = orc.sigma(Gf, Pf, cr.V)
    Sn = np_baseline.sigma(L, cr.ns, nts, Gf, Pf, cr.V)
    assert np.abs(S - Sn).max() < 1e-12 * max(1.0, np.abs(S).max())

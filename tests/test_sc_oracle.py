"""Self-consistent loop pieces of the oracle, pinned by closed forms: the
Galitskii-Migdal quadrature on the IR grid, the electron count N(mu) of the
non-interacting G against the Fermi sum over the band energies, and the mu
bisection.  (No counterpart in the reference: its loop keeps mu fixed and has
no energy; these pins are what makes the restatement trustworthy.)"""
import numpy as np
import pytest
import scipy.linalg

from _helpers import crystal
from mbsymmetry_gb300.crystal import load_ir
from mbsymmetry_gb300.transformer import build_transforms, gm_matrix
from oracle import Oracle


@pytest.mark.parametrize("nts,beta", [(62, 50.0), (100, 100.0)])
def test_gm_matrix_closed_form(nts, beta):
    # int_0^beta G(tau) G(beta - tau) dtau = beta e^{-beta|e|} / (1 + e^{-beta|e|})^2
    # for G(tau) = -e^{-e tau} (1 - f(e)), one level at energy e
    tr = build_transforms(load_ir(nts), beta)
    M = gm_matrix(tr)
    assert np.allclose(M, M.T, atol=1e-13)
    tau = tr.tau_fermi[1:-1]
    for e in (-0.7, -0.1, 0.0, 0.05, 0.3):
        if e >= 0:
            g = -np.exp(-e * tau) / (1.0 + np.exp(-beta * e))
        else:
            g = -np.exp(-e * (tau - beta)) / (np.exp(beta * e) + 1.0)
        x = np.exp(-beta * abs(e))
        assert abs(g @ M @ g - beta * x / (1.0 + x) ** 2) < 1e-11


def _fermi_count(cr, L, mu, beta, ns):
    w = np.bincount(L.irre_index, minlength=L.ink)
    fa = L.flat_ao_size
    Fb = L.G_flat_to_block(cr.F.reshape(ns, fa))
    Sb = L.G_flat_to_block(cr.S.reshape(ns, fa))
    n = 0.0
    for s in range(ns):
        for ik in range(L.ink):
            e = scipy.linalg.eigh(Fb[s, ik], Sb[s, ik], eigvals_only=True)
            n += w[ik] * np.sum(0.5 * (1.0 - np.tanh(0.5 * beta * (e - mu))))
    return (2.0 / ns) / L.nk * n


@pytest.mark.parametrize("ns", [1, 2])
def test_oracle_n_electrons_noninteracting(ns):
    cr, tr = crystal("C1", ns=ns)
    L = cr.layout
    orc = Oracle(L, ns, tr.nts)
    zero = np.zeros(tr.nts * ns * L.flat_ao_size, np.complex128)
    for mu in (cr.mu - 0.3, cr.mu, cr.mu + 0.2):
        G, _ = orc.dyson(zero, cr.F, cr.S, tr, mu)
        n = orc.n_electrons(G, cr.S)
        assert abs(n - _fermi_count(cr, L, mu, tr.beta, ns)) < 1e-7


def test_oracle_find_mu_hits_target():
    cr, tr = crystal("C1")
    L = cr.layout
    orc = Oracle(L, 1, tr.nts)
    zero = np.zeros(tr.nts * L.flat_ao_size, np.complex128)
    target = float(L.nao) - 0.25  # a metallic filling: N(mu) is steep and smooth
    mu, G, _ = orc.find_mu(zero, cr.F, cr.S, tr, target, cr.mu, step=0.05, tol=1e-11)
    assert abs(orc.n_electrons(G, cr.S) - target) < 1e-11
    assert abs(_fermi_count(cr, L, mu, tr.beta, 1) - target) < 1e-7

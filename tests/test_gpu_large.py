"""Large configurations: the FP64 drop-in against the oracle on sampled tau
points (the full CPU oracle would take hours), the full W~ solve against the
oracle, and the sliced split-precision path (precision "ozaki") against FP64
at its stated bound: Sigma, G and the correlation energy within 1e-7 Ha.

* C3: Fm-3m 4x4x4 (64 k, 8 irreducible), nao=52, naux=250, nts=120; AO blocks
  up to 16, aux blocks up to 64; V 12.2 GB.
* C4: P6_3mc-like hexagonal 4x4x3 (48 k, 8 irreducible), nao=72, naux=350,
  nts=120, beta=200; AO and aux blocks up to 30; V 17.1 GB."""
import numpy as np
import pytest

from _helpers import crystal, p_slices
from oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,max_block", [("C3", 64), ("C4", 30)])
def test_large_fp64_matches_oracle_and_sliced_within_bound(name, max_block):
    from mbsymmetry_gb300.solver import GWSolver
    cr, tr = crystal(name)
    L = cr.layout
    nts = tr.nts
    assert L.max_block() == max_block and L.ink == 8
    s = GWSolver(L, 1, tr)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    s.dyson(cr.mu)
    G0 = s.G_tau()
    s.solve_P0()
    P0 = s.P0_q_t_QP()
    s.set_G(G0)
    s.solve()
    Pt, Sig = s.P0_q_t_QP(), s.Selfenergy()
    e64 = s.energy()[0]
    s.dyson(cr.mu)
    G64 = s.G_tau()
    s.single_prec_run(True, "ozaki")
    s.set_G(G0)
    s.solve()
    Sig_oz, e_oz = s.Selfenergy(), s.energy()[0]
    s.dyson(cr.mu)
    G_oz = s.G_tau()
    s.close()

    orc = Oracle(L, 1, nts)
    Gf = orc.rotate_G(G0)
    P0r = orc.p0(Gf, cr.V, nt_max=2)
    assert np.abs(p_slices(L, nts, P0, [0, 1]) - p_slices(L, nts, P0r, [0, 1])).max() < 1e-10
    Ptr = orc.p_tilde(orc.mirror_P0(P0), tr)
    assert np.abs(Ptr - Pt).max() < 1e-10
    Sr = orc.sigma(Gf, orc.rotate_P(Pt), cr.V, nt_max=2)
    assert np.abs(Sig.reshape(nts, -1)[:2] - Sr.reshape(nts, -1)[:2]).max() < 1e-10

    err, gerr = np.abs(Sig_oz - Sig).max(), np.abs(G_oz - G64).max()
    print(f"{name}: max|Sigma_ozaki - Sigma_fp64| = {err:.3e} (max|Sigma| = {np.abs(Sig).max():.3e}), "
          f"G {gerr:.3e}, E_corr {e_oz:.12f} vs {e64:.12f}")
    assert err < 1e-7 and gerr < 1e-7
    assert abs(e_oz - e64) < 1e-7

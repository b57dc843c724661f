"""GPU self-consistent loop (device mu search, energies, mixing, graph loop)
against the oracle's restatement of the same formulas (parity unpinned by
the reference, which has no such loop; the oracle pieces are pinned by closed
forms in test_sc_oracle.py)."""
import numpy as np
import pytest

from _helpers import crystal
from mbsymmetry_gb300.transformer import gm_matrix
from oracle import Oracle

pytestmark = pytest.mark.gpu

TOL_MU_SEARCH = 1e-10   # |N - target| the device search is asked for


def _solver(cr, tr, ns, precision="fp64"):
    from mbsymmetry_gb300.solver import GWSolver
    s = GWSolver(cr.layout, ns, tr, precision=precision)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    s.set_hcore(cr.H)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    return s


@pytest.mark.parametrize("metallic", [False, True])
def test_find_mu_matches_oracle(metallic):
    cr, tr = crystal("C1")
    L = cr.layout
    target = float(L.nao) - (0.25 if metallic else 0.0)
    s = _solver(cr, tr, 1)
    mu, n = s.find_mu(target, cr.mu + 0.1, step=0.05, tol=TOL_MU_SEARCH, max_evals=40)
    G = s.G_tau()
    s.close()
    assert abs(n - target) <= TOL_MU_SEARCH
    orc = Oracle(L, 1, tr.nts)
    zero = np.zeros(tr.nts * L.flat_ao_size, np.complex128)
    Gr, _ = orc.dyson(zero, cr.F, cr.S, tr, mu)
    assert np.abs(G - Gr).max() < 1e-10
    assert abs(orc.n_electrons(Gr, cr.S) - target) < 1e-9
    if metallic:  # N(mu) is steep: the root is unique to ~tol / slope
        mur, _, _ = orc.find_mu(zero, cr.F, cr.S, tr, target, cr.mu, tol=1e-12)
        assert abs(mu - mur) < 1e-8


def test_energy_matches_oracle():
    cr, tr = crystal("C1")
    L = cr.layout
    orc = Oracle(L, 1, tr.nts)
    zero = np.zeros(tr.nts * L.flat_ao_size, np.complex128)
    G0, _ = orc.dyson(zero, cr.F, cr.S, tr, cr.mu)
    Sig, _, _ = orc.gw_sigma(G0, cr.V, tr)
    G1, _ = orc.dyson(Sig, cr.F, cr.S, tr, cr.mu)
    ec_r, eo_r, _ = orc.energy(Sig, G1, cr.F, cr.S, gm_matrix(tr), cr.H)
    s = _solver(cr, tr, 1)
    s.set_Selfenergy(Sig)
    s.set_G(G1)
    ec, eo = s.energy(with_one_body=True)
    s.close()
    assert abs(ec - ec_r) < 1e-10 and abs(eo - eo_r) < 1e-10
    assert ec < 0.0


@pytest.mark.parametrize("ns", [1, 2])
def test_sc_loop_matches_oracle(ns):
    cr, tr = crystal("C1", ns=ns)
    L = cr.layout
    target = float(L.nao)
    s = _solver(cr, tr, ns)
    s.dyson(cr.mu)
    G0 = s.G_tau()
    recs = s.sc_loop(3, 0.5, target, cr.mu, step=0.05, tol=TOL_MU_SEARCH, max_evals=40)
    G, Sig = s.G_tau(), s.Selfenergy()
    s.close()
    for r in recs:
        assert abs(r["n_electrons"] - target) <= 1e-9
        assert r["precision"] == 0 and 1 <= r["mu_evals"] <= 40
    orc = Oracle(L, ns, tr.nts)
    zero = np.zeros_like(G0)
    Gr, Sr, rr = orc.sc_loop(G0, zero, cr.V, cr.F, cr.S, tr, gm_matrix(tr), 3, 0.5, target, cr.mu,
                             H=cr.H, mus=[r["mu"] for r in recs])
    for a, b in zip(recs, rr):
        assert abs(a["e_corr"] - b["e_corr"]) < 1e-9
        assert abs(a["e_one"] - b["e_one"]) < 1e-9
        assert abs(a["n_electrons"] - b["n_electrons"]) < 1e-9
    assert np.abs(G - Gr).max() < 1e-9
    assert np.abs(Sig - Sr).max() < 1e-9


def test_sc_loop_reproducible_and_mixed_final_fp64():
    cr, tr = crystal("C1")
    L = cr.layout
    target = float(L.nao)
    runs = []
    for precision, final in (("fp64", False), ("fp64", False), ("tf32x3", True)):
        s = _solver(cr, tr, 1, precision)
        s.dyson(cr.mu)
        recs = s.sc_loop(3, 0.5, target, cr.mu, tol=TOL_MU_SEARCH, max_evals=40, final_fp64=final)
        runs.append((recs, s.G_tau()))
        s.close()
    (r1, g1), (r2, g2), (r3, g3) = runs
    assert r1 == r2 and np.array_equal(g1, g2)            # graph replay is bitwise reproducible
    assert [r["precision"] for r in r3] == [1, 1, 0]
    assert abs(r3[-1]["e_corr"] - r1[-1]["e_corr"]) < 1e-5
    assert np.abs(g3 - g1).max() < 1e-5


def test_sc_loop_checkpoint_resume_is_exact(tmp_path):
    """2 iterations, checkpoint (G, Sigma, mu), a new handle resumes for 1:
    bitwise the same G and records as 3 iterations in one run."""
    import io
    import json
    cr, tr = crystal("C1")
    target = float(cr.layout.nao)
    s = _solver(cr, tr, 1)
    s.dyson(cr.mu)
    G0 = s.G_tau()
    r3 = s.sc_loop(3, 0.5, target, cr.mu, tol=TOL_MU_SEARCH, max_evals=40)
    g3 = s.G_tau()
    s.set_G(G0)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    log = io.StringIO()
    r2 = s.sc_loop(2, 0.5, target, cr.mu, tol=TOL_MU_SEARCH, max_evals=40, log=log)
    s.save_state(str(tmp_path / "state"), mu=r2[-1]["mu"], iteration=2)
    s.close()
    lines = [json.loads(x) for x in log.getvalue().splitlines()]
    assert [x["iteration"] for x in lines] == [0, 1] and lines[1]["mu"] == r2[1]["mu"]
    s2 = _solver(cr, tr, 1)
    hdr = s2.load_state(str(tmp_path / "state"))
    assert hdr["iteration"] == 2
    r1 = s2.sc_loop(1, 0.5, target, hdr["mu"], tol=TOL_MU_SEARCH, max_evals=40)
    g = s2.G_tau()
    s2.close()
    assert r2 == r3[:2] and r1[0] == r3[2]
    assert np.array_equal(g, g3)

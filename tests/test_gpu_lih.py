"""GPU parity on the reference's LiH fixture (ns=2, nk=8, nts=74) through the
C ABI, against the golden fixtures and the FP64 oracle.  Tolerances are the
reference tests' own (test_cugw.cpp:72,98,186,203 -> 1e-10; :301 -> 1e-9)."""
import numpy as np
import pytest

from _helpers import lih, p_slices
from oracle import Oracle

pytestmark = pytest.mark.gpu

# G(tau) of this fixture reaches |G| = 329 (the LiH overlap S(k) is nearly
# singular), so the reference test's 1e-10 absolute bound on G is 3e-13
# relative -- the rounding floor of two FP64 inversion/transform orders.  The
# GPU result is held to 2e-10 absolute (6e-13 relative) against the dense
# golden path; Sigma, P0 and P~ keep the reference's bounds.
TOL_G = 2e-10


@pytest.fixture(scope="module")
def solver():
    from mbsymmetry_gb300.solver import GWSolver
    d = lih()
    s = GWSolver(d["layout"], d["ns"], d["tr"])
    s.set_shared_Coulomb(d["V"])
    s.set_fock(d["F"], d["S"])
    yield s, d
    s.close()


def _g0(s, d):
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    s.dyson(d["mu"])          # sc.init_g(): Dyson with Sigma = 0


def test_dyson_g0(solver):
    s, d = solver
    _g0(s, d)
    G = s.G_tau()
    assert np.abs(G - d["golden"]["G"]).max() < TOL_G
    assert s.stats()["leakage"] < 1e-8


def test_solve_P0(solver):
    s, d = solver
    _g0(s, d)
    s.solve_P0()
    P0 = s.P0_q_t_QP()
    L, nts = d["layout"], d["tr"].nts
    nt = int(d["golden"]["nt_p0"])
    assert np.abs(p_slices(L, nts, P0, range(nt)) - d["golden"]["P0_t"]).max() < 1e-10
    assert np.abs(p_slices(L, nts, P0, range(nts // 2, nts))).max() == 0.0


def test_compute_Pq_from_P0q(solver):
    s, d = solver
    _g0(s, d)
    s.solve_P0()
    s.compute_Pq_from_P0q()
    P = s.P0_q_t_QP()
    L, nts = d["layout"], d["tr"].nts
    assert np.abs(p_slices(L, nts, P, d["golden"]["t_pt"]) - d["golden"]["P_tilde_t"]).max() < 1e-9


def test_solve_sigma_from_P0(solver):
    s, d = solver
    _g0(s, d)
    s.solve_sigma()
    Sig = s.Selfenergy()
    L, nts, ns = d["layout"], d["tr"].nts, d["ns"]
    orc = Oracle(L, ns, nts)
    G = s.G_tau()
    Gf = orc.rotate_G(G)
    P0 = orc.mirror_P0(orc.p0(Gf, d["V"]))
    ref = orc.sigma(Gf, orc.rotate_P(P0), d["V"])
    assert np.abs(Sig - ref).max() < 1e-10


def test_full_solve_and_dyson(solver):
    s, d = solver
    _g0(s, d)
    s.solve()
    Sig = s.Selfenergy()
    L, nts, ns = d["layout"], d["tr"].nts, d["ns"]
    nt = int(d["golden"]["nt_sigma"])
    assert np.abs(Sig.reshape(nts, ns, -1)[:nt].reshape(-1) - d["golden"]["Sigma_t"]).max() < 1e-10
    s.dyson(d["mu"])
    assert np.abs(s.G_tau() - d["golden"]["G_after_gw"]).max() < TOL_G


def test_graph_iteration_matches_and_is_deterministic(solver):
    s, d = solver
    _g0(s, d)
    s.iteration(d["mu"])
    G1 = s.G_tau()
    S1 = s.Selfenergy()
    assert np.abs(G1 - d["golden"]["G_after_gw"]).max() < TOL_G
    _g0(s, d)
    s.iteration(d["mu"])     # graph replay
    assert np.array_equal(s.G_tau(), G1) and np.array_equal(s.Selfenergy(), S1)

"""The FP64 oracle against the LiH golden fixtures (reference data).

The golden G, P0, P~ and Sigma come from dense restatements of the
reference's dense solver (Dyson, gw.cpp compute_full_P0_t /
compute_Sigma_from_P_t / compute_P_from_P0) run on the reference's dense
adapted-basis inputs; the relations recorded by tests/golden/make_golden.py
are the pins of the oracle (reference tests Dyson.BlockDyson, CuGWP.LiHnk2).
"""
import numpy as np
import pytest

from _helpers import lih, p_slices
from oracle import Oracle


@pytest.fixture(scope="module")
def run():
    d = lih()
    L, tr, ns = d["layout"], d["tr"], d["ns"]
    orc = Oracle(L, ns, tr.nts)
    zero = np.zeros(tr.nts * ns * L.flat_ao_size, np.complex128)
    G, leak = orc.dyson(zero, d["F"], d["S"], tr, d["mu"])
    Gf = orc.rotate_G(G)
    P0 = orc.p0(Gf, d["V"])
    P = orc.p_tilde(P0, tr)
    Sig = orc.sigma(Gf, orc.rotate_P(P), d["V"])
    return d, G, P0, P, Sig, leak


def test_recorded_relations():
    g = lih()["golden"]
    assert g["rel_dyson_block_vs_dense"] < 1e-10      # test_dyson.cpp:82 tolerance
    assert g["rel_p_tilde_block_vs_dense"] < 1e-9     # test_cugw.cpp:301 tolerance
    assert g["rel_V_spectra_block_vs_dense"] < 1e-10
    assert g["rel_p0_oracle_vs_numpy"] < 1e-12
    assert g["rel_sigma_oracle_vs_numpy"] < 1e-12
    # block P0 / Sigma vs the reference's dense solver (gw.cpp:65-127) on the dense chain
    assert g["rel_p0_block_vs_dense_gw"] < 1e-10
    assert g["rel_sigma_block_vs_dense_gw"] < 1e-10


def test_dyson_G(run):
    d, G, *_ , leak = run
    assert np.abs(G - d["golden"]["G"]).max() < 1e-10
    assert leak < 1e-8


def test_p0(run):
    d, G, P0, *_ = run
    L, nts = d["layout"], d["tr"].nts
    nt = int(d["golden"]["nt_p0"])
    assert np.abs(p_slices(L, nts, P0, range(nt)) - d["golden"]["P0_t"]).max() < 1e-12
    # the oracle leaves t >= nts/2 at zero, as solve_P0 does
    assert np.abs(p_slices(L, nts, P0, range(nts // 2, nts))).max() == 0.0


def test_p_tilde(run):
    d, G, P0, P, *_ = run
    L, nts = d["layout"], d["tr"].nts
    got = p_slices(L, nts, P, d["golden"]["t_pt"])
    assert np.abs(got - d["golden"]["P_tilde_t"]).max() < 1e-9


def test_sigma(run):
    d, G, P0, P, Sig, _ = run
    L, nts, ns = d["layout"], d["tr"].nts, d["ns"]
    nt = int(d["golden"]["nt_sigma"])
    got = Sig.reshape(nts, ns, L.flat_ao_size)[:nt].reshape(-1)
    assert np.abs(got - d["golden"]["Sigma_t"]).max() < 1e-10  # dense chain: 1.2e-12


def test_thread_count_invariance():
    d = lih()
    L, tr, ns = d["layout"], d["tr"], d["ns"]
    zero = np.zeros(tr.nts * ns * L.flat_ao_size, np.complex128)
    res = []
    for th in (1, 3):
        orc = Oracle(L, ns, tr.nts, threads=th)
        G, _ = orc.dyson(zero, d["F"], d["S"], tr, d["mu"])
        res.append(orc.p0(orc.rotate_G(G), d["V"], nt_max=3))
    assert np.array_equal(res[0], res[1])

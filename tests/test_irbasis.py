"""IR sparse-sampling grids: pin the basis against the reference's 1e3_72
grid and check every committed grid with exact single-pole round trips."""
import numpy as np
import pytest

from _helpers import lih
from mbsymmetry_gb300.crystal import load_ir
from mbsymmetry_gb300.irbasis import IRBasis
from mbsymmetry_gb300.transformer import build_transforms


def _single_pole_error(tr):
    beta, tau = tr.beta, tr.tau_fermi
    worst = 0.0
    for e in (-3.0, -0.5, 0.0, 0.2, 2.5):
        if e >= 0:
            g = -np.exp(-e * tau) / (1 + np.exp(-beta * e))
        else:
            g = -np.exp(e * (beta - tau)) / (1 + np.exp(beta * e))
        exact_w = 1.0 / (tr.omega_fermi() - e)
        worst = max(worst, np.abs(tr.Tnt @ g[1:-1] - exact_w).max(), np.abs((tr.Ttn @ exact_w) - g).max())
    return worst


def test_basis_matches_reference_grid():
    ir = lih()["ir"]
    F = IRBasis("F", 1e3, 72)
    B = IRBasis("B", 1e3, 71)
    lmax = 36  # functions whose singular values are well above FP64 resolution
    # the bosonic l = 0 function agrees to ~1e-8, every other function far better
    for basis, st, tol in ((F, "fermi", 1e-8), (B, "bose", 1e-7)):
        u = basis.u(ir[f"{st}/xsample"])[:, :lmax]
        ref = ir[f"{st}/uxl"][:, :lmax]
        assert np.abs(u - ref).max() / np.abs(ref).max() < tol
        uh = basis.uhat(ir[f"{st}/wsample"])[:, :lmax]
        refh = (ir[f"{st}/uwl_re"] + 1j * ir[f"{st}/uwl_im"])[:, :lmax]
        assert np.abs(uh - refh).max() / np.abs(refh).max() < tol
        assert np.abs(basis.u(np.array([1.0]))[0, :lmax] - ir[f"{st}/ux1l"][:lmax]).max() < 10 * tol


def test_reference_grid_round_trip():
    assert _single_pole_error(lih()["tr"]) < 1e-11


@pytest.mark.parametrize("nts,beta,tol", [(62, 50.0, 1e-9), (100, 100.0, 1e-8), (120, 100.0, 1e-7),
                                          (150, 200.0, 1e-6)])
def test_committed_grids_round_trip(nts, beta, tol):
    ir = load_ir(nts)
    tr = build_transforms(ir, beta)
    assert tr.nts == nts and tr.nw == nts - 2 and tr.nw_b == nts - 3
    assert np.linalg.cond(ir["fermi/uxl"]) < 1e4
    assert _single_pole_error(tr) < tol


@pytest.mark.parametrize("nts", [62, 100, 120, 150])
def test_committed_grids_sample_symmetrically(nts):
    """Matsubara sampling closed under nu -> -nu, like the reference's own grid
    (and sparse-ir's): time reversal maps the sampled frequencies onto
    themselves."""
    ir = load_ir(nts)
    wf, wb = ir["fermi/wsample"].ravel(), ir["bose/wsample"].ravel()
    assert set(wf.tolist()) == set((-wf - 1).tolist()) and set(wb.tolist()) == set((-wb).tolist())
    ref = lih()["ir"]
    assert set(ref["fermi/wsample"].ravel().tolist()) == set((-ref["fermi/wsample"].ravel() - 1).tolist())

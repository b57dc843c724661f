"""The GPU engine on tight-binding crystals from Gaussian orbitals
(mbsymmetry_gb300/orbitals.py: Slater-Koster F, V from Gaussian auxiliary
functions, bases and rotations from O_h, the selection rule from the data):
the FP64 path against the oracle at 1e-10, the reference's iBZ-vs-full-BZ
relation (SymmetryMBPT/test/test_cugw.cpp:306-436) on the FP64 path at 1e-10,
and the sliced path against FP64 at the stated 1e-7 Ha."""
import numpy as np
import pytest

from mbsymmetry_gb300.crystal import CONFIGS, load_ir
from mbsymmetry_gb300.orbitals import make_orbital_crystal
from mbsymmetry_gb300.transformer import build_transforms

pytestmark = pytest.mark.gpu


def _sigma(cr, tr, precision, G0=None):
    """Sigma from G0: the given one, or the handle's own Dyson G0 at mu."""
    from mbsymmetry_gb300.solver import GWSolver
    s = GWSolver(cr.layout, cr.ns, tr, precision=precision)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    if G0 is None:
        s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
        s.dyson(cr.mu)
    else:
        s.set_G(G0)
    s.solve()
    out = s.Selfenergy()
    s.close()
    return out


def test_orbital_crystal_on_the_gpu():
    from oracle import Oracle
    spec = CONFIGS["C1"]
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = make_orbital_crystal(spec, rotate=True)
    cf = make_orbital_crystal(spec, rotate=False)
    L, nts, ns = cr.layout, tr.nts, cr.ns
    orc = Oracle(L, ns, nts)
    G0, _ = orc.dyson(np.zeros(nts * ns * L.flat_ao_size, np.complex128), cr.F, cr.S, tr, cr.mu)
    _, Sr, *_ = orc.iteration(G0, cr.V, cr.F, cr.S, tr, cr.mu)
    s64 = _sigma(cr, tr, "fp64", G0)
    soz = _sigma(cr, tr, "ozaki", G0)
    x = _sigma(cr, tr, "fp64").reshape(nts, ns, -1)
    sfull = _sigma(cf, tr, "fp64").reshape(nts, ns, -1)
    d_full = 0.0
    for ik, k in enumerate(L.irre_list):
        n = L.kao_slice_sizes[k]
        d_full = max(d_full, float(np.abs(x[:, :, L.kao_slice_offsets_irre[ik]:][:, :, :n]
                                          - sfull[:, :, cf.layout.kao_slice_offsets_irre[k]:][:, :, :n]).max()))
    e64, eoz = float(np.abs(s64 - Sr).max()), float(np.abs(soz - s64).max())
    print(f"orbital C1: FP64 vs oracle {e64:.1e}, iBZ vs full BZ {d_full:.1e}, sliced vs FP64 {eoz:.1e} "
          f"(max|Sigma| {np.abs(s64).max():.2f})")
    assert e64 < 1e-10 and d_full < 1e-10 and eoz < 1e-7


def test_wurtzite_orbital_crystal_with_time_reversal_on_the_gpu():
    """P6_3mc orbital crystal on a 2x2x3 mesh, where time reversal brings
    kz = 2/3 into the stars of kz = 1/3: the GPU's rotation path conjugates G
    and P~ there; the iBZ run agrees with the full mesh and with the oracle."""
    import dataclasses
    from oracle import Oracle
    spec = dataclasses.replace(CONFIGS["C4"], name="wurtzite", mesh=(2, 2, 3), nao=16, naux=40, nts=62, beta=50.0)
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = make_orbital_crystal(spec, rotate=True)
    cf = make_orbital_crystal(spec, rotate=False)
    L, nts, ns = cr.layout, tr.nts, cr.ns
    assert np.any(L.conj_index != np.arange(L.nk))
    orc = Oracle(L, ns, nts)
    G0, _ = orc.dyson(np.zeros(nts * ns * L.flat_ao_size, np.complex128), cr.F, cr.S, tr, cr.mu)
    _, Sr, *_ = orc.iteration(G0, cr.V, cr.F, cr.S, tr, cr.mu)
    e64 = float(np.abs(_sigma(cr, tr, "fp64", G0) - Sr).max())
    x = _sigma(cr, tr, "fp64").reshape(nts, ns, -1)
    sfull = _sigma(cf, tr, "fp64").reshape(nts, ns, -1)
    d_full = max(float(np.abs(x[:, :, L.kao_slice_offsets_irre[ik]:][:, :, :L.kao_slice_sizes[k]]
                              - sfull[:, :, cf.layout.kao_slice_offsets_irre[k]:][:, :, :L.kao_slice_sizes[k]]).max())
                 for ik, k in enumerate(L.irre_list))
    print(f"wurtzite orbital 2x2x3: FP64 vs oracle {e64:.1e}, iBZ vs full BZ {d_full:.1e}")
    assert e64 < 1e-10 and d_full < 1e-9

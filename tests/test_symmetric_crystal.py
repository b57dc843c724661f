"""Group-consistent synthetic crystals and the reference's iBZ-vs-full-BZ
relation on the oracle (SymmetryMBPT/test/test_cugw.cpp:306-436,
CuGWRotP0 / CuGWRotSigma): the same crystal computed on the irreducible k
points with the orep / auxrep rotations and on every k point of the mesh
gives the same G, P~ (every q) and Sigma (irreducible k).  The labelled
crystal (random rotations, V not symmetric) is the negative control."""
import numpy as np
import pytest

from mbsymmetry_gb300.crystal import CONFIGS, load_ir, make_crystal
from mbsymmetry_gb300.transformer import build_transforms
from oracle import Oracle


def _both(symmetric, ns=1):
    import dataclasses
    spec = dataclasses.replace(CONFIGS["C1"], ns=ns)
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    return (make_crystal(spec, rotate=True, symmetric=symmetric),
            make_crystal(spec, rotate=False, symmetric=symmetric), tr)


def _chain(cr, tr, mu):
    L, ns, nts = cr.layout, cr.ns, tr.nts
    orc = Oracle(L, ns, nts)
    G, _ = orc.dyson(np.zeros(nts * ns * L.flat_ao_size, np.complex128), cr.F, cr.S, tr, mu)
    Gf = orc.rotate_G(G)
    P = orc.p_tilde(orc.mirror_P0(orc.p0(Gf, cr.V)), tr)
    Pf = orc.rotate_P(P)
    return Gf, Pf, orc.sigma(Gf, Pf, cr.V)


def _sigma_irr_diff(cr, cf, Sr, Sf, nts):
    Lr, Lf, ns = cr.layout, cf.layout, cr.ns
    Sr, Sf = Sr.reshape(nts, ns, -1), Sf.reshape(nts, ns, -1)
    d = 0.0
    for ik, k in enumerate(Lr.irre_list):
        n = Lr.kao_slice_sizes[k]
        a = Sr[:, :, Lr.kao_slice_offsets_irre[ik]:Lr.kao_slice_offsets_irre[ik] + n]
        b = Sf[:, :, Lf.kao_slice_offsets_irre[k]:Lf.kao_slice_offsets_irre[k] + n]
        d = max(d, float(np.abs(a - b).max()))
    return d


@pytest.mark.parametrize("ns", [1, 2])
def test_irreducible_and_full_mesh_agree(ns):
    cr, cf, tr = _both(True, ns)
    assert np.array_equal(cr.V, cf.V) and cr.layout.ink < cf.layout.ink == cf.layout.nk
    Gr, Pr, Sr = _chain(cr, tr, cr.mu)
    Gf, Pf, Sf = _chain(cf, tr, cr.mu)
    print(f"ns={ns}: G {np.abs(Gr - Gf).max():.1e}, P~ {np.abs(Pr - Pf).max():.1e} (max {np.abs(Pf).max():.2f}), "
          f"Sigma {_sigma_irr_diff(cr, cf, Sr, Sf, tr.nts):.1e}")
    assert np.abs(Gr - Gf).max() < 1e-12       # G(k) = orep G(k_irr) orep^H on every k
    assert np.abs(Pr - Pf).max() < 1e-12       # P~(q) = auxrep P~(q_irr) auxrep^H on every q
    assert _sigma_irr_diff(cr, cf, Sr, Sf, tr.nts) < 1e-12


def test_symmetric_V_keeps_the_hermitian_pair_relation():
    cr, _, _ = _both(True)
    L, V = cr.layout, cr.V
    for k1 in range(L.nk):
        for k2 in range(L.nk):
            p, pr = k1 * L.nk + k2, k2 * L.nk + k1
            q = L.pair_q(k1, k2)
            rev = {tuple(int(x) for x in t): i for i, t in enumerate(L.tensor_irreps[pr])}
            for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
                qb, b1, b2 = L.aux_sizes[q][iq], L.ao_sizes[k1][i1], L.ao_sizes[k2][i2]
                o = L.kpair_slice_offsets[p] + L.tensor_offsets[p][b]
                br = rev[(int(iq), int(i2), int(i1))]
                orr = L.kpair_slice_offsets[pr] + L.tensor_offsets[pr][br]
                a = V[o:o + qb * b1 * b2].reshape(qb, b1, b2)
                r = V[orr:orr + qb * b1 * b2].reshape(qb, b2, b1)
                assert np.abs(r - a.transpose(0, 2, 1).conj()).max() < 1e-14


def test_labelled_crystal_is_not_group_consistent():
    """Negative control: random rotations and unsymmetrised V break the relation."""
    cr, cf, tr = _both(False)
    _, Pr, _ = _chain(cr, tr, cr.mu)
    _, Pf, _ = _chain(cf, tr, cr.mu)
    assert np.abs(Pr - Pf).max() > 1e-3

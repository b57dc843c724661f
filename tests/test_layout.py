"""Layout model and synthetic crystals (host logic, no GPU)."""
import numpy as np
import pytest

from _helpers import crystal, lih
from mbsymmetry_gb300.crystal import CONFIGS, make_crystal
from oracle import Oracle


@pytest.mark.parametrize("name,ink", [("C1", 4), ("C2", 4)])
def test_fcc_irreducible_counts(name, ink):
    cr, _ = crystal(name)
    L = cr.layout
    assert L.nk == 27 and L.ink == ink
    assert cr.star_sizes.sum() == L.nk


def test_c3_c5_meshes():
    # only the k-mesh symmetry part (cheap): 64 k -> 8 and 125 k -> 10 irreducible
    from mbsymmetry_gb300.crystal import _fcc_ops, _kmesh, _stars
    ops, inv = _fcc_ops()
    for mesh, ink in (((4, 4, 4), 8), ((5, 5, 5), 10)):
        reps, *_ = _stars(_kmesh(mesh), ops, inv)
        assert len(reps) == ink


def test_hex_time_reversal_mesh():
    from mbsymmetry_gb300.crystal import _hex_ops, _kmesh, _stars
    ops, inv = _hex_ops()
    km = _kmesh((4, 4, 3))
    reps, star_of, index, conj = _stars(km, ops, inv)
    assert len(km) == 48 and not inv
    assert np.bincount(star_of).sum() == 48


@pytest.mark.parametrize("rotate", [True, False])
def test_crystal_invariants(rotate):
    cr, _ = crystal("C1", rotate=rotate)
    L = cr.layout
    for q in range(L.nk):
        mq = L.mom_cons(0, q, 0)
        assert np.array_equal(L.aux_sizes[q], L.aux_sizes[mq])
    # Hermitian pair relation V(k2,k1)_{Q,j,i} = conj(V(k1,k2)_{Q,i,j})
    for k1 in range(L.nk):
        for k2 in range(L.nk):
            p, pr = k1 * L.nk + k2, k2 * L.nk + k1
            rev = {tuple(t): i for i, t in enumerate(L.tensor_irreps[pr])}
            q = L.pair_q(k1, k2)
            for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p][:3]):
                qb, b1, b2 = L.aux_sizes[q][iq], L.ao_sizes[k1][i1], L.ao_sizes[k2][i2]
                o = L.kpair_slice_offsets[p] + L.tensor_offsets[p][b]
                br = rev[(iq, i2, i1)]
                orr = L.kpair_slice_offsets[pr] + L.tensor_offsets[pr][br]
                a = cr.V[o:o + qb * b1 * b2].reshape(qb, b1, b2)
                r = cr.V[orr:orr + qb * b1 * b2].reshape(qb, b2, b1)
                assert np.abs(r - a.transpose(0, 2, 1).conj()).max() == 0.0
    if not rotate:
        assert L.ink == L.nk


def test_oracle_layout_agrees_with_python():
    for lay in (lih()["layout"], crystal("C1")[0].layout):
        o = Oracle(lay, 1, 8)
        assert o.lib.gwo_flat_ao_full(o.h) == lay.flat_ao_size_full
        assert o.lib.gwo_flat_aux_full(o.h) == lay.flat_aux_size_full
        assert o.lib.gwo_flat_orep(o.h) == lay.orep.size
        assert o.lib.gwo_flat_auxrep(o.h) == lay.auxrep.size


def test_reproducible_generation():
    a = make_crystal(CONFIGS["C1"])
    b = make_crystal(CONFIGS["C1"])
    assert np.array_equal(a.V, b.V) and np.array_equal(a.F, b.F) and a.mu == b.mu

"""V stored only for the pairs with an irreducible first k, and P0 re-indexed
through the group (mbsymmetry_gb300/vstore.py), against the oracle's
all-pairs P0 loop (SymmetryMBPT/src/cpu_ref/gw_block.cpp:19-79): the same P0
at every irreducible q from a fraction of V."""
import dataclasses

import numpy as np
import pytest

from mbsymmetry_gb300 import orbitals as O
from mbsymmetry_gb300 import vstore
from mbsymmetry_gb300.crystal import CONFIGS, load_ir
from mbsymmetry_gb300.transformer import build_transforms
from oracle import Oracle

CASES = {
    "fcc-C1": (CONFIGS["C1"], 1e-13),
    "fcc-C1-ns2": (dataclasses.replace(CONFIGS["C1"], ns=2), 1e-13),
    # time reversal brings kz = 2/3 into the stars: c(-k, q) = conj(c(k, -q))
    "wurtzite-2x2x3": (dataclasses.replace(CONFIGS["C4"], name="wurtzite", mesh=(2, 2, 3), nao=16, naux=40,
                                           nts=62, beta=50.0), 1e-11),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_p0_from_pairs_with_an_irreducible_first_k(case):
    spec, bound = CASES[case]
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = O.make_orbital_crystal(spec, rotate=True, transports=True)
    L, nts, ns = cr.layout, tr.nts, cr.ns
    orc = Oracle(L, ns, nts)
    G, _ = orc.dyson(np.zeros(nts * ns * L.flat_ao_size, np.complex128), cr.F, cr.S, tr, cr.mu)
    Gf = orc.rotate_G(G)
    P0 = orc.p0(Gf, cr.V)                                   # all pairs (k, k + q)
    Vc, offs = vstore.compress(L, cr.V)
    assert set(offs) == {k1 * L.nk + k2 for k1 in L.irre_list for k2 in range(L.nk)}
    assert Vc.size < 0.35 * cr.V.size
    nt_max = nts // 2
    for rotate_v in (False, True):   # rotate each contribution, or the stored V block once per (k, q)
        P0s, off_block = vstore.p0_from_stored_pairs(L, ns, nts, Gf, Vc, offs, cr.p0_transports,
                                                     rotate_v=rotate_v)
        d = 0.0
        for iq, q in enumerate(L.irre_list):
            base, qs = nts * L.qaux_slice_offsets_irre[iq], L.qaux_slice_sizes[q]
            d = max(d, float(np.abs(P0[base:base + nt_max * qs] - P0s[base:base + nt_max * qs]).max()))
        assert d < bound and off_block < 1e-13 and np.abs(P0).max() > 0.5


def test_unstored_pairs_are_never_read():
    spec = CONFIGS["C1"]
    cr = O.make_orbital_crystal(spec, rotate=True, transports=True)
    L = cr.layout
    Vc, offs = vstore.compress(L, cr.V)
    k_not_irr = next(k for k in range(L.nk) if k not in set(int(x) for x in L.irre_list))
    with pytest.raises(KeyError):
        vstore._dense_pair(L, Vc, offs, k_not_irr, 0)

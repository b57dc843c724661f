"""The C oracle against an independent numpy restatement on a rotated crystal
(irreducible k only stored: exercises orep/auxrep rotations and conj)."""
import numpy as np
import pytest

from _helpers import crystal
from oracle import Oracle


def _rot_numpy(L, ns, nts, G_irr, blocks_of, rep, slice_sz, slice_off_irre, off_of, per_t, batch):
    """Restatement of the iBZ -> BZ rotation (cugw_routines_block.cu:134-186)."""
    out = {}
    for k in range(L.nk):
        ck = L.conj_index[k]
        ick = L.irre_index[ck]
        kk = L.irre_list[ick]
        res = np.zeros((batch, slice_sz[k]), np.complex128)
        for b in range(batch):
            src = G_irr[b * per_t + slice_off_irre[ick]: b * per_t + slice_off_irre[ick] + slice_sz[kk]] \
                if per_t else None
            if L.index[ck] == ck:
                res[b] = src
            else:
                for ib, (i1, i2) in enumerate(blocks_of[ck]):
                    m, n = rep[1][ck][i1], rep[1][kk][i2]
                    O = rep[0](ck, ib).reshape(m, n)
                    X = src[off_of[kk][i2]: off_of[kk][i2] + n * n].reshape(n, n)
                    res[b, off_of[ck][i1]: off_of[ck][i1] + m * m] = (O @ X @ O.conj().T).ravel()
            if k != ck:
                res[b] = res[b].conj()
        out[k] = res
    return out


@pytest.mark.parametrize("physical", [False, True])
def test_rotated_p0_sigma_against_numpy(physical):
    cr, tr = crystal("C1", physical=physical)
    L, ns, nts = cr.layout, cr.ns, tr.nts
    assert L.ink < L.nk
    orc = Oracle(L, ns, nts)
    zero = np.zeros(nts * ns * L.flat_ao_size, np.complex128)
    G, _ = orc.dyson(zero, cr.F, cr.S, tr, cr.mu)
    Gf = orc.rotate_G(G)
    # numpy rotation of G
    orep = lambda ck, ib: L.orep[L.korep_slice_offsets[ck] + L.orep_offsets[ck][ib]:][:L.ao_sizes[ck][L.orep_irreps[ck][ib][0]] * L.ao_sizes[L.irre_list[L.irre_index[ck]]][L.orep_irreps[ck][ib][1]]]  # noqa: E731
    Gn = _rot_numpy(L, ns, nts, G, L.orep_irreps, (orep, L.ao_sizes), L.kao_slice_sizes, L.kao_slice_offsets_irre,
                    L.ao_offsets, L.flat_ao_size, nts * ns)
    for k in range(L.nk):
        o = L.kao_slice_offsets[k] * ns * nts
        assert np.abs(Gf[o:o + nts * ns * L.kao_slice_sizes[k]] - Gn[k].ravel()).max() < 1e-13

    # P0 via einsum for a few tau
    P0 = orc.p0(Gf, cr.V, nt_max=3)
    pref = -1.0 / L.nk * (2.0 if ns == 1 else 1.0)

    def gblk(k, t, s, ib):
        b = L.ao_sizes[k][ib]
        o = L.kao_slice_offsets[k] * ns * nts + (t * ns + s) * L.kao_slice_sizes[k] + L.ao_offsets[k][ib]
        return Gf[o:o + b * b].reshape(b, b)

    for iqr, q in enumerate(L.irre_list):
        for t in range(3):
            ref = np.zeros(L.qaux_slice_sizes[q], np.complex128)
            for k1 in range(L.nk):
                k2 = L.mom_cons(k1, 0, q)
                p = k1 * L.nk + k2
                for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
                    qb, b1, b2 = L.aux_sizes[q][iq], L.ao_sizes[k1][i1], L.ao_sizes[k2][i2]
                    o = L.kpair_slice_offsets[p] + L.tensor_offsets[p][b]
                    Vb = cr.V[o:o + qb * b1 * b2].reshape(qb, b1, b2)
                    po = L.aux_offsets[q][iq]
                    for s in range(ns):
                        blk = np.einsum("tp,Qpm,Ptn,mn->QP", gblk(k1, nts - 1 - t, s, i1), Vb, Vb.conj(),
                                        gblk(k2, t, s, i2))
                        ref[po:po + qb * qb] += pref * blk.ravel()
            got = P0[nts * L.qaux_slice_offsets_irre[iqr] + t * L.qaux_slice_sizes[q]:][:L.qaux_slice_sizes[q]]
            assert np.abs(got - ref).max() < 1e-12

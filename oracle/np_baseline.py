"""numpy/BLAS restatement of the P0 and Sigma contractions (the CPU baseline's
second figure).

TEST INFRASTRUCTURE ONLY: timed by bench.py's CPU-baseline leg and checked
against the C oracle by tests/test_np_baseline.py.  The product package never
imports it.

Same loop nests as the C oracle (SymmetryMBPT/src/cpu_ref/gw_block.cpp:6-158)
with the tau loop moved innermost into batched matrix products, as the
reference's Eigen GEMMs would run them with a BLAS: per V block and spin,
  P0:    X1[tau] = G1(beta - tau) V_(p, (Q,m)),  X2[tau] = conj(V)_((P,t), n) G2(tau)^T,
         P0[tau][Q][P] += X1[tau]_(Q, (t,m)) X2[tau]_((t,m), P)       (gw_block.cpp:57-74)
  Sigma: Y1[tau] = V_((Q,i), m) G2(tau),  Y2[tau] = Y1[tau]_(Q, (i,n))^T P~(q, tau),
         Sigma[tau] += Y2[tau]_(i, (n,P)) conj(V)_((n,P), j)          (gw_block.cpp:134-150)
Inputs are the oracle's full-BZ G and P~ (Oracle.rotate_G / rotate_P).
"""
from __future__ import annotations

import numpy as np


def _gk(L, G_full, ns, nts, k):
    """[t][s][kslice] view of G^k in the full-BZ buffer."""
    o = L.kao_slice_offsets[k] * ns * nts
    return G_full[o:o + nts * ns * L.kao_slice_sizes[k]].reshape(nts, ns, L.kao_slice_sizes[k])


def p0(L, ns, nts, G_full, V, nt_max=None):
    """P0 [q_irr][t][qslice] for t < nt_max (default nts / 2), prefactor applied."""
    nt = nts // 2 if nt_max is None else nt_max
    pref = -1.0 / L.nk * (2.0 if ns == 1 else 1.0)
    out = np.zeros(nts * L.flat_aux_size, np.complex128)
    for iqr, q in enumerate(L.irre_list):
        Pq = np.zeros((nt, L.qaux_slice_sizes[q]), np.complex128)
        for k1 in range(L.nk):
            k2 = L.mom_cons(k1, 0, q)  # k2 = k1 + q
            p = k1 * L.nk + k2
            g1, g2 = _gk(L, G_full, ns, nts, k1), _gk(L, G_full, ns, nts, k2)
            for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
                qb, b1, b2 = L.aux_sizes[q][iq], L.ao_sizes[k1][i1], L.ao_sizes[k2][i2]
                o = L.kpair_slice_offsets[p] + L.tensor_offsets[p][b]
                Vb = V[o:o + qb * b1 * b2].reshape(qb, b1, b2)
                Vp = Vb.transpose(1, 0, 2).reshape(b1, qb * b2)        # [p][(Q,m)]
                Vc = Vb.conj().reshape(qb * b1, b2)                    # [(P,t)][n]
                oa, ob, po = L.ao_offsets[k1][i1], L.ao_offsets[k2][i2], L.aux_offsets[q][iq]
                for s in range(ns):
                    G1 = g1[nts - 1 - np.arange(nt), s, oa:oa + b1 * b1].reshape(nt, b1, b1)
                    G2 = g2[:nt, s, ob:ob + b2 * b2].reshape(nt, b2, b2)
                    X1 = (G1 @ Vp).reshape(nt, b1, qb, b2).transpose(0, 2, 1, 3).reshape(nt, qb, b1 * b2)
                    X2 = (Vc @ G2.transpose(0, 2, 1)).reshape(nt, qb, b1 * b2)
                    Pq[:, po:po + qb * qb] += (X1 @ X2.transpose(0, 2, 1)).reshape(nt, qb * qb)
        o = nts * L.qaux_slice_offsets_irre[iqr]
        out[o:o + nt * L.qaux_slice_sizes[q]] = pref * Pq.ravel()
    return out


def sigma(L, ns, nts, G_full, P_full, V, nt_max=None):
    """Sigma [t][s][flat_ao] for t < nt_max (default nts) from the full-BZ G and P~."""
    nt = nts if nt_max is None else nt_max
    out = np.zeros((nts, ns, L.flat_ao_size), np.complex128)
    for ik, k1 in enumerate(L.irre_list):
        ko = L.kao_slice_offsets_irre[ik]
        for q in range(L.nk):
            k2 = L.mom_cons(k1, q, 0)  # k2 = k1 - q
            p = k1 * L.nk + k2
            g2 = _gk(L, G_full, ns, nts, k2)
            po = nts * L.qaux_slice_offsets[q]
            Pt = P_full[po:po + nts * L.qaux_slice_sizes[q]].reshape(nts, L.qaux_slice_sizes[q])[:nt]
            for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
                qb, b1, b2 = L.aux_sizes[q][iq], L.ao_sizes[k1][i1], L.ao_sizes[k2][i2]
                o = L.kpair_slice_offsets[p] + L.tensor_offsets[p][b]
                Vb = V[o:o + qb * b1 * b2].reshape(qb, b1, b2)
                VV = Vb.conj().transpose(2, 0, 1).reshape(b2 * qb, b1)  # [(n,P)][j]
                aq = L.aux_offsets[q][iq]
                PQP = Pt[:, aq:aq + qb * qb].reshape(nt, qb, qb)
                oa, ob = L.ao_offsets[k1][i1], L.ao_offsets[k2][i2]
                for s in range(ns):
                    G2 = g2[:nt, s, ob:ob + b2 * b2].reshape(nt, b2, b2)
                    Y1 = (Vb.reshape(qb * b1, b2) @ G2).reshape(nt, qb, b1 * b2)
                    Y2 = Y1.transpose(0, 2, 1) @ PQP                                 # [t][(i,n)][P]
                    S = Y2.reshape(nt, b1, b2 * qb) @ VV                             # [t][i][j]
                    out[:nt, s, ko + oa:ko + oa + b1 * b1] += S.reshape(nt, b1 * b1)
    out *= -1.0 / L.nk
    return out.ravel()

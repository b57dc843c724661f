"""V stored only for the pairs whose first k is irreducible, and P0 re-indexed
through the group so that it reads no other pair.

The reference stores V(k1, k2) for all nk^2 pairs
(``SymmetryMBPT/include/common/df_integral_block_t.h:94-98``) because its P0
loop reads V(k, k + q) for every k of the mesh at an irreducible q
(``SymmetryMBPT/src/cuda/cugw_routines_block.cu:279-290``,
``src/cpu_ref/gw_block.cpp:19-79``); Sigma reads only V(k_irr, k2).  With
the contribution of one k to P0,

    c(k, q)_QP = sum_{t', p, m, n} G^k(beta - tau)_{t'p} V^Q_{pm}(k, k + q) G^{k+q}(tau)_{mn} conj(V^P_{t'n}(k, k + q)),

covariance gives c(g k_r, q) = A c(k_r, q') A^H for q' = g^-1 q and the aux
transport A = Y(q)^H D_aux(g, q') Y(q') between the adapted bases, and time
reversal c(-k, q) = conj(c(k, -q)).  So

    P0(q_irr) = pref * sum_{k_r} sum_{k in the star of k_r} A_k c(k_r, q'_k) A_k^H

reads V(k_r, k_r + q') only.  The transports are dense naux x naux
matrices per (k, irreducible q): they mix the rows of an irrep, which the
reference's rotation data (one block-diagonal auxrep per q, taking q_irr to
q) cannot express; ``orbitals.make_orbital_crystal(..., transports=True)``
builds them from the group.  This module is the host restatement of the
scheme (numpy), checked against the oracle's all-pairs loop; the GPU
engine keeps all pairs resident.
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np

from .layout import BlockLayout


def stored_pairs(layout: BlockLayout) -> np.ndarray:
    """Pair indices k1 * nk + k2 with k1 irreducible (every k2)."""
    nk = layout.nk
    return np.array([k1 * nk + k2 for k1 in sorted(int(k) for k in layout.irre_list) for k2 in range(nk)],
                    dtype=np.int64)


def compress(layout: BlockLayout, V: np.ndarray) -> Tuple[np.ndarray, Dict[int, int]]:
    """The stored pairs' slices of the flat V, concatenated, and each stored
    pair's offset in the result."""
    out, offs, acc = [], {}, 0
    for p in stored_pairs(layout):
        o, n = int(layout.kpair_slice_offsets[p]), int(layout.kpair_slice_sizes[p])
        out.append(V[o:o + n])
        offs[int(p)] = acc
        acc += n
    return (np.concatenate(out) if out else np.zeros(0, np.complex128)), offs


def _dense_pair(layout: BlockLayout, Vc: np.ndarray, offs: Dict[int, int], k1: int, k2: int) -> np.ndarray:
    """V(k1, k2) as a dense (naux, nao, nao) array in the adapted bases (stored pairs only)."""
    nk = layout.nk
    p = k1 * nk + k2
    if p not in offs:
        raise KeyError(f"pair ({k1}, {k2}) is not stored")
    q = layout.pair_q(k1, k2)
    aq = np.concatenate([[0], np.cumsum(layout.aux_sizes[q])])
    a1 = np.concatenate([[0], np.cumsum(layout.ao_sizes[k1])])
    a2 = np.concatenate([[0], np.cumsum(layout.ao_sizes[k2])])
    out = np.zeros((aq[-1], a1[-1], a2[-1]), np.complex128)
    base = offs[p]
    for b, (iq, i1, i2) in enumerate(layout.tensor_irreps[p]):
        n = (aq[iq + 1] - aq[iq]) * (a1[i1 + 1] - a1[i1]) * (a2[i2 + 1] - a2[i2])
        o = base + int(layout.tensor_offsets[p][b])
        out[aq[iq]:aq[iq + 1], a1[i1]:a1[i1 + 1], a2[i2]:a2[i2 + 1]] = \
            Vc[o:o + n].reshape(aq[iq + 1] - aq[iq], a1[i1 + 1] - a1[i1], a2[i2 + 1] - a2[i2])
    return out


def _dense_G(layout: BlockLayout, G_full: np.ndarray, ns: int, nts: int, k: int) -> np.ndarray:
    """G^k as dense (nts, ns, nao, nao) from the full-mesh G of the rotation step."""
    sz = int(layout.kao_slice_sizes[k])
    g = G_full[int(layout.kao_slice_offsets[k]) * ns * nts:][:nts * ns * sz].reshape(nts, ns, sz)
    a = np.concatenate([[0], np.cumsum(layout.ao_sizes[k])])
    out = np.zeros((nts, ns, a[-1], a[-1]), np.complex128)
    for b in range(len(a) - 1):
        n = a[b + 1] - a[b]
        o = int(layout.ao_offsets[k][b])
        out[:, :, a[b]:a[b + 1], a[b]:a[b + 1]] = g[:, :, o:o + n * n].reshape(nts, ns, n, n)
    return out


def _contribution(V: np.ndarray, G1: np.ndarray, G2: np.ndarray, nts: int, ns: int, nt_max: int) -> np.ndarray:
    """c[tau]_QP = sum_s sum G1(beta - tau)_{t'p} V^Q_{pm} G2(tau)_{mn} conj(V^P_{t'n})
    (the oracle's loop body, gw_block.cpp:57-74) for dense V (naux, n1, n2)."""
    c = np.zeros((nt_max, V.shape[0], V.shape[0]), np.complex128)
    for t in range(nt_max):
        for s in range(ns):
            X1 = np.einsum("tp,Qpm->Qtm", G1[nts - 1 - t, s], V, optimize=True)
            X2 = np.einsum("mn,Ptn->Ptm", G2[t, s], V.conj(), optimize=True)
            c[t] += np.einsum("Qtm,Ptm->QP", X1, X2, optimize=True)
    return c


def p0_from_stored_pairs(layout: BlockLayout, ns: int, nts: int, G_full: np.ndarray, Vc: np.ndarray,
                         offs: Dict[int, int], transports: Dict[Tuple[int, int], Tuple[int, int, np.ndarray]],
                         nt_max: int = None, rotate_v: bool = False) -> Tuple[np.ndarray, float]:
    """P0 at the irreducible q for tau < nt_max, in the oracle's layout
    ([ink][nts][qslice]), reading only stored pairs.  transports[(k, q)] =
    (k_r, q', A) for every k of the mesh and irreducible q (the time-reversal
    partners -k map to (k_r, q', A) of k with conjugation, flagged by a
    negative k_r - 1).  rotate_v: apply A to the stored block's aux index
    (A V, once per (k, q), tau-independent) and contract that, instead of
    rotating the contribution (A c A^H for every tau); the same P0.  Also
    returns the largest entry of P0 outside its diagonal blocks (zero by
    symmetry)."""
    nk = layout.nk
    nt_max = nts // 2 if nt_max is None else nt_max
    pref = -1.0 / nk * (2.0 if ns == 1 else 1.0)
    Gd = {}

    def G(k):
        if k not in Gd:
            Gd[k] = _dense_G(layout, G_full, ns, nts, k)
        return Gd[k]

    out = np.zeros(nts * layout.flat_aux_size, np.complex128)
    off_block = 0.0
    cache = {}
    for iq, q in enumerate(int(x) for x in layout.irre_list):
        na = int(sum(layout.aux_sizes[q]))
        acc = np.zeros((nt_max, na, na), np.complex128)
        for k in range(nk):
            kr, qp, A = transports[(k, q)]
            conj = kr < 0
            kr = -kr - 1 if conj else kr
            k2 = layout.mom_cons(kr, 0, qp)                        # k_r + q'
            if rotate_v:                                           # c(A V) = A c(V) A^H
                V = _dense_pair(layout, Vc, offs, kr, k2)
                Ar = A.conj() if conj else A                       # A of the partner -k (see above)
                c = _contribution(np.tensordot(Ar, V, 1), G(kr), G(k2), nts, ns, nt_max)
                acc += c.conj() if conj else c
                continue
            key = (kr, qp)
            if key not in cache:
                cache[key] = _contribution(_dense_pair(layout, Vc, offs, kr, k2), G(kr), G(k2), nts, ns, nt_max)
            c = cache[key].conj() if conj else cache[key]
            acc += A[None] @ c @ A.conj().T[None]
        acc *= pref
        a = np.concatenate([[0], np.cumsum(layout.aux_sizes[q])])
        mask = np.ones((na, na), dtype=bool)
        base = nts * int(layout.qaux_slice_offsets_irre[iq])
        qsz = int(layout.qaux_slice_sizes[q])
        for b in range(len(a) - 1):
            n = a[b + 1] - a[b]
            mask[a[b]:a[b + 1], a[b]:a[b + 1]] = False
            o = int(layout.aux_offsets[q][b])
            for t in range(nt_max):
                out[base + t * qsz + o:base + t * qsz + o + n * n] = acc[t, a[b]:a[b + 1], a[b]:a[b + 1]].ravel()
        if mask.any():
            off_block = max(off_block, float(np.abs(acc[:, mask]).max()))
    return out, off_block

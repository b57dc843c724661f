"""Irrep-blocked ("flat block") tensor layout.

This is the layout contract of SymmetryMBPT's ``symmetry_utils_t``
(``SymmetryMBPT/include/common/symmetry_utils.h:17-315``,
``SymmetryMBPT/src/common/symmetry_utils.cpp:6-341``):

* G, F, S, Sigma: per k point a list of square irrep blocks (``ao_sizes``),
  each stored row-major at ``ao_offsets`` inside the k slice; slices of the
  irreducible k points are concatenated (``kao_slice_offsets_irre``).
* P0 / P: the same per q point in the auxiliary space (``aux_sizes``).
* V: per stored k pair ``k1*nk + k2`` a slice of non-zero blocks, each
  ``[q_b][k1_b][k2_b]`` row-major, listed by ``tensor_irreps`` (iq, ik1, ik2)
  at ``tensor_offsets`` (``scripts/common/blk_utils.py:227-282``).
* Rotations iBZ -> BZ: block-sparse ``orep``/``auxrep`` per k with
  (row-block, column-block) pairs ``orep_irreps`` at ``orep_offsets``.

The class holds plain numpy arrays and produces the flattened (CSR-style)
arrays handed to the C ABI (``include/gwgb.h``, ``gwgb_layout``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np


def _offsets(sizes, square=True):
    out = np.zeros(len(sizes), dtype=np.int64)
    acc = 0
    for i, s in enumerate(sizes):
        out[i] = acc
        acc += int(s) * int(s) if square else int(s)
    return out, acc


def wrap_1stbz(k: np.ndarray) -> np.ndarray:
    """Fold reduced coordinates into [0, 1) (``symmetry_utils.h:300-314``)."""
    kk = np.array(k, dtype=np.float64)
    for j in range(kk.shape[0]):
        while kk[j] - 9.9999999999e-1 > 0.0:
            kk[j] -= 1.0
        if abs(kk[j]) < 1e-9:
            kk[j] = 0.0
        while kk[j] < 0:
            kk[j] += 1.0
    return kk


def find_pos(k: np.ndarray, mesh: np.ndarray) -> int:
    """Index of ``k`` in ``mesh`` (``symmetry_utils.h:285-298``)."""
    d = np.abs(mesh - k[None, :]).max(axis=1)
    hit = np.nonzero(d < 1e-9)[0]
    if hit.size == 0:
        raise ValueError(f"k point {k} has not been found in the mesh")
    return int(hit[0])


def momentum_tables(kmesh: np.ndarray):
    """``q_ind_``/``q_ind2_`` exactly as ``symmetry_utils.cpp:22-39`` builds them."""
    nk = kmesh.shape[0]
    qmesh = np.array([wrap_1stbz(kmesh[0] - kmesh[j]) for j in range(nk)])
    q_ind = np.zeros((nk, nk), dtype=np.int32)
    q_ind2 = np.zeros((nk, nk), dtype=np.int32)
    for i in range(nk):
        for j in range(nk):
            q = find_pos(wrap_1stbz(kmesh[i] - kmesh[j]), qmesh)
            q_ind[j, q] = i
            q_ind2[i, j] = q
    return q_ind, q_ind2


@dataclass
class BlockLayout:
    nk: int
    kmesh: np.ndarray
    ao_sizes: List[np.ndarray]           # per full-BZ k
    aux_sizes: List[np.ndarray]          # per full-BZ q
    tensor_irreps: List[np.ndarray]      # per pair k1*nk+k2, (nb, 3)
    irre_list: np.ndarray                # ink, full-BZ index of stored k
    index: np.ndarray                    # nk, irreducible representative (full-BZ index)
    irre_index: np.ndarray               # nk, position of representative in irre_list
    conj_index: np.ndarray               # nk
    orep: Optional[np.ndarray] = None    # flat complex rotation blocks (all k)
    orep_irreps: Optional[List[np.ndarray]] = None
    auxrep: Optional[np.ndarray] = None
    auxrep_irreps: Optional[List[np.ndarray]] = None
    ao_block_offsets: Optional[List[np.ndarray]] = None
    aux_block_offsets: Optional[List[np.ndarray]] = None
    # derived
    q_ind: np.ndarray = field(init=False)
    q_ind2: np.ndarray = field(init=False)

    def __post_init__(self):
        self.kmesh = np.asarray(self.kmesh, dtype=np.float64)
        self.ao_sizes = [np.asarray(a, dtype=np.int32) for a in self.ao_sizes]
        self.aux_sizes = [np.asarray(a, dtype=np.int32) for a in self.aux_sizes]
        self.tensor_irreps = [np.asarray(a, dtype=np.int32).reshape(-1, 3) for a in self.tensor_irreps]
        self.irre_list = np.asarray(self.irre_list, dtype=np.int32)
        self.index = np.asarray(self.index, dtype=np.int32)
        self.irre_index = np.asarray(self.irre_index, dtype=np.int32)
        self.conj_index = np.asarray(self.conj_index, dtype=np.int32)
        nk = self.nk
        assert len(self.ao_sizes) == nk and len(self.aux_sizes) == nk
        assert len(self.tensor_irreps) == nk * nk, "V must be stored for all nk^2 pairs"
        self.q_ind, self.q_ind2 = momentum_tables(self.kmesh)
        self.ao_offsets = [_offsets(s)[0] for s in self.ao_sizes]
        self.aux_offsets = [_offsets(s)[0] for s in self.aux_sizes]
        self.kao_slice_sizes = np.array([_offsets(s)[1] for s in self.ao_sizes], dtype=np.int64)
        self.qaux_slice_sizes = np.array([_offsets(s)[1] for s in self.aux_sizes], dtype=np.int64)
        self.kao_slice_offsets = np.concatenate([[0], np.cumsum(self.kao_slice_sizes)[:-1]]).astype(np.int64)
        self.qaux_slice_offsets = np.concatenate([[0], np.cumsum(self.qaux_slice_sizes)[:-1]]).astype(np.int64)
        if self.ao_block_offsets is None:
            self.ao_block_offsets = [np.concatenate([[0], np.cumsum(s)[:-1]]).astype(np.int32) for s in self.ao_sizes]
        if self.aux_block_offsets is None:
            self.aux_block_offsets = [np.concatenate([[0], np.cumsum(s)[:-1]]).astype(np.int32) for s in self.aux_sizes]
        # iBZ re-packing (symmetry_utils.cpp:174-191)
        ink = len(self.irre_list)
        self.kao_slice_sizes_irre = np.array([self.kao_slice_sizes[k] for k in self.irre_list], dtype=np.int64)
        self.qaux_slice_sizes_irre = np.array([self.qaux_slice_sizes[k] for k in self.irre_list], dtype=np.int64)
        self.kao_slice_offsets_irre = np.concatenate([[0], np.cumsum(self.kao_slice_sizes_irre)[:-1]]).astype(np.int64)
        self.qaux_slice_offsets_irre = np.concatenate([[0], np.cumsum(self.qaux_slice_sizes_irre)[:-1]]).astype(np.int64)
        # V pair slices and block offsets
        self.tensor_offsets = []
        sizes = np.zeros(nk * nk, dtype=np.int64)
        for p in range(nk * nk):
            k1, k2 = divmod(p, nk)
            ti = self.tensor_irreps[p]
            offs = np.zeros(len(ti), dtype=np.int64)
            acc = 0
            for b, (iq, i1, i2) in enumerate(ti):
                offs[b] = acc
                q = self.pair_q(k1, k2)
                acc += int(self.aux_sizes[q][iq]) * int(self.ao_sizes[k1][i1]) * int(self.ao_sizes[k2][i2])
            self.tensor_offsets.append(offs)
            sizes[p] = acc
        self.kpair_slice_sizes = sizes
        self.kpair_slice_offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
        # rotations: identity when none given (symmetry_utils.cpp:263-307)
        if self.orep is None:
            self.orep, self.orep_irreps = self._identity_rep(self.ao_sizes)
        if self.auxrep is None:
            self.auxrep, self.auxrep_irreps = self._identity_rep(self.aux_sizes)
        self.orep_irreps = [np.asarray(a, dtype=np.int32).reshape(-1, 2) for a in self.orep_irreps]
        self.auxrep_irreps = [np.asarray(a, dtype=np.int32).reshape(-1, 2) for a in self.auxrep_irreps]
        self.orep_offsets, self.korep_slice_offsets, self.korep_slice_sizes = self._rep_offsets(
            self.orep_irreps, self.ao_sizes)
        self.auxrep_offsets, self.kauxrep_slice_offsets, self.kauxrep_slice_sizes = self._rep_offsets(
            self.auxrep_irreps, self.aux_sizes)

    # -- helpers ---------------------------------------------------------- #
    def pair_q(self, k1: int, k2: int) -> int:
        """The q whose aux blocks label V(k1, k2).

        The reference uses V(k1, k1+q) in P0 (``gw_block.cpp:23-24``) and
        V(k1, k1-q) in Sigma (``gw_block.cpp:101-102``) with the same
        ``aux_sizes(q)``; the layout therefore requires aux_sizes(q) ==
        aux_sizes(-q).  Here q is taken as k2 - k1.
        """
        return int(self.mom_cons(k2, k1, 0))

    def _identity_rep(self, sizes):
        flat = []
        irreps = []
        for s in sizes:
            blocks = [np.eye(int(b), dtype=np.complex128).ravel() for b in s]
            flat.append(np.concatenate(blocks) if blocks else np.zeros(0, np.complex128))
            irreps.append(np.stack([np.arange(len(s)), np.arange(len(s))], axis=1).astype(np.int32))
        return np.concatenate(flat), irreps

    def _rep_offsets(self, irreps, sizes):
        offs = []
        slice_sizes = np.zeros(self.nk, dtype=np.int64)
        for k in range(self.nk):
            ck = self.conj_index[k]
            ik = self.irre_index[ck]
            kk = self.irre_list[ik]
            o = np.zeros(len(irreps[k]), dtype=np.int64)
            acc = 0
            for b, (i1, i2) in enumerate(irreps[k]):
                o[b] = acc
                acc += int(sizes[ck][i1]) * int(sizes[kk][i2])
            offs.append(o)
            slice_sizes[k] = acc
        slice_offsets = np.concatenate([[0], np.cumsum(slice_sizes)[:-1]]).astype(np.int64)
        return offs, slice_offsets, slice_sizes

    @property
    def ink(self) -> int:
        return len(self.irre_list)

    def mom_cons(self, i: int, j: int, k: int) -> int:
        """k_i - k_j + k_k on the mesh (``symmetry_utils.cpp:337-341``)."""
        return int(self.q_ind[k, self.q_ind2[i, j]])

    @property
    def flat_ao_size(self) -> int:
        return int(self.kao_slice_sizes_irre.sum())

    @property
    def flat_aux_size(self) -> int:
        return int(self.qaux_slice_sizes_irre.sum())

    @property
    def flat_ao_size_full(self) -> int:
        return int(self.kao_slice_sizes.sum())

    @property
    def flat_aux_size_full(self) -> int:
        return int(self.qaux_slice_sizes.sum())

    @property
    def flat_V_size(self) -> int:
        return int(self.kpair_slice_sizes.sum())

    @property
    def nao(self) -> int:
        return int(self.ao_sizes[0].sum())

    @property
    def naux(self) -> int:
        return int(self.aux_sizes[0].sum())

    def max_block(self) -> int:
        return int(max(max(int(s.max()) for s in self.ao_sizes), max(int(s.max()) for s in self.aux_sizes)))

    # -- C ABI marshalling -------------------------------------------------- #
    def to_c(self):
        """Return (gwgb_layout struct, keep-alive list) for the C ABI."""
        from ._abi import GwgbLayout
        keep = []

        def arr(a, dt):
            a = np.ascontiguousarray(np.asarray(a), dtype=dt)
            keep.append(a)
            return a.ctypes.data

        def csr(lists, dt):
            ptr = np.zeros(len(lists) + 1, dtype=np.int32)
            for i, l in enumerate(lists):
                ptr[i + 1] = ptr[i] + len(l)
            cat = np.concatenate([np.asarray(l).reshape(-1) for l in lists]) if lists else np.zeros(0)
            return ptr, cat.astype(dt)

        L = GwgbLayout()
        L.nk = self.nk
        L.ink = self.ink
        L.irre_list = arr(self.irre_list, np.int32)
        L.index = arr(self.index, np.int32)
        L.irre_index = arr(self.irre_index, np.int32)
        L.conj_index = arr(self.conj_index, np.int32)
        L.q_ind = arr(self.q_ind, np.int32)
        L.q_ind2 = arr(self.q_ind2, np.int32)
        p, c = csr(self.ao_sizes, np.int32)
        L.ao_block_ptr = arr(p, np.int32)
        L.ao_sizes = arr(c, np.int32)
        p, c = csr(self.aux_sizes, np.int32)
        L.aux_block_ptr = arr(p, np.int32)
        L.aux_sizes = arr(c, np.int32)
        p, c = csr(self.tensor_irreps, np.int32)
        L.kpair_block_ptr = arr(p, np.int32)
        L.tensor_irreps = arr(c, np.int32)
        p, c = csr(self.orep_irreps, np.int32)
        L.orep_block_ptr = arr(p, np.int32)
        L.orep_irreps = arr(c, np.int32)
        p, c = csr(self.auxrep_irreps, np.int32)
        L.auxrep_block_ptr = arr(p, np.int32)
        L.auxrep_irreps = arr(c, np.int32)
        return L, keep

    # -- block <-> dense helpers (block_utils.cpp:6-143) -------------------- #
    def G_flat_to_block(self, G_flat: np.ndarray) -> np.ndarray:
        """(..., flat_ao) over the stored k points -> (..., ink, nao, nao)."""
        nao = self.nao
        out = np.zeros(G_flat.shape[:-1] + (self.ink, nao, nao), dtype=np.complex128)
        for ik, k in enumerate(self.irre_list):
            base = self.kao_slice_offsets_irre[ik]
            for b, s in enumerate(self.ao_sizes[k]):
                o = base + self.ao_offsets[k][b]
                bo = self.ao_block_offsets[k][b]
                out[..., ik, bo:bo + s, bo:bo + s] = G_flat[..., o:o + s * s].reshape(G_flat.shape[:-1] + (s, s))
        return out

    def P_flat_to_block(self, P_flat: np.ndarray) -> np.ndarray:
        """(..., flat_aux) over the stored q points -> (..., ink, naux, naux)."""
        naux = self.naux
        out = np.zeros(P_flat.shape[:-1] + (self.ink, naux, naux), dtype=np.complex128)
        for iq, q in enumerate(self.irre_list):
            base = self.qaux_slice_offsets_irre[iq]
            for b, s in enumerate(self.aux_sizes[q]):
                o = base + self.aux_offsets[q][b]
                bo = self.aux_block_offsets[q][b]
                out[..., iq, bo:bo + s, bo:bo + s] = P_flat[..., o:o + s * s].reshape(P_flat.shape[:-1] + (s, s))
        return out

    def G_block_to_flat(self, G_blk: np.ndarray) -> np.ndarray:
        out = np.zeros(G_blk.shape[:-3] + (self.flat_ao_size,), dtype=np.complex128)
        for ik, k in enumerate(self.irre_list):
            base = self.kao_slice_offsets_irre[ik]
            for b, s in enumerate(self.ao_sizes[k]):
                o = base + self.ao_offsets[k][b]
                bo = self.ao_block_offsets[k][b]
                out[..., o:o + s * s] = G_blk[..., ik, bo:bo + s, bo:bo + s].reshape(G_blk.shape[:-3] + (s * s,))
        return out

    def P_block_to_flat(self, P_blk: np.ndarray) -> np.ndarray:
        out = np.zeros(P_blk.shape[:-3] + (self.flat_aux_size,), dtype=np.complex128)
        for iq, q in enumerate(self.irre_list):
            base = self.qaux_slice_offsets_irre[iq]
            for b, s in enumerate(self.aux_sizes[q]):
                o = base + self.aux_offsets[q][b]
                bo = self.aux_block_offsets[q][b]
                out[..., o:o + s * s] = P_blk[..., iq, bo:bo + s, bo:bo + s].reshape(P_blk.shape[:-3] + (s * s,))
        return out


def layout_from_reference_files(symmetry_info_h5: str, meta_h5: str) -> BlockLayout:
    """Build the layout from the reference's ``symmetry_info.h5`` + ``df_int/meta.h5``.

    Follows ``symmetry_utils.cpp:15-159`` for the no-rotation case
    (``rotate=false``: ink = nk, identity reps); offsets stored in the file
    are checked against the ones this module derives.
    """
    from .h5lite import H5File
    meta = H5File(meta_h5)
    kmesh = meta["grid/k_mesh_scaled"]
    nk = kmesh.shape[0]
    npairs = int(meta["grid/num_kpair_stored"])
    if npairs != nk * nk:
        raise ValueError(f"V must be stored for all k pairs ({npairs} != {nk * nk})")
    f = H5File(symmetry_info_h5)
    ao_sizes = [f[f"block/ao_sizes/{k}"] for k in range(nk)]
    aux_sizes = [f[f"block/aux_sizes/{k}"] for k in range(nk)]
    ti = [f[f"block/tensor_irreps/{p}"] for p in range(npairs)]
    lay = BlockLayout(
        nk=nk, kmesh=kmesh, ao_sizes=ao_sizes, aux_sizes=aux_sizes, tensor_irreps=ti,
        irre_list=np.arange(nk), index=np.arange(nk), irre_index=np.arange(nk),
        conj_index=np.arange(nk),
        ao_block_offsets=[f[f"block/ao_block_offsets/{k}"] for k in range(nk)],
        aux_block_offsets=[f[f"block/aux_block_offsets/{k}"] for k in range(nk)],
    )
    # cross-check the derived offsets with the stored ones
    for k in range(nk):
        assert np.array_equal(lay.ao_offsets[k], f[f"block/ao_offsets/{k}"].astype(np.int64))
        assert np.array_equal(lay.aux_offsets[k], f[f"block/aux_offsets/{k}"].astype(np.int64))
    assert np.array_equal(lay.kao_slice_offsets, f["block/kao_slice_offsets"].astype(np.int64))
    assert np.array_equal(lay.qaux_slice_offsets, f["block/qaux_slice_offsets"].astype(np.int64))
    assert np.array_equal(lay.kpair_slice_offsets, f["block/kpair_slice_offsets"].astype(np.int64))
    assert np.array_equal(lay.kpair_slice_sizes, f["block/kpair_slice_sizes"].astype(np.int64))
    for p in range(npairs):
        assert np.array_equal(lay.tensor_offsets[p], f[f"block/tensor_offsets/{p}"].astype(np.int64)), p
    return lay

"""Readers for the reference's input files (HDF5 via :mod:`h5lite`).

* ``input_flat.h5``: ``HF/{Fock-k, S-k, H-k}`` as [ns][flat_ao_full] complex
  (``SymmetryMBPT/src/scmbpt/sc_loop_block_t.cpp:64-109``).
* ``df_int/VQ_flat_0.h5``: dataset ``/0``, the whole flat V
  (``SymmetryMBPT/include/common/df_integral_block_t.h:38-59``).
* ``symmetry_info.h5`` + ``df_int/meta.h5``: the block layout
  (:func:`mbsymmetry_gb300.layout.layout_from_reference_files`).
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from .h5lite import H5File, as_complex
from .layout import BlockLayout, layout_from_reference_files


@dataclass
class OneBody:
    F: np.ndarray  # [ns][flat_ao] (stored k only)
    S: np.ndarray
    H: np.ndarray


def make_hermitian_kao(X: np.ndarray, layout: BlockLayout) -> np.ndarray:
    """Hermitise every block (``sc_loop_block_t.h:167-184``)."""
    X = X.copy()
    lead = X.shape[:-1]
    Xr = X.reshape(-1, X.shape[-1])
    for i in range(Xr.shape[0]):
        for ik, k in enumerate(layout.irre_list):
            base = layout.kao_slice_offsets_irre[ik]
            for b, s in enumerate(layout.ao_sizes[k]):
                o = base + layout.ao_offsets[k][b]
                m = Xr[i, o:o + s * s].reshape(s, s)
                Xr[i, o:o + s * s] = (0.5 * (m + m.conj().T)).ravel()
    return Xr.reshape(lead + (X.shape[-1],))


def onebody_from_full(F_full, S_full, H_full, layout: BlockLayout, Bz: float = 0.0) -> OneBody:
    """Select the stored k slices, apply the Bz shift and Hermitise
    (``sc_loop_block_t.cpp:78-103``)."""
    ns = F_full.shape[0]
    fa = layout.flat_ao_size
    F = np.zeros((ns, fa), np.complex128)
    S = np.zeros((ns, fa), np.complex128)
    H = np.zeros((ns, fa), np.complex128)
    for ik, k in enumerate(layout.irre_list):
        io, isz = layout.kao_slice_offsets_irre[ik], layout.kao_slice_sizes_irre[ik]
        ko = layout.kao_slice_offsets[k]
        F[:, io:io + isz] = F_full[:, ko:ko + isz]
        S[:, io:io + isz] = S_full[:, ko:ko + isz]
        H[:, io:io + isz] = H_full[:, ko:ko + isz]
    F = F - H
    for s in range(ns):
        H[s] += S[s] * Bz * (0.5 if s == 0 else -0.5)
    F = F + H
    return OneBody(make_hermitian_kao(F, layout), make_hermitian_kao(S, layout),
                   make_hermitian_kao(H, layout))


@dataclass
class ReferenceInputs:
    layout: BlockLayout
    V: np.ndarray
    onebody: OneBody
    ns: int


def load_reference_inputs(block_dir: str) -> ReferenceInputs:
    """Load a reference ``.../block`` directory (LiH fixture layout)."""
    lay = layout_from_reference_files(os.path.join(block_dir, "symmetry_info.h5"),
                                      os.path.join(block_dir, "df_int", "meta.h5"))
    V = H5File(os.path.join(block_dir, "df_int", "VQ_flat_0.h5"))["0"]
    V = V.reshape(-1, 2)
    V = np.ascontiguousarray(V[:, 0] + 1j * V[:, 1])
    assert V.size == lay.flat_V_size, (V.size, lay.flat_V_size)
    f = H5File(os.path.join(block_dir, "input_flat.h5"))
    F = as_complex(f["HF/Fock-k"])
    S = as_complex(f["HF/S-k"])
    H = as_complex(f["HF/H-k"])
    ob = onebody_from_full(F, S, H, lay)
    return ReferenceInputs(layout=lay, V=V, onebody=ob, ns=F.shape[0])

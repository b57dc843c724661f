"""tau <-> i omega transform matrices (intermediate representation, FP64, host).

Restates the matrix construction of SymmetryMBPT's ``transformer_t``
(``SymmetryMBPT/src/common/transformer_t.cpp:7-82``,
``SymmetryMBPT/include/common/transformer_t.h:16-41``): read the IR sampling
data (``fermi|bose/{nx, nw, uwl_re, uwl_im, uxl, ux1l, ux1l_minus, other_uxl,
xsample, wsample}``), pseudo-invert the sampling matrices and apply the
sqrt(beta) scalings, giving

* ``Tnt``    [nw][nts-2]    fermionic tau (interior) -> fermionic i omega,
* ``Ttn``    [nts][nw]      fermionic i omega -> fermionic tau (all points),
* ``Tnt_BF`` [nw_b][nts-2]  fermionic tau -> bosonic i Omega,
* ``Ttn_FB`` [nts][nw_b]    bosonic i Omega -> fermionic tau.

The matrices are built once on the host and uploaded to the engine; the
transforms themselves run on the GPU.  Eigen's complete-orthogonal-
decomposition pseudo-inverse is replaced by numpy's SVD pseudo-inverse (both
give the Moore-Penrose inverse; they agree to rounding).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict

import numpy as np


@dataclass
class IRTransforms:
    beta: float
    nts: int
    nw: int
    nw_b: int
    Tnt: np.ndarray
    Ttn: np.ndarray
    Tnt_BF: np.ndarray
    Ttn_FB: np.ndarray
    Tct: np.ndarray          # scaled fermionic tau(interior) -> IR coefficients
    wsample_fermi: np.ndarray
    wsample_bose: np.ndarray
    tau_fermi: np.ndarray    # the nts fermionic tau points

    @property
    def ncheb(self) -> int:
        return self.nts - 2

    def omega_fermi(self) -> np.ndarray:
        """i omega_n = i (2n+1) pi / beta at the sampling points (transformer_t.h:51-53)."""
        return 1j * (2.0 * self.wsample_fermi + 1.0) * np.pi / self.beta


def _stat(ir: Dict[str, np.ndarray], prefix: str):
    nx = int(ir[f"{prefix}/nx"])
    nw = int(ir[f"{prefix}/nw"])
    Tnc = ir[f"{prefix}/uwl_re"].reshape(nw, nx) + 1j * ir[f"{prefix}/uwl_im"].reshape(nw, nx)
    Ttc_tmp = ir[f"{prefix}/uxl"].reshape(nx, nx)
    Tcn = np.linalg.pinv(Tnc)
    Tct = np.linalg.pinv(Ttc_tmp)
    Ttc = np.zeros((nx + 2, nx))
    Ttc[0] = ir[f"{prefix}/ux1l_minus"]
    Ttc[nx + 1] = ir[f"{prefix}/ux1l"]
    Ttc[1:nx + 1] = Ttc_tmp
    return nx, nw, Tnc, Tcn, Ttc, Tct


def build_transforms(ir: Dict[str, np.ndarray], beta: float) -> IRTransforms:
    """Build the transform matrices from IR sampling data (transformer_t.cpp:48-82)."""
    ncheb, nw, Tnc, Tcn, Ttc, Tct = _stat(ir, "fermi")
    ncheb_b, nw_b, Tnc_B, Tcn_B, Ttc_B, Tct_B = _stat(ir, "bose")
    other_f = ir["fermi/other_uxl"].reshape(ncheb_b, ncheb)
    other_b = ir["bose/other_uxl"].reshape(ncheb, ncheb_b)
    Ttc_other = Ttc_B @ Tct_B @ other_f          # (nts_b, ncheb)
    Ttc_B_other = Ttc @ Tct @ other_b            # (nts, ncheb_b)
    s2b = np.sqrt(2.0 / beta)
    Ttc = Ttc * s2b
    Ttc_B = Ttc_B * s2b
    Ttc_other = Ttc_other * s2b
    Ttc_B_other = Ttc_B_other * s2b
    Tct = Tct * np.sqrt(beta / 2.0)
    Tct_B = Tct_B * np.sqrt(beta / 2.0)
    Tnc = Tnc * np.sqrt(beta)
    Tnc_B = Tnc_B * np.sqrt(beta)
    Tcn = Tcn * np.sqrt(1.0 / beta)
    Tcn_B = Tcn_B * np.sqrt(1.0 / beta)
    Tnt = Tnc @ Tct
    Ttn = Ttc @ Tcn
    Tnt_BF = Tnc_B @ Tct_B @ Ttc_other[1:ncheb_b + 1, :] @ Tct
    Ttn_FB = Ttc_B_other @ Tcn_B
    x = np.asarray(ir["fermi/xsample"], dtype=np.float64)
    tau = np.concatenate([[0.0], (x + 1.0) * beta / 2.0, [beta]])
    return IRTransforms(
        beta=float(beta), nts=ncheb + 2, nw=nw, nw_b=nw_b,
        Tnt=np.ascontiguousarray(Tnt, dtype=np.complex128),
        Ttn=np.ascontiguousarray(Ttn, dtype=np.complex128),
        Tnt_BF=np.ascontiguousarray(Tnt_BF, dtype=np.complex128),
        Ttn_FB=np.ascontiguousarray(Ttn_FB, dtype=np.complex128),
        Tct=np.ascontiguousarray(Tct),
        wsample_fermi=np.asarray(ir["fermi/wsample"], dtype=np.int64).reshape(-1),
        wsample_bose=np.asarray(ir["bose/wsample"], dtype=np.int64).reshape(-1),
        tau_fermi=tau,
    )


def gm_matrix(tr: IRTransforms) -> np.ndarray:
    """Interior-tau quadrature M of the Galitskii-Migdal integral:

        int_0^beta A(tau) B(beta - tau) dtau = sum_ij M_ij A(tau_i) B(tau_j)

    for fermionic A, B represented in the IR basis.  With a_l = sum_i C_li
    A(tau_i) (C = ``Tct``, the scaled fit onto u_l(tau), orthonormal on
    [0, beta]) and the parity u_l(beta - tau) = (-1)^l u_l(tau),
    the integral is sum_l (-1)^l a_l b_l, so M = C^T diag((-1)^l) C.
    Returns an (nts-2) x (nts-2) float64 array."""
    C = np.asarray(tr.Tct, dtype=np.float64)
    sign = np.where(np.arange(C.shape[0]) % 2 == 0, 1.0, -1.0)
    return np.ascontiguousarray(C.T @ (sign[:, None] * C))


def read_ir_file(path: str) -> Dict[str, np.ndarray]:
    """Read the IR sampling fields of a reference IR grid file (e.g. ``1e3_72.h5``)."""
    from .h5lite import H5File
    f = H5File(path)
    out = {}
    for stat in ("fermi", "bose"):
        for key in ("nx", "nw", "uwl_re", "uwl_im", "uxl", "ux1l", "ux1l_minus", "other_uxl",
                    "xsample", "wsample"):
            out[f"{stat}/{key}"] = f[f"{stat}/{key}"]
    return out

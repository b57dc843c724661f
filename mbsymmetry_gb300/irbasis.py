"""Intermediate-representation (IR) sparse-sampling grids, generated in FP64.

The reference reads precomputed IR sampling data from HDF5 files (e.g.
``ir_grid/1e3_72.h5``; reader: ``SymmetryMBPT/src/common/transformer_t.cpp:7-46``);
only the Lambda = 1e3, 72-function grid ships with it.  This module builds
the same fields for any (beta, number of tau points) from the published
construction of the IR basis (Shinaoka et al., PRB 96, 035147 (2017);
sparse sampling: Li et al., PRB 101, 035144 (2020)):

* singular value expansion of the logistic kernels on x, y in [-1, 1],
  K_F(x, y) = exp(-Lambda y (x+1)/2) / (1 + exp(-Lambda y)),
  K_B(x, y) = y exp(-Lambda y (x+1)/2) / (1 - exp(-Lambda y)),
  discretised by composite Gauss-Legendre quadrature graded towards x = +-1
  and y = 0;
* u_l(x) at any x by Nystrom interpolation, u_l(x) = sum_j w_j K(x, y_j) v_l(y_j) / s_l;
* u_l(i nu) in closed form (the x integral of the exponential kernel is
  analytic), normalised as the reference file stores it;
* tau sampling points: the roots of u_L (L = basis size), the sparse-sampling
  rule; Matsubara sampling points: a greedy well-conditioned selection
  (column-pivoted QR of the candidate matrix u_l(i nu_n)).

``tests/test_irbasis.py`` pins the basis functions against the reference's
``1e3_72.h5`` and checks every generated grid with exact single-pole
tau <-> i omega round trips.
"""
from __future__ import annotations

from functools import lru_cache
from typing import Dict, Tuple

import numpy as np

_NGL = 16


def _gl(n=_NGL):
    x, w = np.polynomial.legendre.leggauss(n)
    return x, w


def _graded_breakpoints(lam: float, around_zero: bool) -> np.ndarray:
    """Breakpoints on [-1, 1] graded geometrically towards the ends (or 0)."""
    jmax = int(np.ceil(np.log2(max(lam, 2.0)))) + 6
    if around_zero:
        pos = np.concatenate([[0.0], 2.0 ** -np.arange(jmax, -1, -1)])
        inner = np.linspace(0.0, 1.0, 17)
        pos = np.unique(np.concatenate([pos, inner]))
        return np.unique(np.concatenate([-pos[::-1], pos]))
    g = 1.0 - 2.0 ** -np.arange(0, jmax + 1)        # 0, 0.5, 0.75, ...
    g = np.concatenate([g, [1.0]])
    inner = np.linspace(0.0, 1.0, 17)
    pos = np.unique(np.concatenate([g, inner]))
    return np.unique(np.concatenate([-pos[::-1], pos]))


def _composite(bp: np.ndarray):
    t, w = _gl()
    a, b = bp[:-1, None], bp[1:, None]
    x = (0.5 * (b - a) * t[None, :] + 0.5 * (a + b)).ravel()
    ww = (0.5 * (b - a) * w[None, :]).ravel()
    return x, ww


def _kernel(stat: str, lam: float, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    X = x[:, None]
    Y = y[None, :]
    ly = lam * Y
    if stat == "F":
        # exp(-ly(x+1)/2)/(1+exp(-ly)), evaluated stably for both signs of y
        e = np.where(ly >= 0, -ly * (X + 1.0) / 2.0, ly * (1.0 - X) / 2.0)
        return np.exp(e) / (1.0 + np.exp(-np.abs(ly)))
    # bosonic: y exp(-ly(x+1)/2)/(1-exp(-ly))
    a = np.abs(ly)
    e = np.where(ly >= 0, -ly * (X + 1.0) / 2.0, ly * (1.0 - X) / 2.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        out = np.abs(Y) * np.exp(e) / (-np.expm1(-a))
    return np.where(a < 1e-300, 1.0 / lam, out)


@lru_cache(maxsize=16)
def _sve(stat: str, lam: float):
    xb = _graded_breakpoints(lam, around_zero=False)
    yb = _graded_breakpoints(lam, around_zero=True)
    x, wx = _composite(xb)
    y, wy = _composite(yb)
    K = _kernel(stat, lam, x, y)
    A = np.sqrt(wx)[:, None] * K * np.sqrt(wy)[None, :]
    U, s, Vt = np.linalg.svd(A, full_matrices=False)
    u = U / np.sqrt(wx)[:, None]   # u_l(x_i)
    v = Vt.T / np.sqrt(wy)[:, None]  # v_l(y_j)
    # sign convention: u_l(1) > 0
    u1 = _nystrom_u(stat, lam, np.array([1.0]), y, wy, v, s)[0]
    sgn = np.where(u1 < 0, -1.0, 1.0)
    return x, wx, y, wy, s, u * sgn[None, :], v * sgn[None, :]


def _nystrom_u(stat, lam, xs, y, wy, v, s):
    K = _kernel(stat, lam, np.asarray(xs, dtype=np.float64), y)
    return (K * wy[None, :]) @ v / s[None, :]


class IRBasis:
    """First ``size`` IR basis functions of one statistics at cutoff Lambda."""

    def __init__(self, stat: str, lam: float, size: int):
        assert stat in ("F", "B")
        self.stat, self.lam, self.size = stat, float(lam), int(size)
        x, wx, y, wy, s, u, v = _sve(stat, float(lam))
        if size + 1 > len(s):
            raise ValueError("basis size exceeds the discretisation")
        self._y, self._wy, self._v, self._s = y, wy, v, s
        self.s = s[:size]

    def u(self, xs: np.ndarray, nfun: int = None) -> np.ndarray:
        """u_l(x) for l < nfun, shape (len(xs), nfun)."""
        nfun = self.size if nfun is None else nfun
        return _nystrom_u(self.stat, self.lam, xs, self._y, self._wy, self._v[:, :nfun], self._s[:nfun])

    def uhat(self, n: np.ndarray, nfun: int = None) -> np.ndarray:
        """Matsubara transform at nu = 2n+1 (F) or 2n (B), shape (len(n), nfun)."""
        nfun = self.size if nfun is None else nfun
        n = np.asarray(n, dtype=np.int64)
        nu = 2 * n + (1 if self.stat == "F" else 0)
        y = self._y
        # x integral of the exponential kernel in closed form (see module doc)
        den = self.lam * y[None, :] - 1j * np.pi * nu[:, None]
        if self.stat == "F":
            kh = 2.0 / den
        else:
            kh = 2.0 * y[None, :] / den
        kh = kh / np.sqrt(2.0)
        return (kh * self._wy[None, :]) @ self._v[:, :nfun] / self._s[None, :nfun]

    def tau_sampling(self) -> np.ndarray:
        """Roots of u_size(x) on (-1, 1): ``size`` points."""
        L = self.size
        bp = _graded_breakpoints(self.lam, around_zero=False)
        grid = np.unique(np.concatenate([np.linspace(a, b, 65) for a, b in zip(bp[:-1], bp[1:])]))
        f = self.u(grid, L + 1)[:, L]
        idx = np.nonzero(np.sign(f[:-1]) * np.sign(f[1:]) < 0)[0]
        roots = []
        for i in idx:
            a, b = grid[i], grid[i + 1]
            fa = f[i]
            for _ in range(60):
                m = 0.5 * (a + b)
                fm = self.u(np.array([m]), L + 1)[0, L]
                if np.sign(fm) == np.sign(fa):
                    a, fa = m, fm
                else:
                    b = m
            roots.append(0.5 * (a + b))
        roots = np.array(roots)
        if len(roots) != L:
            raise RuntimeError(f"found {len(roots)} tau sampling points, expected {L}")
        return roots

    def _uhat_one(self, n: np.ndarray, l: int) -> np.ndarray:
        out = np.empty(len(n), dtype=np.complex128)
        for c in range(0, len(n), 4096):
            out[c:c + 4096] = self.uhat(n[c:c + 4096], l + 1)[:, l]
        return out

    def matsubara_sampling(self, symmetric: bool = True) -> np.ndarray:
        """``size`` Matsubara indices chosen greedily for a well-conditioned
        sampling matrix over a candidate set (every |n| < 2000, then a
        geometric grid up to 50 Lambda).

        symmetric (the default): the set is closed under nu -> -nu, as
        sparse-ir's sampling and the reference's own grid (``1e3_72.h5``)
        are: pairs (nu, -nu) are taken greedily by the residual norm of
        [Re u_l(i nu), Im u_l(i nu)] (u_l(-i nu) = conj(u_l(i nu)) for real
        u_l), with nu = 0 first for an odd bosonic size.  Time reversal then
        maps the sampled frequencies onto themselves, which keeps
        P~(-q) = conj(P~(q)) exact through the nonlinear W~ step.
        symmetric=False: column-pivoted QR of the complex rows (an
        unsymmetric set)."""
        import scipy.linalg
        L = self.size
        nmax = int(max(4000, 50 * self.lam))
        pos = np.unique(np.concatenate([np.arange(0, 2000),
                                        np.round(np.geomspace(2000, nmax, 3000)).astype(np.int64)]))
        if not symmetric:
            if self.stat == "F":
                cand = np.concatenate([-pos[::-1] - 1, pos])
            else:
                cand = np.unique(np.concatenate([-pos[::-1], pos]))
            M = np.empty((len(cand), L), dtype=np.complex128)
            for c in range(0, len(cand), 4096):
                M[c:c + 4096] = self.uhat(cand[c:c + 4096], L)
            _, _, piv = scipy.linalg.qr(M.T, pivoting=True, mode="economic")
            return np.sort(cand[piv[:L]])
        M = np.empty((len(pos), L), dtype=np.complex128)
        for c in range(0, len(pos), 4096):
            M[c:c + 4096] = self.uhat(pos[c:c + 4096], L)
        R = np.stack([M.real, M.imag], axis=1)          # (candidate, re/im, l): residual rows

        def take(i, rows):
            for r in rows:                               # Gram-Schmidt of the chosen rows out of every residual
                v = R[i, r].copy()
                nv = np.linalg.norm(v)
                if nv > 0:
                    v /= nv
                    R[...] -= np.einsum("crl,l->cr", R, v)[:, :, None] * v[None, None, :]
            R[i] = 0.0

        if self.stat == "F" and L % 2:
            raise ValueError("a symmetric fermionic sampling set has an even size")
        chosen = []
        i0 = int(np.nonzero(pos == 0)[0][0])
        if self.stat == "B" and L % 2 == 1:              # nu = 0 (a real row) completes an odd size
            take(i0, (0,))
            chosen.append(i0)
        elif self.stat == "B":
            R[i0] = 0.0                                  # nu = 0 has no partner
        pairs = []
        while len(pairs) < L // 2:
            i = int(np.argmax(np.einsum("crl,crl->c", R, R)))
            take(i, (0, 1))
            pairs.append(i)
        n = pos[np.array(pairs, dtype=np.int64)]
        neg = -n - 1 if self.stat == "F" else -n
        n = np.concatenate([n, pos[np.array(chosen, dtype=np.int64)]])
        return np.sort(np.unique(np.concatenate([n, neg])))


def find_lambda(size: int, eps: float = 1e-13, lo: float = 10.0, hi: float = 1e9) -> float:
    """Smallest Lambda on a log grid whose fermionic and bosonic bases both
    have ``size + 2`` singular values above eps * s_0 (so u_size and the
    sampling functions are well determined in FP64)."""
    grid = np.exp(np.linspace(np.log(lo), np.log(hi), 73))
    for lam in grid:
        ok = True
        for stat in ("F", "B"):
            s = _sve(stat, float(lam))[4]
            ok &= np.count_nonzero(s / s[0] > eps) >= size + 2
        if ok:
            return float(lam)
    raise ValueError("no Lambda found")


def ir_fields(lam: float, nl_f: int, nl_b: int) -> Dict[str, np.ndarray]:
    """The sampling data fields ``transformer_t`` reads
    (``transformer_t.cpp:17-33, 53-56``)."""
    F = IRBasis("F", lam, nl_f)
    B = IRBasis("B", lam, nl_b)
    xf, xb = F.tau_sampling(), B.tau_sampling()
    wf, wb = F.matsubara_sampling(), B.matsubara_sampling()
    if len(wf) != nl_f or len(wb) != nl_b:
        raise RuntimeError(f"Matsubara sampling sizes {len(wf)}/{len(wb)} != {nl_f}/{nl_b}")
    out = {}
    for stat, basis, xs, ws, other in (("fermi", F, xf, wf, xb), ("bose", B, xb, wb, xf)):
        L = basis.size
        uw = basis.uhat(ws)
        out[f"{stat}/nx"] = np.int64(L)
        out[f"{stat}/nw"] = np.int64(L)
        out[f"{stat}/uwl_re"] = np.ascontiguousarray(uw.real)
        out[f"{stat}/uwl_im"] = np.ascontiguousarray(uw.imag)
        out[f"{stat}/uxl"] = basis.u(xs)
        out[f"{stat}/ux1l"] = basis.u(np.array([1.0]))[0]
        out[f"{stat}/ux1l_minus"] = basis.u(np.array([-1.0]))[0]
        out[f"{stat}/other_uxl"] = basis.u(other)
        out[f"{stat}/xsample"] = xs
        out[f"{stat}/wsample"] = ws
    return out


def make_ir_grid(nts: int, eps: float = 1e-13) -> Tuple[float, Dict[str, np.ndarray]]:
    """IR data for ``nts`` tau points (nts - 2 fermionic basis functions)."""
    nl = nts - 2
    lam = find_lambda(nl, eps)
    return lam, ir_fields(lam, nl, nl - 1)

"""Irrep block sizes from the space group: the physical counterpart of the
labelled-block generator in crystal.py, for symmorphic cubic crystals.

SymmetryAdaptation (the reference's offline tool,
``SymmetryAdaptation/src/dirac_character.cpp:7-126``,
``src/k_space_structure.cpp``, ``src/wigner_d.cpp``) block-diagonalises the
orbital basis at every k by the irreps of the little co-group G_k, found
through Dirac characters (class sums).  This module restates that decomposition
for the Fm-3m point group O_h on an FCC lattice:

* the 48 operations are the signed 3 x 3 permutation matrices;
* G_k = {R : R k = k modulo a reciprocal lattice vector};
* the representation on Bloch sums of atom-centred shells with angular
  momentum l <= 2: D(R)[(b, nu), (a, mu)] = exp(-i (R k).T) D^l(R)[nu, mu]
  for R tau_a = tau_b + T (D^0 = 1, D^1 = R on (x, y, z), D^2 = the action
  Q -> R Q R^T on an orthonormal basis of traceless symmetric matrices);
* a random combination of the class sums C_j of G_k is diagonalised; its
  eigenspaces are the isotypic components, and each component's class-sum
  eigenvalues lambda_j = |C_j| chi(g_j) / d give the irrep dimension from
  sum_j |lambda_j|^2 / |C_j| = |G_k| / d^2.

An irrep Gamma of dimension d with multiplicity m contributes d blocks of
size m (the rows of Gamma), which is how the flat layout lists them.
Non-symmorphic groups (P6_3mc) would need projective representations at the
zone boundary and are not covered.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass
from typing import Dict, List, Sequence, Tuple

import numpy as np

FCC_A = np.array([[0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]]).T  # columns: primitive vectors


def oh_operations() -> List[np.ndarray]:
    """The 48 proper and improper rotations of O_h (signed permutation matrices)."""
    ops = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            R = np.zeros((3, 3), dtype=int)
            for i, (j, s) in enumerate(zip(perm, signs)):
                R[i, j] = s
            ops.append(R)
    return ops


def _d2_basis() -> List[np.ndarray]:
    """Orthonormal (Frobenius) basis of traceless symmetric 3 x 3 matrices: xy, yz, zx, x2-y2, 3z2-r2."""
    def sym(i, j):
        Q = np.zeros((3, 3))
        Q[i, j] = Q[j, i] = 1.0
        return Q / np.sqrt(2.0)
    return [sym(0, 1), sym(1, 2), sym(0, 2), np.diag([1.0, -1.0, 0.0]) / np.sqrt(2.0),
            np.diag([-1.0, -1.0, 2.0]) / np.sqrt(6.0)]


_D2 = _d2_basis()


def shell_matrix(l: int, R: np.ndarray) -> np.ndarray:
    """D^l(R) on real s, p (x, y, z) or d functions: (P_R f)(r) = f(R^-1 r)."""
    R = np.asarray(R, dtype=float)
    if l == 0:
        return np.ones((1, 1))
    if l == 1:
        return R.copy()
    if l == 2:
        return np.array([[np.sum(Qn * (R @ Qm @ R.T)) for Qm in _D2] for Qn in _D2])
    raise ValueError("l <= 2 only")


@dataclass
class Basis:
    """Atom positions (cubic coordinates) and the shells (l values) on each atom."""
    positions: np.ndarray
    shells: Sequence[Sequence[int]]

    @property
    def size(self) -> int:
        return sum(2 * l + 1 for sh in self.shells for l in sh)


def _is_lattice(v: np.ndarray, A: np.ndarray = FCC_A) -> bool:
    c = np.linalg.solve(A, v)
    return np.allclose(c, np.round(c), atol=1e-9)


def little_group(k_cart: np.ndarray, ops: List[np.ndarray]) -> List[np.ndarray]:
    """Operations R with R k - k a reciprocal lattice vector (k in units of 2 pi)."""
    Brec = np.linalg.inv(FCC_A).T  # reciprocal primitive vectors (columns), units of 2 pi
    out = []
    for R in ops:
        d = np.linalg.solve(Brec, R @ k_cart - k_cart)
        if np.allclose(d, np.round(d), atol=1e-9):
            out.append(R)
    return out


def bloch_representation(k_cart: np.ndarray, R: np.ndarray, basis: Basis) -> np.ndarray:
    """D(R) on the Bloch sums sum_L exp(i k.L) phi_{a,mu}(r - tau_a - L) (k in units of 2 pi)."""
    n = basis.size
    D = np.zeros((n, n), dtype=complex)
    offs = np.cumsum([0] + [sum(2 * l + 1 for l in sh) for sh in basis.shells])
    kR = R @ k_cart
    pos = np.asarray(basis.positions, dtype=float)
    for a in range(len(pos)):
        ra = R @ pos[a]
        b = next(b for b in range(len(pos)) if _is_lattice(ra - pos[b]))
        if [l for l in basis.shells[a]] != [l for l in basis.shells[b]]:
            raise ValueError("an operation maps atoms with different shells onto each other")
        T = ra - pos[b]
        phase = np.exp(-2j * np.pi * kR @ T)
        oa, ob = offs[a], offs[b]
        for l in basis.shells[a]:
            w = 2 * l + 1
            D[ob:ob + w, oa:oa + w] = phase * shell_matrix(l, R)
            oa += w
            ob += w
    return D


def _classes(G: List[np.ndarray]) -> List[List[int]]:
    key = lambda M: tuple(np.asarray(M).ravel())
    index = {key(g): i for i, g in enumerate(G)}
    seen, classes = set(), []
    for i, g in enumerate(G):
        if i in seen:
            continue
        cls = sorted({index[key(s @ g @ np.round(np.linalg.inv(s)).astype(int))] for s in G})
        seen.update(cls)
        classes.append(cls)
    return classes


def irrep_content(k_cart: np.ndarray, basis: Basis, ops: List[np.ndarray] = None,
                  seed: int = 0) -> List[Tuple[int, int]]:
    """[(irrep dimension d, multiplicity m)] of the representation at k, one entry
    per isotypic component (sorted by d, then m)."""
    ops = oh_operations() if ops is None else ops
    G = little_group(np.asarray(k_cart, dtype=float), ops)
    Ds = [bloch_representation(k_cart, R, basis) for R in G]
    cls = _classes(G)
    C = [sum(Ds[i] for i in c) for c in cls]
    rng = np.random.default_rng(seed)
    coef = rng.standard_normal(len(C)) + 1j * rng.standard_normal(len(C))
    M = sum(c * Cj for c, Cj in zip(coef, C))
    w, V = np.linalg.eig(M)
    out, used = [], np.zeros(len(w), dtype=bool)
    scale = max(1.0, np.abs(w).max())
    for i in range(len(w)):
        if used[i]:
            continue
        grp = np.where(~used & (np.abs(w - w[i]) < 1e-7 * scale))[0]
        used[grp] = True
        Q, _ = np.linalg.qr(V[:, grp])
        lam = [np.trace(Q.conj().T @ Cj @ Q) / len(grp) for Cj in C]
        s = sum(abs(lj) ** 2 / len(c) for lj, c in zip(lam, cls))
        d = int(round(np.sqrt(len(G) / s)))
        if d < 1 or len(grp) % d:
            raise RuntimeError("inconsistent isotypic component")
        out.append((d, len(grp) // d))
    return sorted(out)


def block_sizes(k_cart: np.ndarray, basis: Basis, ops: List[np.ndarray] = None) -> List[int]:
    """Block sizes of the flat layout at k: d blocks of size m per irrep (d, m)."""
    return [m for d, m in irrep_content(k_cart, basis, ops) for _ in range(d)]


def fcc_kmesh(n: int) -> np.ndarray:
    """n x n x n Monkhorst-Pack-style mesh (Gamma-centred), Cartesian, units of 2 pi."""
    Brec = np.linalg.inv(FCC_A).T
    f = np.array([(i / n, j / n, l / n) for i in range(n) for j in range(n) for l in range(n)])
    return f @ Brec.T


def shells_for(count: int, lmax: int = 2) -> List[int]:
    """A shell list (l values, l <= lmax) with exactly `count` functions: shells
    added in the order s, p, d, s, p, d, ... while they fit, then s shells for
    the rest (4 -> s p, 13 -> s p d s p)."""
    out, left = [], count
    while left > 0:
        added = False
        for l in range(lmax + 1):
            if 2 * l + 1 <= left:
                out.append(l)
                left -= 2 * l + 1
                added = True
        if not added:
            break
    out += [0] * left
    return sorted(out)

def layout_block_sizes(nk_side: int, ao: Basis, aux: Basis) -> Dict[str, List[List[int]]]:
    """Per k of an n^3 FCC mesh: AO and aux block sizes from the O_h decomposition."""
    ops = oh_operations()
    ks = fcc_kmesh(nk_side)
    return {"ao": [block_sizes(k, ao, ops) for k in ks], "aux": [block_sizes(k, aux, ops) for k in ks]}


def fcc_basis(count: int, atoms: int) -> Basis:
    """`count` functions on 2 atoms (rock salt: (0,0,0), (1/2,1/2,1/2)) or 4 atoms
    (those two plus the pair (1/4,1/4,1/4), (3/4,3/4,3/4), which O_h maps onto each
    other); the pair shares a shell list, each single atom has its own."""
    if atoms == 2:
        a = count // 2
        return Basis(np.array([[0, 0, 0], [0.5, 0.5, 0.5]]), [shells_for(a), shells_for(count - a)])
    if atoms == 4:
        c = count // 4
        r = count - 2 * c
        a = r // 2
        return Basis(np.array([[0, 0, 0], [0.5, 0.5, 0.5], [0.25, 0.25, 0.25], [0.75, 0.75, 0.75]]),
                     [shells_for(a), shells_for(r - a), shells_for(c), shells_for(c)])
    raise ValueError("2 or 4 atoms")

"""Irrep block sizes from the space group: the physical counterpart of the
labelled-block generator in crystal.py, for the symmorphic cubic crystals
(O_h) and the non-symmorphic wurtzite structure (P6_3mc).

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

Non-symmorphic groups (P6_3mc, the wurtzite structure of config C4): the
operations are {R | t} with fractional translations t (the 6_3 screw axis and
the c glides), and on Bloch sums at k the operations of the little group form
a projective representation of the little co-group (the factor system
exp(-i k . (R_g t_h + t_g - t_gh)) is non-trivial at the zone boundary, where
every irrep of P6_3mc at A is two-dimensional).  ``projective_content``
decomposes any unitary (projective) representation without classes: the
average over the group of D(h) A D(h)^H for a random A in the span of the D(g)
is central, its eigenspaces are the isotypic components, and the average of
D(h) X D(h)^H for a random Hermitian X acts on a component as I_d x M_m, so its
eigenvalues there come in m distinct values of multiplicity d.
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


# --------------------------------------------------------------------------- #
# non-symmorphic: P6_3mc (wurtzite)
# --------------------------------------------------------------------------- #
HEX_C = 1.633  # ideal c/a
HEX_A = np.array([[1.0, -0.5, 0.0], [0.0, np.sqrt(3.0) / 2.0, 0.0], [0.0, 0.0, HEX_C]])  # columns: a1, a2, a3

# The 12 operations of P6_3mc (International Tables No. 186) as coordinate
# triplets in the hexagonal setting, with the translation along c (in units of
# c): the 6_3 and 2_1 screw rotations and one class of mirrors carry c/2 (c
# glides), in the origin where the wurtzite sites are (1/3, 2/3, z) and
# (2/3, 1/3, z + 1/2) (Wyckoff 2b); tests check that every operation maps
# the structure onto itself.
_P63MC = [("x", "y", "z", 0.0), ("-y", "x-y", "z", 0.0), ("-x+y", "-x", "z", 0.0), ("-x", "-y", "z", 0.5),
          ("y", "-x+y", "z", 0.5), ("x-y", "x", "z", 0.5), ("y", "x", "z", 0.5), ("x-y", "-y", "z", 0.5),
          ("-x", "-x+y", "z", 0.5), ("-y", "-x", "z", 0.0), ("-x+y", "y", "z", 0.0), ("x", "x-y", "z", 0.0)]


def _triplet_row(expr: str) -> np.ndarray:
    row, sign = np.zeros(3, dtype=int), 1
    for ch in expr:
        if ch in "+-":
            sign = 1 if ch == "+" else -1
        else:
            row["xyz".index(ch)] += sign
            sign = 1
    return row


def p63mc_operations() -> List[Tuple[np.ndarray, np.ndarray]]:
    """(M, t): x -> M x + t on fractional coordinates of the hexagonal lattice."""
    return [(np.array([_triplet_row(a), _triplet_row(b), _triplet_row(c)]), np.array([0.0, 0.0, tz]))
            for a, b, c, tz in _P63MC]


def wurtzite_basis(count: int, u: float = 0.375) -> Basis:
    """`count` functions on the four wurtzite sites (fractional coordinates): species
    A at (1/3, 2/3, 0) and (2/3, 1/3, 1/2), species B at the same raised by u c;
    the two sites of a species share a shell list (B gets the smaller half)."""
    a = (count + 1) // 2
    a -= a % 2 if (count - a) % 2 else 0
    half_a, half_b = a // 2, (count - a) // 2
    if 2 * half_a + 2 * half_b != count:
        half_a = (count - 2 * (count // 4)) // 2
        half_b = count // 4
    pos = np.array([[1 / 3, 2 / 3, 0.0], [2 / 3, 1 / 3, 0.5], [1 / 3, 2 / 3, u], [2 / 3, 1 / 3, 0.5 + u]])
    sa, sb = shells_for(half_a), shells_for(half_b)
    return Basis(pos, [sa, sa, sb, sb])


def sg_little_group(k_frac: np.ndarray, ops) -> list:
    """Space-group operations whose rotation maps k (reduced reciprocal coordinates)
    onto itself modulo a reciprocal lattice vector."""
    out = []
    for M, t in ops:
        d = np.linalg.inv(M).T @ k_frac - k_frac
        if np.allclose(d, np.round(d), atol=1e-9):
            out.append((M, t))
    return out


def sg_bloch_representation(k_frac: np.ndarray, M: np.ndarray, t: np.ndarray, basis: Basis,
                            A: np.ndarray = HEX_A) -> np.ndarray:
    """D({M|t}) on the Bloch sums at k (reduced reciprocal coordinates; positions and
    t fractional): atom a goes to M tau_a + t = tau_b + T, phase exp(-2 pi i (M k) . T),
    shells rotated by the Cartesian R = A M A^-1."""
    n = basis.size
    D = np.zeros((n, n), dtype=complex)
    offs = np.cumsum([0] + [sum(2 * l + 1 for l in sh) for sh in basis.shells])
    R = A @ M @ np.linalg.inv(A)
    kR = np.linalg.inv(M).T @ k_frac
    pos = np.asarray(basis.positions, dtype=float)
    for a in range(len(pos)):
        ra = M @ pos[a] + t
        b = next(b for b in range(len(pos)) if np.allclose(ra - pos[b], np.round(ra - pos[b]), atol=1e-9))
        if list(basis.shells[a]) != list(basis.shells[b]):
            raise ValueError("an operation maps atoms with different shells onto each other")
        T = np.round(ra - pos[b])
        phase = np.exp(-2j * np.pi * kR @ T)
        oa, ob = offs[a], offs[b]
        for l in basis.shells[a]:
            w = 2 * l + 1
            D[ob:ob + w, oa:oa + w] = phase * shell_matrix(l, R)
            oa += w
            ob += w
    return D


def projective_content(Ds: List[np.ndarray], seed: int = 0) -> List[Tuple[int, int]]:
    """[(irrep dimension d, multiplicity m)] of a unitary, possibly projective,
    representation given by its matrices on the (little) group."""
    rng = np.random.default_rng(seed)
    G = len(Ds)
    n = Ds[0].shape[0]
    A = sum((rng.standard_normal() + 1j * rng.standard_normal()) * D for D in Ds)
    C = sum(D @ A @ D.conj().T for D in Ds) / G
    X = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    X = X + X.conj().T
    Y = sum(D @ X @ D.conj().T for D in Ds) / G
    w, V = np.linalg.eig(C)
    scale = max(1.0, np.abs(w).max())
    out, used = [], np.zeros(n, dtype=bool)
    for i in range(n):
        if used[i]:
            continue
        grp = np.where(~used & (np.abs(w - w[i]) < 1e-7 * scale))[0]
        used[grp] = True
        Q, _ = np.linalg.qr(V[:, grp])
        y = np.sort(np.linalg.eigvalsh(Q.conj().T @ Y @ Q))
        ys = max(1.0, np.abs(y).max())
        m = 1 + int(np.sum(np.diff(y) > 1e-7 * ys))
        if len(grp) % m:
            raise RuntimeError("inconsistent isotypic component")
        out.append((len(grp) // m, m))
    return sorted(out)


def sg_block_sizes(k_frac: np.ndarray, basis: Basis, ops=None, A: np.ndarray = HEX_A) -> List[int]:
    """Block sizes at k from the space group (default P6_3mc): d blocks of size m per irrep."""
    ops = p63mc_operations() if ops is None else ops
    G = sg_little_group(np.asarray(k_frac, dtype=float), ops)
    Ds = [sg_bloch_representation(np.asarray(k_frac, dtype=float), M, t, basis, A) for M, t in G]
    return [m for d, m in projective_content(Ds) for _ in range(d)]

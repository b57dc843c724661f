"""Tight-binding crystals from Gaussian orbitals: seeded inputs whose block
structure comes from the space group through the physics, not from labels.

The reference obtains its inputs from PySCF (Gaussian density fitting) and
SymmetryAdaptation's block diagonalisation
(``scripts/integrals/init_data_full_block.py``,
``SymmetryAdaptation/src/dirac_character.cpp:7-126``,
``SymmetryAdaptation/src/space_group_rep.cpp``).  Neither runs here; this
module builds inputs of the same kind for an FCC crystal (O_h; the 2-atom
rock-salt or the 4-atom basis of ``symmetry.fcc_basis``) and for wurtzite
(P6_3mc, ``symmetry.wurtzite_basis``: non-symmorphic, projective
representations at the zone boundary, no inversion).  Both are handled as
space groups, operations (M, t) on fractional coordinates:

* orbitals: s/p/d shells on the atoms; real solid harmonics (1; x, y, z;
  r.Q_n.r for the orthonormal traceless Q_n of ``symmetry``) times Gaussians.
  Atoms of one orbit under the group (a species) share shells, exponents and
  hopping parameters, so every datum below is invariant under the group.
* F(k)_ij = sum_L exp(2 pi i k.L) E_ij(tau_j + L - tau_i) + onsite energies:
  Slater-Koster two-centre hoppings.  E(d) = D(R_d) E0(|d|) D(R_d)^T with
  R_d a rotation taking z onto d and E0 the bond-frame matrix, diagonal in
  the sigma / pi / delta channels; by default nearest-neighbour bonds only,
  strengths U(-1, 1) Ha and onsite energies N(0, 0.5) Ha (further shells,
  when asked for, decay as exp(-(|d| - d_nn) / lambda)); the strength of
  the ordered shell pair (j, i) is (-1)^(l_i + l_j) times that of (i, j),
  which makes F Hermitian.  S = I.
* V^Q_ij(k1, k2) = sum_{L_Q, L_j} exp(2 pi i (-p.L_Q + k2.L_j))
  (Q, tau_Q + L_Q | i, tau_i | j, tau_j + L_j), p = k2 - k1 (the q that
  labels the pair's aux blocks): Bloch sums of three-centre overlaps of
  Gaussian auxiliary functions (exponents 0.3 - 3.0) with two orbitals, over
  the configurations whose three pair distances are all within a cutoff
  (a set invariant under the group and under exchanging i and j, so the
  Hermitian pair relation V(k2, k1)_{Q,j,i} = conj(V(k1, k2)_{Q,i,j}) is
  exact).  Integrals are Cartesian-factorised (Gaussian product theorem,
  moments of exp(-eta u^2)).
* symmetry-adapted bases: at a star representative k_r, the eigenvectors of
  A = sum_h c_h (D(h) + D(h)^H) over the little group, with seeded real c_h
  and D(h) the representation on the Bloch sums (``symmetry.
  bloch_representation``).  A acts on an isotypic component C^d x C^m as
  Gamma(a) x I_m, so its eigenspaces are the rows of the irreps: d blocks of
  size m per irrep of dimension d and multiplicity m, the layout's blocks.
  Every operator that commutes with the little group (F, G, P0) is
  block-diagonal in them.  At k = g k_r (g the first operation, in the
  group's order, that maps k_r to k) the basis is D(g) U(k_r) W_k, W_k a
  seeded block-unitary gauge, and orep(k) = U(k)^H D(g) U(k_r) = W_k^H.
* aux bases: the same construction, and the basis at -q is the complex
  conjugate of the one at q (the pairing that the P0 loop, which reads
  V(k, k + q), and the Sigma loop, which reads V(k, k - q), assume when
  they use the same aux blocks for both).  Where an operation u takes k_r
  to -k_r, the matrix diagonalised is B + D(u)^H conj(B) D(u) with B the
  sum above, so that conj(Y(k_r)) and D(u) Y(k_r) span the same eigenspaces
  in the same order: -q is then reached from q_r by g u and auxrep stays
  block-diagonal.  At self-conjugate q the basis is real.  Rows that time
  reversal glues together (the A-L-H face of wurtzite) end up in one block.
* time reversal: where the point group lacks the operation (wurtzite), k =
  -k' joins the star of k' through time reversal (``conj_index``); its bases
  are conj(U(k')), conj(Y(k')) and the rotation path conjugates G and P~
  there (F(-k) = conj(F(k)) and V(-k1, -k2) = conj(V(k1, k2)) for real
  orbitals).
* selection rule: a block of V(k1, k2) is stored unless the group forbids it,
  i.e. unless it vanishes for a generic tensor averaged over the pair's
  magnetic stabiliser (the operations that fix k1 and k2, and time reversal
  after I h, which real orbitals make a symmetry: V(-k1, -k2) =
  conj(V(k1, k2))).  The data vanish on every forbidden block to rounding;
  a few allowed blocks can vanish too (the (Q|ij) = (Q|ji) symmetry of real
  orbitals, which the rule does not use) and are stored as zeros.

A crystal built with ``rotate=True`` (irreducible k, rotations) and one with
``rotate=False`` (every k, identity rotations) hold the same V and F in the
same bases, so the reference's iBZ-vs-full-BZ relation
(``SymmetryMBPT/test/test_cugw.cpp:306-436``) holds on them exactly.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field
from typing import Dict, List, Tuple

import numpy as np

from . import symmetry
from .crystal import Crystal, CrystalSpec, _find, _kmesh, _rand_unitary, _stars, half_filling_mu
from .layout import BlockLayout, wrap_1stbz

# --------------------------------------------------------------------------- #
# model parameters
# --------------------------------------------------------------------------- #


@dataclass
class OrbitalModel:
    """Length scales and parameter ranges of the tight-binding model (bohr, Ha)."""
    a_lat: float = 7.0                       # conventional cubic lattice constant (fcc)
    a_lat_hex: float = 6.1                   # in-plane lattice constant (hexagonal; c = 1.633 a)
    ao_exponents: Tuple[float, float] = (0.3, 1.2)
    aux_exponents: Tuple[float, float] = (0.3, 3.0)
    onsite: float = 0.5                      # onsite energies ~ N(0, onsite)
    hopping: float = 1.0                     # bond-frame strengths ~ U(-hopping, hopping) at d_nn
    decay: float = 1.5                       # lambda of exp(-(d - d_nn) / lambda) beyond the first shell
    neighbour_shells: int = 1                # hoppings over this many neighbour distances
    v_cutoff: float = 1.2                    # three-centre pair distances up to this many a_lat
    seed: int = 20260201


# --------------------------------------------------------------------------- #
# Slater-Koster bond matrices
# --------------------------------------------------------------------------- #
# Bond along z: the component of each real harmonic in the sigma, pi and delta
# channels (p: x, y, z; d: xy, yz, zx, x2-y2, 3z2-r2, the order of symmetry._D2).
_CHANNEL_INDEX = {0: {"s": 0},
                  1: {"s": 2, "px": 0, "py": 1},
                  2: {"s": 4, "px": 2, "py": 1, "dx": 0, "dy": 3}}
_CHANNEL_M = {"s": 0, "px": 1, "py": 1, "dx": 2, "dy": 2}


def bond_frame_matrix(l_row: int, l_col: int, v: np.ndarray) -> np.ndarray:
    """E0 for a bond along +z: v[|m|] between the components of one channel."""
    E = np.zeros((2 * l_row + 1, 2 * l_col + 1))
    for ch, ir in _CHANNEL_INDEX[l_row].items():
        ic = _CHANNEL_INDEX[l_col].get(ch)
        if ic is not None:
            E[ir, ic] = v[_CHANNEL_M[ch]]
    return E


def bond_rotation(d: np.ndarray) -> np.ndarray:
    """A proper rotation whose third column is d / |d| (it takes z onto d)."""
    z = np.asarray(d, dtype=float) / np.linalg.norm(d)
    a = np.array([1.0, 0.0, 0.0]) if abs(z[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    x = a - z * (a @ z)
    x /= np.linalg.norm(x)
    return np.stack([x, np.cross(z, x), z], axis=1)


def sk_block(l_row: int, l_col: int, v: np.ndarray, d: np.ndarray) -> np.ndarray:
    """<row shell at 0 | H | column shell at d> = D(R_d) E0 D(R_d)^T."""
    R = bond_rotation(d)
    return symmetry.shell_matrix(l_row, R) @ bond_frame_matrix(l_row, l_col, v) @ symmetry.shell_matrix(l_col, R).T


# --------------------------------------------------------------------------- #
# Gaussian three-centre overlaps
# --------------------------------------------------------------------------- #
_CART = {0: [(0, 0, 0)], 1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
         2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (0, 1, 1), (1, 0, 1)]}


def _cart_to_solid(l: int) -> np.ndarray:
    """Rows: the real solid harmonics of shell l in the Cartesian monomials _CART[l]."""
    if l == 0:
        return np.ones((1, 1))
    if l == 1:
        return np.eye(3)
    return np.array([[Q[0, 0], Q[1, 1], Q[2, 2], 2 * Q[0, 1], 2 * Q[1, 2], 2 * Q[0, 2]] for Q in symmetry._D2])


_C2S = {l: _cart_to_solid(l) for l in range(3)}


def _shift_poly(c: np.ndarray, a: int) -> np.ndarray:
    """Coefficients of (u + c)^a in powers of u, batched over c: (N, a + 1)."""
    one = np.ones_like(c)
    if a == 0:
        return one[:, None]
    if a == 1:
        return np.stack([c, one], axis=1)
    return np.stack([c * c, 2 * c, one], axis=1)


def _poly_mul(p: np.ndarray, q: np.ndarray) -> np.ndarray:
    out = np.zeros((p.shape[0], p.shape[1] + q.shape[1] - 1))
    for i in range(p.shape[1]):
        out[:, i:i + q.shape[1]] += p[:, i:i + 1] * q
    return out


def _moments(eta: np.ndarray, nmax: int) -> np.ndarray:
    """int u^n exp(-eta u^2) du for n = 0..nmax: (N, nmax + 1)."""
    m = np.zeros((eta.shape[0], nmax + 1))
    g = np.sqrt(np.pi / eta)
    for n in range(0, nmax + 1, 2):
        m[:, n] = g
        g = g * (n + 1) / (2 * eta)
    return m


def _axis_table(PA, PB, PC, eta, la, lb, lc) -> np.ndarray:
    """int (x-A)^a (x-B)^b (x-C)^c exp(-eta (x-P)^2) dx for a <= la, b <= lb, c <= lc."""
    M = _moments(eta, la + lb + lc)
    out = np.zeros((PA.shape[0], la + 1, lb + 1, lc + 1))
    for a in range(la + 1):
        pa = _shift_poly(PA, a)
        for b in range(lb + 1):
            pab = _poly_mul(pa, _shift_poly(PB, b))
            for c in range(lc + 1):
                p = _poly_mul(pab, _shift_poly(PC, c))
                out[:, a, b, c] = np.einsum("nk,nk->n", p, M[:, :p.shape[1]])
    return out


def three_centre(A: np.ndarray, a: float, la: int, B: np.ndarray, b: float, lb: int,
                 C: np.ndarray, c: float, lc: int) -> np.ndarray:
    """int chi_A chi_B chi_C over space for N configurations of the centres
    (A, B, C: (N, 3)): (N, 2la+1, 2lb+1, 2lc+1), unnormalised shells
    S_l(r - X) exp(-x |r - X|^2)."""
    eta = a + b + c
    P = (a * A + b * B + c * C) / eta
    K = np.exp(-(a * b * np.sum((A - B) ** 2, 1) + a * c * np.sum((A - C) ** 2, 1)
                 + b * c * np.sum((B - C) ** 2, 1)) / eta)
    e = np.full(A.shape[0], eta)
    tabs = [_axis_table(P[:, x] - A[:, x], P[:, x] - B[:, x], P[:, x] - C[:, x], e, la, lb, lc) for x in range(3)]
    ca, cb, cc = _CART[la], _CART[lb], _CART[lc]
    cart = np.empty((A.shape[0], len(ca), len(cb), len(cc)))
    for i, ma in enumerate(ca):
        for j, mb in enumerate(cb):
            for k, mc in enumerate(cc):
                cart[:, i, j, k] = K * tabs[0][:, ma[0], mb[0], mc[0]] * tabs[1][:, ma[1], mb[1], mc[1]] \
                    * tabs[2][:, ma[2], mb[2], mc[2]]
    return np.einsum("ai,bj,ck,nijk->nabc", _C2S[la], _C2S[lb], _C2S[lc], cart, optimize=True)


def shell_norm(alpha: float, l: int) -> float:
    """1 / sqrt(int (S_l exp(-alpha r^2))^2) (equal for every component of the shell)."""
    z = np.zeros((1, 3))
    s = three_centre(z, alpha, l, z, alpha, l, z, 0.0, 0)[0, :, :, 0]
    return 1.0 / np.sqrt(s[0, 0])


# --------------------------------------------------------------------------- #
# the crystal
# --------------------------------------------------------------------------- #
@dataclass
class _Shells:
    """Per-function bookkeeping of a basis: atom, shell (l, index on the atom), offsets."""
    basis: symmetry.Basis
    shells: List[Tuple[int, int, int, int]] = field(default_factory=list)  # (atom, shell index, l, offset)

    def __post_init__(self):
        off = 0
        for a, sh in enumerate(self.basis.shells):
            for s, l in enumerate(sh):
                self.shells.append((a, s, l, off))
                off += 2 * l + 1


def atom_species(basis: symmetry.Basis, ops) -> np.ndarray:
    """Orbit index of every atom under the space group ((M, t) on fractional
    coordinates); atoms of an orbit share shells and parameters."""
    pos = np.asarray(basis.positions, dtype=float)
    sp = -np.ones(len(pos), dtype=int)
    n = 0
    for a in range(len(pos)):
        if sp[a] >= 0:
            continue
        for M, t in ops:
            ra = M @ pos[a] + t
            for b in range(len(pos)):
                d = ra - pos[b]
                if sp[b] < 0 and np.allclose(d, np.round(d), atol=1e-9):
                    sp[b] = n
        n += 1
    return sp


def _lattice_vectors(A: np.ndarray, rmax: float) -> Tuple[np.ndarray, np.ndarray]:
    """Integer coordinates n and vectors L = A n (columns of A: primitive
    vectors) with |L| <= rmax."""
    m = int(np.ceil(rmax * np.linalg.norm(np.linalg.inv(A), 2))) + 2
    rng = np.arange(-m, m + 1)
    n = np.array(list(itertools.product(rng, rng, rng)))
    L = n @ A.T
    keep = np.linalg.norm(L, axis=1) <= rmax + 1e-9
    return n[keep], L[keep]


def _fractional(basis: symmetry.Basis, A: np.ndarray) -> symmetry.Basis:
    return symmetry.Basis(np.linalg.solve(A, np.asarray(basis.positions, dtype=float).T).T, basis.shells)


class _Generator:
    """The crystal's space group in one form for both lattices: operations
    (M, t) on fractional coordinates (O_h on the FCC primitive vectors with
    t = 0; P6_3mc with its screw and glide translations), k in reduced
    reciprocal coordinates transforming as inv(M)^T k, and the representation
    on Bloch sums from ``symmetry.sg_bloch_representation``."""

    def __init__(self, spec: CrystalSpec, model: OrbitalModel):
        self.spec, self.model = spec, model
        if spec.lattice == "fcc":
            self.A = symmetry.FCC_A
            Ainv = np.linalg.inv(self.A)
            self.ops = [(np.round(Ainv @ R @ self.A).astype(int), np.zeros(3)) for R in symmetry.oh_operations()]
            self.ao = _fractional(symmetry.fcc_basis(spec.nao, spec.atoms), self.A)
            self.aux = _fractional(symmetry.fcc_basis(spec.naux, spec.atoms), self.A)
            self.a_lat = model.a_lat
        elif spec.lattice == "hex":
            self.A = symmetry.HEX_A
            self.ops = symmetry.p63mc_operations()
            self.ao, self.aux = symmetry.wurtzite_basis(spec.nao), symmetry.wurtzite_basis(spec.naux)
            self.a_lat = model.a_lat_hex
        else:
            raise ValueError(f"unknown lattice {spec.lattice!r}")
        self.ops_k = [np.round(np.linalg.inv(M).T).astype(int) for M, _ in self.ops]
        self.kmesh = _kmesh(spec.mesh)
        self.nk = nk = len(self.kmesh)
        inversion = any(np.array_equal(K, -np.eye(3, dtype=int)) for K in self.ops_k)
        self.inv_op = next((g for g, K in enumerate(self.ops_k) if np.array_equal(K, -np.eye(3, dtype=int))), None)
        self.reps, self.star_of, self.index, self.conj_index = _stars(self.kmesh, self.ops_k, inversion)
        self.minus = np.array([_find(wrap_1stbz(-self.kmesh[k]), self.kmesh) for k in range(nk)])
        self.perm = np.array([[_find(wrap_1stbz(K @ k), self.kmesh) for k in self.kmesh] for K in self.ops_k])
        # the operation taking each point-group-reached k from its representative
        self.op_of = np.array([next(g for g in range(len(self.ops)) if self.perm[g][self.index[k]] == k)
                               if self.conj_index[k] == k else -1 for k in range(nk)])
        # per representative: an operation taking k_r to -k_r (inversion first), if the point group has one
        self.minus_op = {}
        for kr in self.reps:
            cands = [g for g in range(len(self.ops)) if self.perm[g][kr] == self.minus[kr]]
            self.minus_op[kr] = (self.inv_op if self.inv_op in cands else cands[0]) if cands else None
        self._dcache = {}
        self.species = atom_species(self.ao, self.ops)
        rng = np.random.default_rng(model.seed + spec.seed)
        self.coef = rng.uniform(0.5, 1.5, size=len(self.ops))  # c_h, one per group operation
        self.par_rng = rng

    # -- group helpers ----------------------------------------------------- #
    def little_group(self, k: int) -> List[int]:
        return [g for g in range(len(self.ops)) if self.perm[g][k] == k]

    def D(self, g: int, k: int, basis: symmetry.Basis, then: int = None) -> np.ndarray:
        """Representation on the Bloch sums at k of operation g, or of the
        product g u when ``then`` = u (u applied first); cached per operation,
        k and basis."""
        key = (g, k, id(basis), then)
        if key not in self._dcache:
            M, t = self.ops[g]
            if then is not None:
                Mu, tu = self.ops[then]
                M, t = M @ Mu, M @ tu + t
            self._dcache[key] = symmetry.sg_bloch_representation(self.kmesh[k], M, t, basis, self.A)
        return self._dcache[key]

    def adapted_basis(self, k: int, basis: symmetry.Basis) -> Tuple[np.ndarray, List[int]]:
        """Eigenvectors of A = B + Theta(B), B = sum_h c_h (D(h) + D(h)^H) over
        the little group of k, grouped by eigenvalue: (U, block sizes).
        Theta(B) = D(u)^H conj(B) D(u) for an operation u taking k to -k (B
        alone when there is none) makes conj(U) and D(u) U span the same
        eigenspaces in the same order, which the aux bases at q and -q need."""
        B = sum(self.coef[h] * (Dh + Dh.conj().T) for h in self.little_group(k)
                for Dh in [self.D(h, k, basis)])
        u = self.minus_op.get(k)
        if u is not None:
            Du = self.D(u, k, basis)
            B = B + Du.conj().T @ B.conj() @ Du
        if self.minus[k] == k:           # self-conjugate: a real matrix, real eigenvectors
            assert np.abs(B.imag).max() < 1e-10
            w, U = np.linalg.eigh(B.real)
        else:
            w, U = np.linalg.eigh(B)
        scale = max(1.0, np.abs(w).max())
        sizes, i = [], 0
        while i < len(w):
            j = i + 1
            while j < len(w) and w[j] - w[i] < 1e-8 * scale:
                j += 1
            sizes.append(j - i)
            i = j
        return U.astype(np.complex128), sizes

    # -- parameters -------------------------------------------------------- #
    def shell_parameters(self):
        m, rng = self.model, self.par_rng
        ao_sh = _Shells(self.ao)
        aux_sh = _Shells(self.aux)
        keys_ao = sorted({(int(self.species[a]), s) for (a, s, _, _) in ao_sh.shells})
        keys_aux = sorted({(int(self.species[a]), s) for (a, s, _, _) in aux_sh.shells})
        onsite = {k: rng.normal(0.0, m.onsite) for k in keys_ao}
        ao_exp = {k: rng.uniform(*m.ao_exponents) for k in keys_ao}
        aux_exp = {k: rng.uniform(*m.aux_exponents) for k in keys_aux}
        hop = {}
        for i, ki in enumerate(keys_ao):
            for kj in keys_ao[i:]:
                hop[(ki, kj)] = rng.uniform(-m.hopping, m.hopping, size=3)
        return ao_sh, aux_sh, onsite, ao_exp, aux_exp, hop

    def _cart(self, basis: symmetry.Basis) -> np.ndarray:
        """Atom positions in Cartesian coordinates (units of the lattice constant)."""
        return np.asarray(basis.positions, dtype=float) @ self.A.T

    def neighbour_distances(self, n: int) -> np.ndarray:
        """The n smallest distinct interatomic distances (bohr)."""
        pos = self._cart(self.ao)
        _, L = _lattice_vectors(self.A, 3.0)
        d = np.linalg.norm(pos[None, :, None, :] + L[None, None, :, :] - pos[:, None, None, :], axis=-1)
        d = np.sort(d[d > 1e-9].ravel())
        shells = [d[0]]
        for x in d[1:]:
            if x > shells[-1] * (1 + 1e-6):
                shells.append(x)
            if len(shells) == n:
                break
        return np.array(shells[:n]) * self.a_lat

    # -- F(k) in the orbital Bloch basis ----------------------------------- #
    def fock_ao(self, ao_sh, onsite, hop) -> np.ndarray:
        m, nao = self.model, self.spec.nao
        pos = self._cart(self.ao)
        shells = self.neighbour_distances(m.neighbour_shells)
        d_nn, cutoff = shells[0], shells[-1] * (1 + 1e-6)
        nvec, Lvec = _lattice_vectors(self.A, cutoff / self.a_lat + 2.0)
        phase = np.exp(2j * np.pi * (self.kmesh @ nvec.T))     # (nk, nL)
        blocks = np.zeros((len(nvec), nao, nao))
        for (ai, si, li, oi) in ao_sh.shells:
            ki = (int(self.species[ai]), si)
            for (aj, sj, lj, oj) in ao_sh.shells:
                kj = (int(self.species[aj]), sj)
                if ki <= kj:
                    v = hop[(ki, kj)]
                else:
                    v = hop[(kj, ki)] * (-1.0) ** (li + lj)
                for n in range(len(nvec)):
                    d = (pos[aj] + Lvec[n] - pos[ai]) * self.a_lat
                    r = np.linalg.norm(d)
                    if r < 1e-9 or r > cutoff:
                        continue
                    blocks[n, oi:oi + 2 * li + 1, oj:oj + 2 * lj + 1] = sk_block(
                        li, lj, v * np.exp(-(r - d_nn) / m.decay), d)
        F = np.einsum("kn,nij->kij", phase, blocks)
        for (a, s, l, o) in ao_sh.shells:
            F[:, np.arange(o, o + 2 * l + 1), np.arange(o, o + 2 * l + 1)] += onsite[(int(self.species[a]), s)]
        return F

    # -- V(k1, k2) in the orbital / aux Bloch bases ------------------------- #
    def coulomb_ao(self, ao_sh, aux_sh, ao_exp, aux_exp) -> np.ndarray:
        """(nk * nk, naux, nao, nao): V^Q_ij(k1, k2) for every pair, p = k2 - k1."""
        m, nk = self.model, self.nk
        naux, nao = self.spec.naux, self.spec.nao
        rc = m.v_cutoff
        pos_ao, pos_aux = self._cart(self.ao), self._cart(self.aux)
        nvec, Lvec = _lattice_vectors(self.A, rc + 2.0)
        natom = len(pos_ao)
        k1 = np.repeat(np.arange(nk), nk)
        k2 = np.tile(np.arange(nk), nk)
        kf1, kf2 = self.kmesh[k1], self.kmesh[k2]
        V = np.zeros((nk * nk, naux, nao, nao), dtype=np.complex128)
        aux_by_atom = {a: [x for x in aux_sh.shells if x[0] == a] for a in range(natom)}
        ao_by_atom = {a: [x for x in ao_sh.shells if x[0] == a] for a in range(natom)}
        norm_ao = {x: shell_norm(ao_exp[(int(self.species[x[0]]), x[1])], x[2]) for x in ao_sh.shells}
        norm_aux = {x: shell_norm(aux_exp[(int(self.species[x[0]]), x[1])], x[2]) for x in aux_sh.shells}
        for aq in range(natom):
            for ai in range(natom):
                for aj in range(natom):
                    A_i = pos_ao[ai]
                    cq = pos_aux[aq] + Lvec
                    cj = pos_ao[aj] + Lvec
                    iq = np.where(np.linalg.norm(cq - A_i, axis=1) <= rc + 1e-9)[0]
                    ij = np.where(np.linalg.norm(cj - A_i, axis=1) <= rc + 1e-9)[0]
                    if len(iq) == 0 or len(ij) == 0:
                        continue
                    gq, gj = np.meshgrid(iq, ij, indexing="ij")
                    gq, gj = gq.ravel(), gj.ravel()
                    ok = np.linalg.norm(cq[gq] - cj[gj], axis=1) <= rc + 1e-9
                    gq, gj = gq[ok], gj[ok]
                    AQ, AJ = cq[gq] * self.a_lat, cj[gj] * self.a_lat
                    AI = np.broadcast_to(A_i * self.a_lat, AQ.shape)
                    ph = np.exp(2j * np.pi * (-(kf2 - kf1) @ nvec[gq].T + kf2 @ nvec[gj].T))  # (pairs, conf)
                    for xq in aux_by_atom[aq]:
                        eq = aux_exp[(int(self.species[aq]), xq[1])]
                        for xi in ao_by_atom[ai]:
                            ei = ao_exp[(int(self.species[ai]), xi[1])]
                            for xj in ao_by_atom[aj]:
                                ej = ao_exp[(int(self.species[aj]), xj[1])]
                                T = three_centre(AQ, eq, xq[2], AI, ei, xi[2], AJ, ej, xj[2])
                                T *= norm_aux[xq] * norm_ao[xi] * norm_ao[xj]
                                nq, ni, nj = T.shape[1:]
                                blk = (ph @ T.reshape(len(T), -1)).reshape(-1, nq, ni, nj)
                                V[:, xq[3]:xq[3] + nq, xi[3]:xi[3] + ni, xj[3]:xj[3] + nj] += blk
        return V

    # -- the selection rule -------------------------------------------------- #
    def selection_rule(self, p: int, adapted, rng) -> np.ndarray:
        """A generic V(k1, k2) invariant under the pair's magnetic stabiliser, in
        the adapted bases (normalised to max 1): the operations h that fix k1
        and k2 act as V -> (D_aux(h, p) x D(h, k1) x conj D(h, k2)) V = T_h V,
        and time reversal after an operation g that takes the pair to
        (-k1, -k2) (real orbitals give V(-k1, -k2) = conj(V(k1, k2))) as
        V -> conj(T_g V).  Its zero blocks are the blocks the group forbids."""
        k1, k2 = divmod(p, self.nk)
        kq = _find(wrap_1stbz(self.kmesh[k2] - self.kmesh[k1]), self.kmesh)
        ng = len(self.ops)
        unitary = [g for g in range(ng) if self.perm[g][k1] == k1 and self.perm[g][k2] == k2]
        anti = [g for g in range(ng) if self.perm[g][k1] == self.minus[k1] and self.perm[g][k2] == self.minus[k2]]
        X = rng.normal(size=(self.spec.naux, self.spec.nao, self.spec.nao)) \
            + 1j * rng.normal(size=(self.spec.naux, self.spec.nao, self.spec.nao))
        acc = np.zeros_like(X)
        for g, conj in [(g, False) for g in unitary] + [(g, True) for g in anti]:
            T = np.matmul(np.matmul(self.D(g, k1, self.ao), np.tensordot(self.D(g, kq, self.aux), X, 1)),
                          self.D(g, k2, self.ao).conj().T)
            acc += T.conj() if conj else T
        out = adapted(p, acc)
        return out / np.abs(out).max()

    # -- bases and rotations ------------------------------------------------ #
    def bases(self, rng):
        """AO bases U[k], aux bases Y[q] (full matrices), block sizes per k / q,
        and the full rotation matrices orep[k] = U[k]^H D U[k_r], auxrep[q].
        A k that time reversal brings into the star (conj_index[k] = k' != k,
        k = -k') takes conj(U[k']) and the rotation of k': the rotation path
        conjugates G and P~ there."""
        nk = self.nk
        U, Y, ao_sizes, aux_sizes = [None] * nk, [None] * nk, [None] * nk, [None] * nk
        orep, auxrep = [None] * nk, [None] * nk
        rep_ao = {kr: self.adapted_basis(kr, self.ao) for kr in self.reps}
        rep_aux = {kr: self.adapted_basis(kr, self.aux) for kr in self.reps}

        def gauge(sizes, real):
            blocks = []
            for b in sizes:
                if real:
                    q, r = np.linalg.qr(rng.normal(size=(b, b)))
                    blocks.append((q * np.sign(np.diag(r))[None, :]).astype(np.complex128))
                else:
                    blocks.append(_rand_unitary(rng, b))
            return _block_diag(blocks)

        by_group = [k for k in range(nk) if self.conj_index[k] == k]
        by_tr = [k for k in range(nk) if self.conj_index[k] != k]
        for k in by_group:
            kr = int(self.index[k])
            Ur, sz = rep_ao[kr]
            Dg = self.D(int(self.op_of[k]), kr, self.ao)
            W = np.eye(len(Ur), dtype=np.complex128) if k == kr else gauge(sz, False)
            U[k] = Dg @ Ur @ W
            ao_sizes[k] = list(sz)
            orep[k] = U[k].conj().T @ Dg @ Ur
        for q in by_group:
            if Y[q] is not None:
                continue
            qr = int(self.index[q])
            Yr, sz = rep_aux[qr]
            g = int(self.op_of[q])
            Dg = self.D(g, qr, self.aux)
            W = np.eye(len(Yr), dtype=np.complex128) if q == qr else gauge(sz, self.minus[q] == q)
            Y[q] = Dg @ Yr @ W
            aux_sizes[q] = list(sz)
            auxrep[q] = Y[q].conj().T @ Dg @ Yr
            mq = int(self.minus[q])
            if mq != q and self.conj_index[mq] == mq:   # -q in the star by the group: g u takes q_r there
                assert self.index[mq] == qr and Y[mq] is None and self.minus_op[qr] is not None
                Y[mq] = Y[q].conj()
                aux_sizes[mq] = list(sz)
                auxrep[mq] = Y[mq].conj().T @ self.D(g, qr, self.aux, then=self.minus_op[qr]) @ Yr
        for k in by_tr:
            c = int(self.conj_index[k])
            U[k], ao_sizes[k], orep[k] = U[c].conj(), list(ao_sizes[c]), orep[c]
            Y[k], aux_sizes[k], auxrep[k] = Y[c].conj(), list(aux_sizes[c]), auxrep[c]
        return U, Y, ao_sizes, aux_sizes, orep, auxrep


def _block_diag(blocks) -> np.ndarray:
    n = sum(b.shape[0] for b in blocks)
    out = np.zeros((n, n), dtype=np.complex128)
    o = 0
    for b in blocks:
        out[o:o + b.shape[0], o:o + b.shape[0]] = b
        o += b.shape[0]
    return out


def _diag_blocks(M: np.ndarray, sizes) -> Tuple[List[np.ndarray], float]:
    """The diagonal blocks of M and the largest entry outside them."""
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(int)
    mask = np.ones(M.shape, dtype=bool)
    out = []
    for i in range(len(sizes)):
        a, b = offs[i], offs[i + 1]
        out.append(M[a:b, a:b].copy())
        mask[a:b, a:b] = False
    return out, float(np.abs(M[mask]).max()) if mask.any() else 0.0


@dataclass
class OrbitalCrystal(Crystal):
    """A Crystal plus the data in the orbital Bloch bases and the adapted bases,
    for checks: U[k], Y[q] (columns = adapted functions), F_ao[k], V_ao[pair]."""
    U: List[np.ndarray] = None
    Y: List[np.ndarray] = None
    F_ao: np.ndarray = None
    V_ao: np.ndarray = None
    V_block_norms: Dict = None     # (pair, iq, i1, i2) -> max |V| of every candidate block
    off_block: Dict = None         # largest off-block entries of F, orep, auxrep in the adapted bases
    p0_transports: Dict = None     # (k, q_irr) -> (k_r or -k_r - 1, q', A): see vstore.p0_from_stored_pairs


def p0_transports(gen: _Generator, Y, irre_list) -> Dict:
    """For every k of the mesh and irreducible q: the stored pair (k_r, q')
    and the aux transport A with c(k, q) = A c(k_r, q') A^H, where k = g k_r
    (g the operation that brings k into its star), q' = g^-1 q and
    A = Y(q)^H D_aux(g, q') Y(q').  A time-reversal partner k = -k'' uses
    c(k, q) = conj(c(k'', -q)) and is returned as (-k_r - 1, q', conj(A))."""
    inv_perm = np.argsort(gen.perm, axis=1)          # inv_perm[g][q] = g^-1 q
    out = {}
    for q in (int(x) for x in irre_list):
        for k in range(gen.nk):
            tr = gen.conj_index[k] != k
            kk, qq = (int(gen.minus[k]), int(gen.minus[q])) if tr else (k, q)
            g = int(gen.op_of[kk])
            qp = int(inv_perm[g][qq])
            A = Y[qq].conj().T @ gen.D(g, qp, gen.aux) @ Y[qp]
            kr = int(gen.index[kk])
            out[(k, q)] = (-kr - 1, qp, A.conj()) if tr else (kr, qp, A)
    return out


def make_orbital_crystal(spec: CrystalSpec, rotate: bool = True, model: OrbitalModel = None,
                         keep_ao_data: bool = False, transports: bool = False) -> OrbitalCrystal:
    """Build the crystal (module docstring).  ``rotate=False`` stores every k
    point with identity rotations (same bases, V and F as ``rotate=True``).
    ``keep_ao_data`` keeps F and V in the orbital Bloch bases for checks;
    ``transports`` (with ``rotate``) adds the aux transports that P0 needs to
    read only the pairs with an irreducible first k (``vstore``)."""
    model = OrbitalModel() if model is None else model
    gen = _Generator(spec, model)
    nk = gen.nk
    ao_sh, aux_sh, onsite, ao_exp, aux_exp, hop = gen.shell_parameters()
    F_ao = gen.fock_ao(ao_sh, onsite, hop)
    V_ao = gen.coulomb_ao(ao_sh, aux_sh, ao_exp, aux_exp)
    U, Y, ao_sizes, aux_sizes, orep_full, auxrep_full = gen.bases(np.random.default_rng(model.seed + spec.seed + 1))
    off = {"F": 0.0, "orep": 0.0, "auxrep": 0.0}

    # V in the adapted bases; the blocks that the group forbids are left out
    layout0 = BlockLayout(nk=nk, kmesh=gen.kmesh, ao_sizes=ao_sizes, aux_sizes=aux_sizes,
                          tensor_irreps=[np.zeros((0, 3), int)] * (nk * nk),
                          irre_list=np.arange(nk), index=np.arange(nk), irre_index=np.arange(nk),
                          conj_index=np.arange(nk))

    def adapted(p, X):
        """conj(Y(q))^T x conj(U(k1))^T x U(k2)^T applied to V(k1, k2)[Q', i', j']."""
        k1, k2 = divmod(p, nk)
        x = np.tensordot(Y[layout0.pair_q(k1, k2)].conj().T, X, 1)
        return np.matmul(np.matmul(U[k1].conj().T, x), U[k2])

    if keep_ao_data:
        Vsa = np.stack([adapted(p, V_ao[p]) for p in range(nk * nk)])
    else:                                   # in place: one copy of the largest array
        Vsa = V_ao
        for p in range(nk * nk):
            Vsa[p] = adapted(p, V_ao[p])
        V_ao = None
    vmax = float(np.abs(Vsa).max())
    norms, ti = {}, []
    ao_off = [np.concatenate([[0], np.cumsum(s)]).astype(int) for s in ao_sizes]
    aux_off = [np.concatenate([[0], np.cumsum(s)]).astype(int) for s in aux_sizes]
    off["V_forbidden"] = 0.0
    for p in range(nk * nk):
        k1, k2 = divmod(p, nk)
        q = layout0.pair_q(k1, k2)
        allowed = gen.selection_rule(p, adapted, np.random.default_rng((model.seed, p)))
        blocks = []
        for iq in range(len(aux_sizes[q])):
            for i1 in range(len(ao_sizes[k1])):
                for i2 in range(len(ao_sizes[k2])):
                    sl = (slice(aux_off[q][iq], aux_off[q][iq + 1]), slice(ao_off[k1][i1], ao_off[k1][i1 + 1]),
                          slice(ao_off[k2][i2], ao_off[k2][i2 + 1]))
                    n = float(np.abs(Vsa[p][sl]).max()) / vmax
                    norms[(p, iq, i1, i2)] = n
                    if np.abs(allowed[sl]).max() > 1e-12:
                        blocks.append((iq, i1, i2))
                    else:
                        off["V_forbidden"] = max(off["V_forbidden"], n)
        ti.append(np.array(blocks, dtype=np.int32).reshape(-1, 3))

    # rotations (block-diagonal) and the stored k points
    if rotate:
        irre_list = np.array(gen.reps)
        pos = {int(k): i for i, k in enumerate(irre_list)}
        irre_index = np.array([pos[int(gen.index[gen.conj_index[k]])] for k in range(nk)])
        idx, cidx = gen.index.copy(), gen.conj_index.copy()
        orep_b, orep_i, auxrep_b, auxrep_i = [], [], [], []
        for k in range(nk):
            ob, e = _diag_blocks(orep_full[k], ao_sizes[k])
            off["orep"] = max(off["orep"], e)
            ab, e = _diag_blocks(auxrep_full[k], aux_sizes[k])
            off["auxrep"] = max(off["auxrep"], e)
            orep_b += [b.ravel() for b in ob]
            auxrep_b += [b.ravel() for b in ab]
            orep_i.append(np.stack([np.arange(len(ob)), np.arange(len(ob))], 1))
            auxrep_i.append(np.stack([np.arange(len(ab)), np.arange(len(ab))], 1))
        reps_kw = dict(orep=np.concatenate(orep_b), orep_irreps=orep_i,
                       auxrep=np.concatenate(auxrep_b), auxrep_irreps=auxrep_i)
    else:
        irre_list, irre_index, idx, cidx = np.arange(nk), np.arange(nk), np.arange(nk), np.arange(nk)
        reps_kw = {}
    layout = BlockLayout(nk=nk, kmesh=gen.kmesh, ao_sizes=ao_sizes, aux_sizes=aux_sizes, tensor_irreps=ti,
                         irre_list=irre_list, index=idx, irre_index=irre_index, conj_index=cidx,
                         **reps_kw)

    # flat V, scaled to the spec's entry size
    V = np.zeros(layout.flat_V_size, dtype=np.complex128)
    for p in range(nk * nk):
        k1, k2 = divmod(p, nk)
        q = layout.pair_q(k1, k2)
        base = layout.kpair_slice_offsets[p]
        for b, (iq, i1, i2) in enumerate(layout.tensor_irreps[p]):
            blk = Vsa[p, aux_off[q][iq]:aux_off[q][iq + 1], ao_off[k1][i1]:ao_off[k1][i1 + 1],
                      ao_off[k2][i2]:ao_off[k2][i2 + 1]]
            o = base + layout.tensor_offsets[p][b]
            V[o:o + blk.size] = blk.ravel()
    scale = (spec.v_scale / np.sqrt(spec.nao)) / np.sqrt(np.mean(np.abs(V) ** 2))
    V *= scale

    # F, S, H on the stored k points, in the adapted bases
    ns, fa = spec.ns, layout.flat_ao_size
    F = np.zeros((ns, fa), np.complex128)
    S = np.zeros((ns, fa), np.complex128)
    star_size = np.bincount(gen.star_of, minlength=len(gen.reps))
    eigs = []
    for ik, k in enumerate(layout.irre_list):
        fk, e = _diag_blocks(U[k].conj().T @ F_ao[k] @ U[k], ao_sizes[k])
        off["F"] = max(off["F"], e)
        for b, h in enumerate(fk):
            h = 0.5 * (h + h.conj().T)
            o = layout.kao_slice_offsets_irre[ik] + layout.ao_offsets[k][b]
            for sp in range(ns):
                F[sp, o:o + h.size] = h.ravel()
                S[sp, o:o + h.size] = np.eye(h.shape[0]).ravel()
            if k in gen.reps:  # mu from the representatives with their star weights, for both modes
                eigs.extend([(ev, star_size[gen.star_of[k]]) for ev in np.linalg.eigvalsh(h)])
    mu = half_filling_mu(eigs, spec.nao, nk)
    return OrbitalCrystal(spec=spec, layout=layout, V=V, F=F, S=S, H=F.copy(), mu=float(mu),
                          star_sizes=np.array([star_size[gen.star_of[k]] for k in layout.irre_list]),
                          p0_transports=p0_transports(gen, Y, layout.irre_list) if transports and rotate else None,
                          U=U, Y=Y, F_ao=F_ao if keep_ao_data else None,
                          V_ao=V_ao * scale if keep_ao_data else None, V_block_norms=norms, off_block=off)

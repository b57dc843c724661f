"""Seeded synthetic crystals in the irrep-blocked layout.

The reference's inputs come from PySCF (Gaussian density fitting) plus
SymmetryAdaptation's block diagonalisation (``scripts/integrals/
init_data_full_block.py``, ``SymmetryAdaptation/src/dirac_character.cpp``);
neither PySCF nor the benchmark crystals exist here, so this module builds
inputs with the same *layout and symmetry structure* from seeded random
numbers:

* k mesh: Gamma-centred n1 x n2 x n3 grid in reduced coordinates of the
  reciprocal lattice; stars under the crystal's point group (Oh for an fcc
  lattice, C6v for a hexagonal one, plus time reversal k -> -k when the
  group has no inversion); irreducible list, ``index``, ``irre_index`` and
  ``conj_index`` exactly as ``symmetry_utils_t`` defines them
  (``SymmetryMBPT/src/common/symmetry_utils.cpp:41-94``).
* irrep blocks ("labelled blocks"): every star gets a partition of the AO
  and aux spaces into blocks whose mean size shrinks with the order of the
  little group; each block carries a label in Z_4.  Aux blocks of q and -q
  are equal with opposite labels.
* V^Q_ij(k1, k2): block (iq, i1, i2) of pair (k1, k2), q = k2 - k1, is
  non-zero iff label(q, iq) + label(k2, i2) = label(k1, i1) (mod 4) -- the
  abelian stand-in for the selection rule Gamma_Q x Gamma_j contains
  Gamma_i.  Entries are complex Gaussians; V(k2, k1)_{Q,j,i} =
  conj(V(k1, k2)_{Q,i,j}) is enforced (the Hermitian pair relation of
  density-fitted integrals).
* F(k): random Hermitian blocks (band width ~ a few Ha, on-site N(0, 0.5));
  S = I; H = F.
* orep / auxrep: a random unitary per block for every non-representative k.
* mu: half filling of the G0 bands (nel = nao per spin-summed cell).

``symmetric=True`` (fcc) builds data that are exactly consistent with the
group, so that a calculation on the irreducible k points with rotations and
one on every k point of the mesh give the same P0, P~ and Sigma (the
reference's iBZ-vs-full-BZ checks, ``SymmetryMBPT/test/test_cugw.cpp:306-436``):

* gauge 0: V0(k1, k2) is the same on every orbit of pairs under the point
  group (g k1, g k2), with V0(k2, k1)_{Q,j,i} = conj(V0(k1, k2)_{Q,i,j}) on
  the swapped orbit (averaged over the stabiliser when a group operation
  swaps the pair), and F0(k) is the same on every star;
* every k and q gets a basis change, a random unitary per irrep block
  (W_k for AO, X_q for aux; the identity at the representatives, and
  X_{-q} = conj(X_q) so that the Hermitian pair relation survives);
* the data are the gauge-0 data in those bases, V^Q(k1, k2) =
  sum_Q' X_q[Q, Q'] W_k1 V0^Q'(k1, k2) W_k2^H and F(k) = W_k F0 W_k^H, and
  the rotations are orep(k) = W_k, auxrep(q) = X_q: a representation of the
  group in which every datum transforms covariantly.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass
from typing import Dict, List, Optional, Tuple

import numpy as np

from .layout import BlockLayout, wrap_1stbz


# --------------------------------------------------------------------------- #
# point groups in reduced reciprocal coordinates
# --------------------------------------------------------------------------- #
def _fcc_ops() -> Tuple[List[np.ndarray], bool]:
    A = 0.5 * np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]], dtype=float)  # rows: direct vectors
    Bt = np.linalg.inv(A)  # columns: reciprocal vectors (no 2 pi)
    ops = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            R = np.zeros((3, 3))
            for i, p in enumerate(perm):
                R[i, p] = signs[i]
            M = np.linalg.inv(Bt) @ R @ Bt
            ops.append(np.round(M).astype(int))
    return ops, True  # Oh contains inversion


def _hex_ops() -> Tuple[List[np.ndarray], bool]:
    c = 1.633
    A = np.array([[1.0, 0, 0], [-0.5, np.sqrt(3) / 2, 0], [0, 0, c]])
    Bt = np.linalg.inv(A)
    ops = []
    for n in range(6):
        th = n * np.pi / 3
        Rz = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
        for mirror in (False, True):
            R = Rz @ np.diag([1, -1, 1]) if mirror else Rz
            M = np.linalg.inv(Bt) @ R @ Bt
            ops.append(np.round(M).astype(int))
    return ops, False  # C6v has no inversion


@dataclass
class CrystalSpec:
    name: str
    lattice: str                 # "fcc" or "hex"
    mesh: Tuple[int, int, int]
    nao: int
    naux: int
    nts: int
    beta: float
    ns: int = 1
    ao_block: Tuple[int, int] = (1, 8)
    aux_block: Tuple[int, int] = (2, 40)
    seed: int = 20260101
    v_scale: float = 0.5
    atoms: int = 2               # atoms per cell (physical block sizes, fcc only)


#: The five benchmark crystals C1-C5 (their shapes, block-size ranges and V storage).
CONFIGS: Dict[str, CrystalSpec] = {
    "C1": CrystalSpec("C1", "fcc", (3, 3, 3), 8, 36, 62, 50.0, ao_block=(1, 4), aux_block=(2, 12), seed=20260101),
    "C2": CrystalSpec("C2", "fcc", (3, 3, 3), 26, 120, 100, 100.0, ao_block=(1, 8), aux_block=(2, 40), seed=20260102),
    "C3": CrystalSpec("C3", "fcc", (4, 4, 4), 52, 250, 120, 100.0, ao_block=(2, 16), aux_block=(4, 64), seed=20260103, atoms=4),
    "C4": CrystalSpec("C4", "hex", (4, 4, 3), 72, 350, 120, 200.0, ao_block=(2, 30), aux_block=(2, 30), seed=20260104),
    "C5": CrystalSpec("C5", "fcc", (5, 5, 5), 100, 500, 150, 200.0, ao_block=(4, 40), aux_block=(8, 64), seed=20260105, atoms=4),
    # profiling case: C3's orbitals, grid and block sizes on the 3x3x3 mesh (V ~2 GB
    # instead of 12 GB), small enough for multi-pass kernel captures
    "C3m": CrystalSpec("C3m", "fcc", (3, 3, 3), 52, 250, 120, 100.0, ao_block=(2, 16), aux_block=(4, 64),
                       seed=20260106, atoms=4),
}


@dataclass
class Crystal:
    spec: CrystalSpec
    layout: BlockLayout
    V: np.ndarray        # flat block V, all nk^2 pairs
    F: np.ndarray        # [ns][flat_ao]
    S: np.ndarray
    H: np.ndarray
    mu: float
    star_sizes: np.ndarray  # per irreducible k

    @property
    def ns(self):
        return self.spec.ns


def _kmesh(mesh):
    n1, n2, n3 = mesh
    pts = []
    for i in range(n1):
        for j in range(n2):
            for l in range(n3):
                pts.append([i / n1, j / n2, l / n3])
    return np.array(pts)


def _find(k, kmesh):
    d = np.abs(((kmesh - k[None, :]) + 0.5) % 1.0 - 0.5).max(axis=1)
    return int(np.argmin(d)) if d.min() < 1e-9 else -1


def _stars(kmesh, ops, inversion):
    """Stars under the group (+ time reversal when the group lacks inversion)."""
    nk = len(kmesh)
    star_of = -np.ones(nk, dtype=int)
    reps = []
    index = np.zeros(nk, dtype=int)       # representative (rotation partner)
    conj_index = np.arange(nk)
    for k in range(nk):
        if star_of[k] >= 0:
            continue
        s = len(reps)
        reps.append(k)
        for M in ops:
            kk = _find(wrap_1stbz(M @ kmesh[k]), kmesh)
            assert kk >= 0, "group operation does not map the mesh onto itself"
            if star_of[kk] < 0:
                star_of[kk] = s
                index[kk] = k
        if not inversion:
            for M in ops:
                kk = _find(wrap_1stbz(-(M @ kmesh[k])), kmesh)
                if star_of[kk] < 0:
                    star_of[kk] = s
                    # -Rk: rotation partner is Rk (a member of the star); conj maps to it
                    partner = _find(wrap_1stbz(M @ kmesh[k]), kmesh)
                    conj_index[kk] = partner
                    index[kk] = k
    return np.array(reps), star_of, index, conj_index


def _partition(rng, n, bmin, bmax, target):
    """Random composition of n into blocks within [bmin, bmax] near ``target``."""
    bmin = max(1, min(bmin, n))
    bmax = max(bmin, min(bmax, n))
    for _ in range(1000):
        sizes = []
        rest = n
        while rest > 0:
            lo = bmin
            hi = min(bmax, rest)
            if rest <= bmax:
                if rest >= bmin:
                    sizes.append(rest)
                    rest = 0
                    break
                sizes = None
                break
            mean = min(max(target, lo), hi)
            s = int(np.clip(round(rng.normal(mean, 0.35 * mean + 0.5)), lo, hi))
            if rest - s > 0 and rest - s < bmin:
                s = rest - bmin if rest - bmin >= lo else s
            sizes.append(s)
            rest -= s
        if sizes and sum(sizes) == n and all(bmin <= x <= bmax for x in sizes):
            rng.shuffle(sizes)
            return sizes
    raise RuntimeError(f"cannot partition {n} into blocks of {bmin}..{bmax}")


def _rand_unitary(rng, n):
    z = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))[None, :]


def _symmetric_V(spec, layout, kmesh, ops, Wk, Xq, sigma, V):
    """Group-consistent V (module docstring): gauge-0 blocks per orbit of pairs
    under the point group and the swap, then the per-k / per-q bases."""
    nk = layout.nk
    perm = np.array([[_find(wrap_1stbz(M @ kmesh[k]), kmesh) for k in range(nk)] for M in ops])
    src = {}  # pair -> (representative pair, swapped)
    sym = {}  # representative -> some operation swaps it onto itself
    for k1 in range(nk):
        for k2 in range(nk):
            if (k1, k2) in src:
                continue
            r = (k1, k2)
            sym[r] = False
            for g in range(len(ops)):
                a, b = int(perm[g][k1]), int(perm[g][k2])
                src.setdefault((a, b), (r, False))
            for g in range(len(ops)):
                a, b = int(perm[g][k2]), int(perm[g][k1])
                if (a, b) == r:
                    sym[r] = True
                src.setdefault((a, b), (r, True))

    def blocks_of(k1, k2):
        p = k1 * nk + k2
        return p, {tuple(int(x) for x in t): i for i, t in enumerate(layout.tensor_irreps[p])}

    V0 = {}
    for r in sym:  # representatives in pair order (deterministic streams)
        k1, k2 = r
        p, idx = blocks_of(k1, k2)
        q = layout.pair_q(k1, k2)
        vrng = np.random.default_rng((spec.seed + 29, p))
        blk = {}
        for t in layout.tensor_irreps[p]:
            iq, i1, i2 = (int(x) for x in t)
            qb, b1, b2 = layout.aux_sizes[q][iq], layout.ao_sizes[k1][i1], layout.ao_sizes[k2][i2]
            blk[(iq, i1, i2)] = sigma * (vrng.normal(size=(qb, b1, b2)) + 1j * vrng.normal(size=(qb, b1, b2))) / np.sqrt(2)
        if sym[r]:  # an operation maps (k2, k1) onto (k1, k2): V0 equals its swapped conjugate
            blk = {t: 0.5 * (x + blk[(t[0], t[2], t[1])].transpose(0, 2, 1).conj()) for t, x in blk.items()}
        V0[r] = blk
    for (k1, k2), (r, sw) in src.items():
        p, _ = blocks_of(k1, k2)
        q = layout.pair_q(k1, k2)
        base = layout.kpair_slice_offsets[p]
        for b, t in enumerate(layout.tensor_irreps[p]):
            iq, i1, i2 = (int(x) for x in t)
            x0 = V0[r][(iq, i2, i1)].transpose(0, 2, 1).conj() if sw else V0[r][(iq, i1, i2)]
            x = np.einsum("QR,ij,Rjl,ml->Qim", Xq[q][iq], Wk[k1][i1], x0, Wk[k2][i2].conj(), optimize=True)
            o = base + layout.tensor_offsets[p][b]
            V[o:o + x.size] = x.ravel()


def _gauge(rng, sizes):
    """A random unitary per irrep block (the block-diagonal basis change of one k)."""
    return [_rand_unitary(rng, int(b)) for b in sizes]


def make_crystal(spec: CrystalSpec, rotate: bool = True, used_pairs_only: bool = False,
                 with_V: bool = True, physical: bool = False, symmetric: bool = False) -> Crystal:
    """Build the crystal.  ``rotate=False`` keeps every k point (ink = nk,
    identity rotations), the reference's no-symmetry mode.

    ``used_pairs_only=True`` stores V blocks only for the k pairs a GW
    iteration reads -- (k1, k1 + q) for irreducible q (P0) and (k1, k2) for
    irreducible k1 (Sigma), with their Hermitian partners -- and leaves the
    other pair slices empty; the stored blocks are identical to the full
    crystal's (every pair draws from its own random stream).  ``with_V=False``
    skips V (an empty array): the layout and one-body data only, e.g. to size
    a configuration before generating it.  ``physical=True`` (fcc) takes the
    AO and aux block sizes of every star from the O_h irreps at its
    representative k (:mod:`symmetry`: d blocks of size m per irrep of
    dimension d and multiplicity m, for spec.atoms atoms with s/p/d shells)
    instead of drawing them in the spec's ranges (hex: from P6_3mc on the four
    wurtzite sites, with its projective representations); block labels and
    the V selection rule stay the labelled ones.  ``symmetric=True`` builds
    group-consistent data (module docstring); the same V, and F in the same
    bases, with ``rotate`` True or False."""
    if symmetric and spec.lattice != "fcc":
        raise ValueError("symmetric crystals are built for the fcc (O_h, with inversion) lattice")
    if symmetric and used_pairs_only:
        raise ValueError("symmetric crystals store V for every pair")
    rng = np.random.default_rng(spec.seed)
    ops, inversion = _fcc_ops() if spec.lattice == "fcc" else _hex_ops()
    kmesh = _kmesh(spec.mesh)
    nk = len(kmesh)
    reps, star_of, index, conj_index = _stars(kmesh, ops, inversion)
    nstar = len(reps)
    star_size = np.bincount(star_of, minlength=nstar)
    order = len(ops) * (1 if inversion else 2)
    little = order // star_size

    # q -> -q map on the mesh
    minus = np.array([_find(wrap_1stbz(-kmesh[k]), kmesh) for k in range(nk)])

    # --- blocks per star (AO) and per {star(q), star(-q)} (aux)
    ao_sizes_star, ao_labels_star, aux_sizes_star, aux_labels_star = {}, {}, {}, {}
    phys = None
    if physical:
        from . import symmetry
        if spec.lattice == "fcc":
            Bt = np.linalg.inv(0.5 * np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]], dtype=float))
            ops_c = symmetry.oh_operations()
            bao, baux = symmetry.fcc_basis(spec.nao, spec.atoms), symmetry.fcc_basis(spec.naux, spec.atoms)
            phys = {s: (np.array(symmetry.block_sizes(Bt @ kmesh[k], bao, ops_c)),
                        np.array(symmetry.block_sizes(Bt @ kmesh[k], baux, ops_c))) for s, k in enumerate(reps)}
        else:  # wurtzite, P6_3mc: projective representations at the zone boundary
            bao, baux = symmetry.wurtzite_basis(spec.nao), symmetry.wurtzite_basis(spec.naux)
            phys = {s: (np.array(symmetry.sg_block_sizes(kmesh[k], bao)),
                        np.array(symmetry.sg_block_sizes(kmesh[k], baux))) for s, k in enumerate(reps)}
    for s, k in enumerate(reps):
        g = little[s]
        shrink = 1.0 / np.sqrt(max(1.0, g / 2.0))
        t_ao = spec.ao_block[0] + (spec.ao_block[1] - spec.ao_block[0]) * shrink
        t_aux = spec.aux_block[0] + (spec.aux_block[1] - spec.aux_block[0]) * shrink
        sz = _partition(rng, spec.nao, spec.ao_block[0], spec.ao_block[1], t_ao) if phys is None else phys[s][0]
        ao_sizes_star[s] = np.array(sz)
        ao_labels_star[s] = rng.integers(0, 4, size=len(sz))
    for s, k in enumerate(reps):
        if s in aux_sizes_star:
            continue
        ms = star_of[minus[k]]
        g = little[s]
        shrink = 1.0 / np.sqrt(max(1.0, g / 2.0))
        t_aux = spec.aux_block[0] + (spec.aux_block[1] - spec.aux_block[0]) * shrink
        sz = (np.array(_partition(rng, spec.naux, spec.aux_block[0], spec.aux_block[1], t_aux)) if phys is None
              else phys[s][1])
        if ms == s:   # self-conjugate star: labels in {0, 2}
            lab = 2 * rng.integers(0, 2, size=len(sz))
            aux_sizes_star[s], aux_labels_star[s] = sz, lab
        else:
            lab = rng.integers(0, 4, size=len(sz))
            aux_sizes_star[s], aux_labels_star[s] = sz, lab
            aux_sizes_star[ms], aux_labels_star[ms] = sz.copy(), (-lab) % 4

    ao_sizes = [ao_sizes_star[star_of[k]] for k in range(nk)]
    ao_lab = [ao_labels_star[star_of[k]] for k in range(nk)]
    aux_sizes = [aux_sizes_star[star_of[k]] for k in range(nk)]
    aux_lab = [aux_labels_star[star_of[k]] for k in range(nk)]

    # --- which k are stored (iBZ) and the index maps
    if rotate:
        irre_list = reps.copy()
        pos = {k: i for i, k in enumerate(irre_list)}
        irre_index = np.array([pos[index[conj_index[k]]] for k in range(nk)])
        idx = index.copy()
        cidx = conj_index.copy()
    else:
        irre_list = np.arange(nk)
        irre_index = np.arange(nk)
        idx = np.arange(nk)
        cidx = np.arange(nk)

    # --- layout (V blocks by the label selection rule)
    q_of_pair = lambda k1, k2: None  # placeholder (layout computes it)  # noqa: E731
    tmp_layout = BlockLayout(nk=nk, kmesh=kmesh, ao_sizes=ao_sizes, aux_sizes=aux_sizes,
                             tensor_irreps=[np.zeros((0, 3), int)] * (nk * nk),
                             irre_list=irre_list, index=idx, irre_index=irre_index, conj_index=cidx)
    used = None
    if used_pairs_only:
        used = set()
        for q in irre_list:
            for k1 in range(nk):
                k2 = tmp_layout.mom_cons(k1, 0, int(q))
                used.update({(k1, k2), (k2, k1)})
        for k1 in irre_list:
            for k2 in range(nk):
                used.update({(int(k1), k2), (k2, int(k1))})
    ti = []
    for k1 in range(nk):
        for k2 in range(nk):
            q = tmp_layout.pair_q(k1, k2)
            blocks = []
            if used is not None and (k1, k2) not in used:
                ti.append(np.zeros((0, 3), dtype=np.int32))
                continue
            for iq, lq in enumerate(aux_lab[q]):
                for i1, l1 in enumerate(ao_lab[k1]):
                    for i2, l2 in enumerate(ao_lab[k2]):
                        if (lq + l2 - l1) % 4 == 0:
                            blocks.append((iq, i1, i2))
            ti.append(np.array(blocks, dtype=np.int32).reshape(-1, 3))

    # rotations: random unitary per block for non-representatives
    orep_blocks, orep_irreps, auxrep_blocks, auxrep_irreps = [], [], [], []
    Wk, Xq = None, None
    if symmetric:  # the basis changes of every k / q (identity at the representatives)
        grng = np.random.default_rng(spec.seed + 23)
        is_rep = np.zeros(nk, dtype=bool)
        is_rep[reps] = True
        Wk = [[np.eye(b) for b in ao_sizes[k]] if is_rep[k] else _gauge(grng, ao_sizes[k]) for k in range(nk)]
        Xq = [None] * nk
        for q in range(nk):
            if Xq[q] is not None:
                continue
            mq = int(minus[q])
            if is_rep[q] or is_rep[mq] or mq == q:
                Xq[q] = [np.eye(b) for b in aux_sizes[q]]
                Xq[mq] = [np.eye(b) for b in aux_sizes[mq]]
            else:
                Xq[q] = _gauge(grng, aux_sizes[q])
                Xq[mq] = [x.conj() for x in Xq[q]]
    for k in range(nk):
        rep_k = (idx[cidx[k]] == cidx[k])
        osz = ao_sizes[k]
        asz = aux_sizes[k]
        orep_irreps.append(np.stack([np.arange(len(osz)), np.arange(len(osz))], 1))
        auxrep_irreps.append(np.stack([np.arange(len(asz)), np.arange(len(asz))], 1))
        for i, b in enumerate(osz):
            u = np.eye(b) if rep_k else (Wk[k][i] if symmetric else _rand_unitary(rng, b))
            orep_blocks.append(u.ravel())
        for i, b in enumerate(asz):
            u = np.eye(b) if rep_k else (Xq[k][i] if symmetric else _rand_unitary(rng, b))
            auxrep_blocks.append(u.ravel())
    layout = BlockLayout(nk=nk, kmesh=kmesh, ao_sizes=ao_sizes, aux_sizes=aux_sizes, tensor_irreps=ti,
                         irre_list=irre_list, index=idx, irre_index=irre_index, conj_index=cidx,
                         orep=np.concatenate(orep_blocks).astype(np.complex128), orep_irreps=orep_irreps,
                         auxrep=np.concatenate(auxrep_blocks).astype(np.complex128), auxrep_irreps=auxrep_irreps)

    # --- V with the Hermitian pair relation V(k2,k1)_{Q,j,i} = conj(V(k1,k2)_{Q,i,j})
    V = np.zeros(layout.flat_V_size if with_V else 0, dtype=np.complex128)
    sigma = spec.v_scale / np.sqrt(spec.nao)
    if symmetric and with_V:
        _symmetric_V(spec, layout, kmesh, ops, Wk, Xq, sigma, V)
    for k1 in (range(nk) if with_V and not symmetric else ()):
        for k2 in range(k1, nk):
            p = k1 * nk + k2
            pr = k2 * nk + k1
            if len(layout.tensor_irreps[p]) == 0:
                continue
            vrng = np.random.default_rng((spec.seed + 7, p))  # one stream per pair
            q = layout.pair_q(k1, k2)
            qr = layout.pair_q(k2, k1)
            base, baser = layout.kpair_slice_offsets[p], layout.kpair_slice_offsets[pr]
            rev = {tuple(t): i for i, t in enumerate(layout.tensor_irreps[pr])}
            for b, (iq, i1, i2) in enumerate(layout.tensor_irreps[p]):
                qb, b1, b2 = aux_sizes[q][iq], ao_sizes[k1][i1], ao_sizes[k2][i2]
                o = base + layout.tensor_offsets[p][b]
                if p == pr:
                    br = rev[(iq, i2, i1)]
                    if br < b:
                        continue
                blk = sigma * (vrng.normal(size=(qb, b1, b2)) + 1j * vrng.normal(size=(qb, b1, b2))) / np.sqrt(2)
                if p == pr and (i1 == i2):
                    blk = 0.5 * (blk + blk.transpose(0, 2, 1).conj())
                V[o:o + qb * b1 * b2] = blk.ravel()
                br = rev[(iq, i2, i1)]
                assert aux_sizes[qr][iq] == qb
                orr = baser + layout.tensor_offsets[pr][br]
                V[orr:orr + qb * b1 * b2] = blk.transpose(0, 2, 1).conj().ravel()

    # --- F, S, H on the stored k points
    ns = spec.ns
    fa = layout.flat_ao_size
    F = np.zeros((ns, fa), np.complex128)
    S = np.zeros((ns, fa), np.complex128)
    frng = np.random.default_rng(spec.seed + 11)
    eigs = []
    F0 = {}  # symmetric: F0 per star (gauge 0), drawn in representative order
    if symmetric:
        for st_, r in enumerate(reps):
            blocks = []
            for s_ in ao_sizes[r]:
                x = frng.uniform(-1, 1, size=(s_, s_)) + 1j * frng.uniform(-1, 1, size=(s_, s_))
                blocks.append(0.5 * (x + x.conj().T) * 0.6 + np.diag(frng.normal(0.0, 0.5, size=s_)))
            F0[st_] = blocks
    for ik, k in enumerate(layout.irre_list):
        w = star_size[star_of[k]] if rotate else 1
        for b, s_ in enumerate(ao_sizes[k]):
            o = layout.kao_slice_offsets_irre[ik] + layout.ao_offsets[k][b]
            if symmetric:
                u = Wk[k][b]
                h = u @ F0[star_of[k]][b] @ u.conj().T
                h = 0.5 * (h + h.conj().T)
            else:
                x = frng.uniform(-1, 1, size=(s_, s_)) + 1j * frng.uniform(-1, 1, size=(s_, s_))
                h = 0.5 * (x + x.conj().T) * 0.6 + np.diag(frng.normal(0.0, 0.5, size=s_))
            for sp in range(ns):
                F[sp, o:o + s_ * s_] = h.ravel()
                S[sp, o:o + s_ * s_] = np.eye(s_).ravel()
            eigs.extend([(e, w) for e in np.linalg.eigvalsh(h)])
    mu = half_filling_mu(eigs, spec.nao, nk)
    return Crystal(spec=spec, layout=layout, V=V, F=F, S=S, H=F.copy(), mu=float(mu),
                   star_sizes=np.array([star_size[star_of[k]] for k in layout.irre_list]))


def half_filling_mu(eigs, nao: int, nk: int) -> float:
    """Chemical potential midway between the last filled and the first empty
    band energy at half filling (nao * nk / 2 states per spin); eigs: (energy,
    weight of its k point) over the stored k points."""
    eigs = sorted(eigs)
    target = nao * nk / 2.0
    acc = 0.0
    for i, (e, w) in enumerate(eigs):
        acc += w
        if acc >= target:
            nxt = eigs[i + 1][0] if i + 1 < len(eigs) else e + 1.0
            return 0.5 * (e + nxt)
    return eigs[-1][0]


def load_ir(nts: int):
    """Committed IR grid for ``nts`` tau points (see data/make_ir_grids.py)."""
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", f"ir_{nts}.npz")
    z = np.load(path)
    return {k.replace("__", "/"): z[k] for k in z.files if k != "Lambda"}

"""Tight-binding crystals from Gaussian orbitals (mbsymmetry_gb300/orbitals.py):
the Slater-Koster and three-centre constructions, the group-derived bases and
rotations, the selection rule, and the reference's iBZ-vs-full-BZ relation
(SymmetryMBPT/test/test_cugw.cpp:306-436) on the oracle."""
import dataclasses

import numpy as np
import pytest

from mbsymmetry_gb300 import orbitals as O
from mbsymmetry_gb300 import symmetry as S
from mbsymmetry_gb300.crystal import CONFIGS, load_ir
from mbsymmetry_gb300.transformer import build_transforms
from oracle import Oracle


@pytest.fixture(scope="module")
def c1():
    return O.make_orbital_crystal(CONFIGS["C1"], rotate=True, keep_ao_data=True)


@pytest.fixture(scope="module")
def gen():
    return O._Generator(CONFIGS["C1"], O.OrbitalModel())


def _rz(t):
    return np.array([[np.cos(t), -np.sin(t), 0], [np.sin(t), np.cos(t), 0], [0, 0, 1.0]])


@pytest.mark.parametrize("lr,lc", [(0, 0), (0, 1), (1, 0), (1, 1), (0, 2), (1, 2), (2, 1), (2, 2)])
def test_bond_frame_matrix_is_axially_symmetric(lr, lc):
    """E0 commutes with every rotation about the bond and with a mirror through
    it (C_inf_v), which makes E(d) = D(R_d) E0 D(R_d)^T independent of the frame."""
    E0 = O.bond_frame_matrix(lr, lc, np.array([0.3, -0.2, 0.1]))
    for R in [_rz(0.37), _rz(2.1), np.diag([1.0, -1.0, 1.0]), np.diag([-1.0, 1.0, 1.0])]:
        assert np.abs(S.shell_matrix(lr, R) @ E0 @ S.shell_matrix(lc, R).T - E0).max() < 1e-14
    d = np.array([0.3, -1.2, 0.7])
    R2 = O.bond_rotation(d) @ _rz(0.9)   # another frame taking z onto d
    E1 = O.sk_block(lr, lc, np.array([0.3, -0.2, 0.1]), d)
    E2 = S.shell_matrix(lr, R2) @ E0 @ S.shell_matrix(lc, R2).T
    assert np.abs(E1 - E2).max() < 1e-14


def test_three_centre_overlap_matches_quadrature():
    """Cartesian-factorised three-centre overlap against a direct grid sum."""
    A, B, C = np.array([[0.1, -0.2, 0.3]]), np.array([[0.6, 0.1, -0.2]]), np.array([[-0.3, 0.4, 0.2]])
    x = np.linspace(-7, 7, 141)
    h = x[1] - x[0]
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    r = np.stack([X, Y, Z], -1)

    def shell(c, a, l):
        u = r - c[0]
        g = np.exp(-a * np.sum(u * u, -1))
        if l == 0:
            return [g]
        if l == 1:
            return [u[..., i] * g for i in range(3)]
        return [np.einsum("...i,ij,...j->...", u, Q, u) * g for Q in S._D2]

    for (la, lb, lc) in [(0, 0, 0), (1, 0, 2), (2, 1, 1), (2, 2, 2)]:
        got = O.three_centre(A, 0.9, la, B, 0.7, lb, C, 1.3, lc)[0]
        fa, fb, fc = shell(A, 0.9, la), shell(B, 0.7, lb), shell(C, 1.3, lc)
        ref = np.array([[[np.sum(p * q * s) * h ** 3 for s in fc] for q in fb] for p in fa])
        assert np.abs(got - ref).max() < 1e-9 * max(1.0, np.abs(ref).max())


def test_fock_is_hermitian_and_covariant(c1, gen):
    """F(k) Hermitian; F(g k) = D(g, k) F(k) D(g, k)^H for every operation and k."""
    F = c1.F_ao
    assert np.abs(F - F.conj().transpose(0, 2, 1)).max() < 1e-14
    for k in range(gen.nk):
        for g in range(0, 48, 5):
            gk = gen.perm[g][k]
            D = gen.D(g, k, gen.ao)
            assert np.abs(D @ F[k] @ D.conj().T - F[gk]).max() < 1e-13


def test_coulomb_pair_relation_and_covariance(c1, gen):
    """V(k2, k1)_{Q,j,i} = conj(V(k1, k2)_{Q,i,j}), and V transforms with
    D_aux(g, p) x D(g, k1) x conj(D(g, k2)) (its first AO index is a conjugated
    Bloch function, the aux index enters conjugated at p = k2 - k1)."""
    V, nk = c1.V_ao, gen.nk
    for k1 in range(nk):
        for k2 in range(nk):
            a, b = V[k1 * nk + k2], V[k2 * nk + k1]
            assert np.abs(b - a.transpose(0, 2, 1).conj()).max() < 1e-13 * np.abs(V).max()
    rng = np.random.default_rng(3)
    for _ in range(12):
        k1, k2, g = int(rng.integers(nk)), int(rng.integers(nk)), int(rng.integers(48))
        p = c1.layout.pair_q(k1, k2)
        img = lambda k: gen.perm[g][k]  # noqa: E731
        Dq, D1, D2 = gen.D(g, p, gen.aux), gen.D(g, k1, gen.ao), gen.D(g, k2, gen.ao)
        want = np.einsum("QR,ia,jb,Rab->Qij", Dq, D1, D2.conj(), V[k1 * nk + k2], optimize=True)
        assert np.abs(want - V[img(k1) * nk + img(k2)]).max() < 1e-12 * np.abs(V).max()


def test_adapted_blocks_match_the_dirac_character_decomposition(gen):
    """Eigen-clusters of the seeded group-algebra element = d blocks of size m
    per irrep, as the class-sum method finds them."""
    spec = CONFIGS["C1"]
    ao, aux = S.fcc_basis(spec.nao, spec.atoms), S.fcc_basis(spec.naux, spec.atoms)   # cubic coordinates
    Bt = np.linalg.inv(S.FCC_A.T)
    for kr in gen.reps:
        kc = Bt @ gen.kmesh[kr]
        assert sorted(gen.adapted_basis(kr, gen.ao)[1]) == sorted(S.block_sizes(kc, ao))
        assert sorted(gen.adapted_basis(kr, gen.aux)[1]) == sorted(S.block_sizes(kc, aux))


def test_block_structure_in_the_adapted_bases(c1):
    """F, orep and auxrep are block-diagonal; the aux basis at -q is the
    conjugate of the one at q; the data vanish on every block the group
    forbids, and on C1 every allowed block is non-zero (the rule and the data
    agree block for block)."""
    assert max(c1.off_block[k] for k in ("F", "orep", "auxrep")) < 1e-13
    assert c1.off_block["V_forbidden"] < 1e-13
    L = c1.layout
    minus = [L.mom_cons(0, q, 0) for q in range(L.nk)]   # -q
    for q in range(L.nk):
        assert np.abs(c1.Y[minus[q]] - c1.Y[q].conj()).max() < 1e-14
    stored = {(p, *(int(x) for x in b)) for p in range(L.nk * L.nk) for b in L.tensor_irreps[p]}
    n = c1.V_block_norms
    assert len(stored) < 0.95 * len(n)
    assert min(n[b] for b in stored) > 1e-9
    assert max(v for b, v in n.items() if b not in stored) < 1e-13


def _characters(gen, k, basis, cols):
    """Characters over the little group of the irrep whose rows the columns span."""
    G = gen.little_group(k)
    Ds = [gen.D(h, k, basis) for h in G]
    span = np.concatenate([D @ cols for D in Ds], axis=1)
    u, s, _ = np.linalg.svd(span, full_matrices=False)
    P = u[:, s > 1e-8 * s[0]]
    m = cols.shape[1]
    return np.array([np.trace(P.conj().T @ D @ P) / m for D in Ds])


def test_selection_rule_at_gamma_follows_the_irreps(c1, gen):
    """At the (Gamma, Gamma) pair every index transforms under O_h; a block of
    irreps (alpha, beta, gamma) can be non-zero only if chi_alpha chi_beta
    conj(chi_gamma) contains the identity, and every block with a zero
    multiplicity is zero in the data."""
    L = c1.layout
    k0 = 0
    assert np.allclose(gen.kmesh[k0], 0)
    aux_off = np.concatenate([[0], np.cumsum(L.aux_sizes[k0])])
    ao_off = np.concatenate([[0], np.cumsum(L.ao_sizes[k0])])
    chi_q = [_characters(gen, k0, gen.aux, c1.Y[k0][:, aux_off[i]:aux_off[i + 1]]) for i in range(len(aux_off) - 1)]
    chi_a = [_characters(gen, k0, gen.ao, c1.U[k0][:, ao_off[i]:ao_off[i + 1]]) for i in range(len(ao_off) - 1)]
    forbidden = 0
    for iq, cq in enumerate(chi_q):
        for i1, ca in enumerate(chi_a):
            for i2, cb in enumerate(chi_a):
                mult = np.mean(cq * ca * cb.conj())
                norm = c1.V_block_norms[(k0 * L.nk + k0, iq, i1, i2)]
                if abs(mult) < 1e-9:
                    forbidden += 1
                    assert norm < 1e-13
    assert forbidden > 0


def _chain(cr, tr):
    L, ns, nts = cr.layout, cr.ns, tr.nts
    orc = Oracle(L, ns, nts)
    G, _ = orc.dyson(np.zeros(nts * ns * L.flat_ao_size, np.complex128), cr.F, cr.S, tr, cr.mu)
    Gf = orc.rotate_G(G)
    P = orc.p_tilde(orc.mirror_P0(orc.p0(Gf, cr.V)), tr)
    Pf = orc.rotate_P(P)
    return Gf, Pf, orc.sigma(Gf, Pf, cr.V)


@pytest.mark.parametrize("ns,change", [(1, {}), (2, {}), (1, {"mesh": (2, 2, 2)}),
                                       (1, {"atoms": 4, "nao": 16, "naux": 40})])
def test_irreducible_and_full_mesh_agree(ns, change):
    """Orbital crystal on the irreducible k with the group's rotations and on
    every k without: G, P~ (every q) and Sigma (irreducible k) agree.  C1's
    3x3x3 mesh, the 2x2x2 mesh (every point self-conjugate: real aux bases),
    and the 4-atom basis (an atom pair exchanged by the group)."""
    spec = dataclasses.replace(CONFIGS["C1"], ns=ns, **change)
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = O.make_orbital_crystal(spec, rotate=True)
    cf = O.make_orbital_crystal(spec, rotate=False)
    assert np.array_equal(cr.V, cf.V) and cr.layout.ink < cf.layout.ink == cf.layout.nk
    Gr, Pr, Sr = _chain(cr, tr)
    Gf, Pf, Sf = _chain(cf, tr)
    assert np.abs(Gr - Gf).max() < 1e-12
    assert np.abs(Pr - Pf).max() < 1e-12
    Lr, Lf, nts = cr.layout, cf.layout, tr.nts
    Sr, Sf = Sr.reshape(nts, ns, -1), Sf.reshape(nts, ns, -1)
    d = 0.0
    for ik, k in enumerate(Lr.irre_list):
        n = Lr.kao_slice_sizes[k]
        d = max(d, float(np.abs(Sr[:, :, Lr.kao_slice_offsets_irre[ik]:Lr.kao_slice_offsets_irre[ik] + n]
                                - Sf[:, :, Lf.kao_slice_offsets_irre[k]:Lf.kao_slice_offsets_irre[k] + n]).max()))
    assert d < 1e-12 and np.abs(Sf).max() > 1.0


def test_a_wrong_rotation_breaks_the_relation():
    """Negative control: one row of one aux rotation block off by a phase (a
    phase on the whole block would cancel in auxrep P~ auxrep^H) and P~ no
    longer agrees."""
    spec = CONFIGS["C1"]
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = O.make_orbital_crystal(spec, rotate=True)
    cf = O.make_orbital_crystal(spec, rotate=False)
    L = cr.layout
    q = next(q for q in range(L.nk) if L.index[q] != q)
    o = L.kauxrep_slice_offsets[q]
    b = int(L.aux_sizes[q][0])
    L.auxrep[o:o + b] *= np.exp(0.3j)   # first row of the first block
    _, Pr, _ = _chain(cr, tr)
    _, Pf, _ = _chain(cf, tr)
    assert np.abs(Pr - Pf).max() > 1e-6


# --------------------------------------------------------------------------- #
# wurtzite (P6_3mc: screw axis and glides, projective representations at the
# zone boundary, no inversion: time reversal brings -k into the stars)
# --------------------------------------------------------------------------- #
def _wurtzite(mesh):
    return dataclasses.replace(CONFIGS["C4"], name="wurtzite", mesh=mesh, nao=16, naux=40, nts=62, beta=50.0)


@pytest.fixture(scope="module")
def wz():
    spec = _wurtzite((3, 3, 2))
    return (O.make_orbital_crystal(spec, rotate=True, keep_ao_data=True), O._Generator(spec, O.OrbitalModel()))


def test_wurtzite_data_are_covariant(wz):
    """F(g k) = D F(k) D^H and V(g k1, g k2) = (D_aux x D x conj D) V(k1, k2)
    for the 12 space-group operations (the screws and glides carry their
    c/2 translations into the Bloch phases), the Hermitian pair relation, and
    block-diagonal F and rotations in the adapted bases."""
    cr, gen = wz
    F, V, nk = cr.F_ao, cr.V_ao, gen.nk
    assert np.abs(F - F.conj().transpose(0, 2, 1)).max() < 1e-14
    for k in range(nk):
        for g in range(len(gen.ops)):
            D = gen.D(g, k, gen.ao)
            assert np.abs(D @ F[k] @ D.conj().T - F[gen.perm[g][k]]).max() < 1e-13
    for k1 in range(nk):
        for k2 in range(nk):
            a, b = V[k1 * nk + k2], V[k2 * nk + k1]
            assert np.abs(b - a.transpose(0, 2, 1).conj()).max() < 1e-13 * np.abs(V).max()
    rng = np.random.default_rng(5)
    for _ in range(12):
        k1, k2, g = int(rng.integers(nk)), int(rng.integers(nk)), int(rng.integers(len(gen.ops)))
        p = cr.layout.pair_q(k1, k2)
        want = np.einsum("QR,ia,jb,Rab->Qij", gen.D(g, p, gen.aux), gen.D(g, k1, gen.ao), gen.D(g, k2, gen.ao).conj(),
                         V[k1 * nk + k2], optimize=True)
        assert np.abs(want - V[gen.perm[g][k1] * nk + gen.perm[g][k2]]).max() < 1e-12 * np.abs(V).max()
    assert max(cr.off_block.values()) < 1e-13


def test_wurtzite_blocks_and_time_reversal_sticking(wz):
    """Block sizes at every representative: the projective-representation
    content (d blocks of size m per irrep, symmetry.sg_block_sizes), except
    where time reversal glues the rows of each irrep pair together (on the
    A-L-H face kz = 1/2, where the screw's factor system makes every irrep
    two-dimensional): there the blocks are those sizes merged in pairs."""
    cr, gen = wz
    L = cr.layout
    merged_points = 0
    for kr in gen.reps:
        for basis, sizes in ((gen.ao, L.ao_sizes[kr]), (gen.aux, L.aux_sizes[kr])):
            theirs, mine = sorted(S.sg_block_sizes(gen.kmesh[kr], basis)), sorted(int(x) for x in sizes)
            if mine != theirs:
                assert abs(gen.kmesh[kr][2] - 0.5) < 1e-12
                pairs = sorted(2 * x for x in theirs[::2])
                assert theirs[::2] == theirs[1::2] and mine == pairs
                merged_points += 1
    assert merged_points > 0


def test_wurtzite_selection_rule_at_gamma_follows_the_irreps(wz):
    """At (Gamma, Gamma) every index transforms under C6v: a block whose
    irreps' character product has no invariant is zero in the data."""
    cr, gen = wz
    L = cr.layout
    aux_off = np.concatenate([[0], np.cumsum(L.aux_sizes[0])])
    ao_off = np.concatenate([[0], np.cumsum(L.ao_sizes[0])])
    chi_q = [_characters(gen, 0, gen.aux, cr.Y[0][:, aux_off[i]:aux_off[i + 1]]) for i in range(len(aux_off) - 1)]
    chi_a = [_characters(gen, 0, gen.ao, cr.U[0][:, ao_off[i]:ao_off[i + 1]]) for i in range(len(ao_off) - 1)]
    forbidden = 0
    for iq, cq in enumerate(chi_q):
        for i1, ca in enumerate(chi_a):
            for i2, cb in enumerate(chi_a):
                if abs(np.mean(cq * ca * cb.conj())) < 1e-9:
                    forbidden += 1
                    assert cr.V_block_norms[(0, iq, i1, i2)] < 1e-13
    assert forbidden > 0


@pytest.mark.parametrize("mesh,bound", [((3, 3, 2), 1e-12), ((2, 2, 3), 1e-10)])
def test_wurtzite_irreducible_and_full_mesh_agree(mesh, bound):
    """iBZ with the space group's rotations against the full mesh.  On the
    2x2x3 mesh time reversal brings kz = 2/3 into the stars of kz = 1/3: G
    and P~ are conjugated there (the rotation path's conj_index), which is
    exact because the committed grids sample +/- Matsubara pairs."""
    spec = _wurtzite(mesh)
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = O.make_orbital_crystal(spec, rotate=True)
    cf = O.make_orbital_crystal(spec, rotate=False)
    if mesh[2] == 3:
        assert np.any(cr.layout.conj_index != np.arange(cr.layout.nk))
    Gr, Pr, Sr = _chain(cr, tr)
    Gf, Pf, Sf = _chain(cf, tr)
    Lr, Lf, nts, ns = cr.layout, cf.layout, tr.nts, cr.ns
    Sr, Sf = Sr.reshape(nts, ns, -1), Sf.reshape(nts, ns, -1)
    d = max(float(np.abs(Sr[:, :, Lr.kao_slice_offsets_irre[ik]:][:, :, :Lr.kao_slice_sizes[k]]
                         - Sf[:, :, Lf.kao_slice_offsets_irre[k]:][:, :, :Lr.kao_slice_sizes[k]]).max())
            for ik, k in enumerate(Lr.irre_list))
    assert np.abs(Gr - Gf).max() < bound and np.abs(Pr - Pf).max() < bound and d < bound


def test_static_and_dynamic_polarisability_is_negative_semidefinite():
    """For a Hermitian F, G0 and V in any bases, P0(q, i Omega) = -(2/nk) sum V
    chi V^H with chi <= 0: every block at every sampled bosonic frequency is
    negative semidefinite (up to the transform's Hermitian-part residue), so
    the W~ solve's A = I - (P0 + P0^H)/2 is >= I.  Checks the oracle's P0
    sign, prefactor and tau -> i Omega transform on physical data."""
    spec = CONFIGS["C1"]
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = O.make_orbital_crystal(spec)
    L, nts, ns = cr.layout, tr.nts, cr.ns
    orc = Oracle(L, ns, nts)
    G, _ = orc.dyson(np.zeros(nts * ns * L.flat_ao_size, np.complex128), cr.F, cr.S, tr, cr.mu)
    P0 = orc.mirror_P0(orc.p0(orc.rotate_G(G), cr.V))
    worst, scale = -np.inf, 0.0
    for iq, q in enumerate(L.irre_list):
        qs = L.qaux_slice_sizes[q]
        Pw = tr.Tnt_BF @ P0[nts * L.qaux_slice_offsets_irre[iq]:][:nts * qs].reshape(nts, qs)[1:-1]
        for b, sz in enumerate(L.aux_sizes[q]):
            o = L.aux_offsets[q][b]
            for blk in Pw[:, o:o + sz * sz].reshape(-1, sz, sz):
                e = np.linalg.eigvalsh(0.5 * (blk + blk.conj().T))
                worst, scale = max(worst, e.max()), max(scale, -e.min())
    assert scale > 1.0 and worst < 1e-9 * scale


def test_orbital_crystal_is_an_insulator_with_negative_correlation_energy():
    """Half filling puts mu in a gap of the Slater-Koster bands (N(G0) = nao
    to 1e-9), and the Galitskii-Migdal correlation energy of the first GW
    Sigma is negative."""
    from mbsymmetry_gb300.transformer import gm_matrix
    spec = CONFIGS["C1"]
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = O.make_orbital_crystal(spec)
    L = cr.layout
    orc = Oracle(L, cr.ns, tr.nts)
    G, _ = orc.dyson(np.zeros(tr.nts * cr.ns * L.flat_ao_size, np.complex128), cr.F, cr.S, tr, cr.mu)
    Sigma, _, _ = orc.gw_sigma(G, cr.V, tr)
    e_corr, _, n = orc.energy(Sigma, G, cr.F, cr.S, gm_matrix(tr))
    assert abs(n - spec.nao) < 1e-9 and e_corr < 0

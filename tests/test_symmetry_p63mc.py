"""P6_3mc (config C4's wurtzite structure): the non-symmorphic space group,
its projective representations on Bloch sums, and the class-free
decomposition (mbsymmetry_gb300/symmetry.py), pinned by known results and by
the O_h class-sum method on the symmorphic fcc crystals."""
import itertools

import numpy as np
import pytest

from mbsymmetry_gb300 import symmetry as S


def _rep(k, basis, ops=None, A=S.HEX_A):
    ops = S.p63mc_operations() if ops is None else ops
    k = np.asarray(k, dtype=float)
    G = S.sg_little_group(k, ops)
    return G, [S.sg_bloch_representation(k, M, t, basis, A) for M, t in G]


def test_operations_map_the_structure_and_close():
    ops = S.p63mc_operations()
    pos = S.wurtzite_basis(4).positions
    for M, t in ops:
        assert round(abs(np.linalg.det(M))) == 1
        for p in pos:
            q = M @ p + t
            assert any(np.allclose(q - r, np.round(q - r), atol=1e-9) for r in pos)
    for (M1, t1), (M2, t2) in itertools.product(ops, ops):  # closed modulo lattice translations
        M, t = M1 @ M2, M1 @ t2 + t1
        assert any(np.array_equal(M, N) and np.allclose(t - s, np.round(t - s)) for N, s in ops)


def test_gamma_content_of_s_and_p_shells():
    """C6v at Gamma, two species on Wyckoff 2b: s -> A1 + B1 per species;
    s + p -> A1 (x2), B1 (x2), E1, E2 per species."""
    s_only = S.Basis(S.wurtzite_basis(4).positions, [[0]] * 4)
    _, Ds = _rep([0, 0, 0], s_only)
    assert S.projective_content(Ds) == [(1, 2), (1, 2)]
    sp = S.Basis(s_only.positions, [[0, 1]] * 4)
    _, Ds = _rep([0, 0, 0], sp)
    assert S.projective_content(Ds) == [(1, 4), (1, 4), (2, 2), (2, 2)]


def _phases(G, Ds):
    """D(g) D(h) = w(g, h) D(gh) for the chosen translations; the w."""
    out = []
    for (g, Dg), (h, Dh) in itertools.product(zip(G, Ds), zip(G, Ds)):
        M = g[0] @ h[0]
        j = next(j for j, (N, _) in enumerate(G) if np.array_equal(N, M))
        P = Dg @ Dh
        i = np.unravel_index(np.argmax(np.abs(Ds[j])), Ds[j].shape)
        w = P[i] / Ds[j][i]
        assert np.allclose(P, w * Ds[j], atol=1e-12) and abs(abs(w) - 1) < 1e-12
        out.append(w)
    return np.array(out)


def test_factor_system_is_trivial_at_gamma_and_not_at_A():
    b = S.wurtzite_basis(16)
    G, Ds = _rep([0, 0, 0], b)
    assert np.allclose(_phases(G, Ds), 1.0)
    G, Ds = _rep([0, 0, 0.5], b)  # A: the 6_3 screw gives D(C2 screw)^2 = -1
    w = _phases(G, Ds)
    assert np.any(np.abs(w - 1) > 0.5)


@pytest.mark.parametrize("k", [[0, 0, 0], [0, 0, 0.5], [0.5, 0, 0], [0.5, 0, 0.5], [1 / 3, 1 / 3, 0],
                               [1 / 3, 1 / 3, 0.5], [0.25, 0, 0], [0.25, 0.25, 1 / 3], [0.5, 0.25, 1 / 3]])
def test_c4_blocks_fill_the_basis(k):
    for n in (72, 350):
        b = S.wurtzite_basis(n)
        assert b.size == n
        content = S.projective_content(_rep(k, b)[1])
        assert sum(d * m for d, m in content) == n


def test_blocks_are_equal_within_a_star():
    b = S.wurtzite_basis(72)
    ops = S.p63mc_operations()
    k = np.array([0.25, 0.0, 1 / 3])
    ref = sorted(S.sg_block_sizes(k, b))
    for M, _ in ops:
        kk = np.linalg.inv(M).T @ k
        assert sorted(S.sg_block_sizes(kk, b)) == ref


def test_class_free_decomposition_matches_oh_class_sums():
    """Symmorphic check: O_h on the fcc mesh, in fractional coordinates with t = 0,
    gives the same (d, m) as the class-sum (Dirac character) method."""
    A = S.FCC_A
    Ainv = np.linalg.inv(A)
    ops_cart = S.oh_operations()
    ops = [(np.round(Ainv @ R @ A).astype(int), np.zeros(3)) for R in ops_cart]
    basis = S.fcc_basis(26, 2)
    bfrac = S.Basis(np.array([Ainv @ p for p in basis.positions]), basis.shells)
    for kc in S.fcc_kmesh(3):
        kf = A.T @ kc
        G = S.sg_little_group(kf, ops)
        Ds = [S.sg_bloch_representation(kf, M, t, bfrac, A) for M, t in G]
        assert S.projective_content(Ds) == S.irrep_content(kc, basis, ops_cart)

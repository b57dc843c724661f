"""Irrep block sizes from O_h (the group-faithful generator): known
decompositions, the representation property, dimension counts and star
invariance on the FCC meshes."""
import numpy as np
import pytest

from mbsymmetry_gb300 import symmetry as sy

SPD = [0, 1, 2]


def test_gamma_point_known_decompositions():
    one = sy.Basis(np.zeros((1, 3)), [SPD])
    # s -> A1g, p -> T1u, d -> Eg + T2g
    assert sy.irrep_content(np.zeros(3), one) == [(1, 1), (2, 1), (3, 1), (3, 1)]
    assert sy.block_sizes(np.zeros(3), one) == [1] * 9
    rs = sy.fcc_basis(18, 2)            # rock salt, s p d s p d per atom pair
    assert sorted(rs.shells[0]) == [0, 1, 2] and sorted(rs.shells[1]) == [0, 1, 2]
    assert sy.irrep_content(np.zeros(3), rs) == [(1, 2), (2, 2), (3, 2), (3, 2)]
    assert len(sy.little_group(np.zeros(3), sy.oh_operations())) == 48


def test_lambda_line_c3v():
    rs = sy.fcc_basis(18, 2)
    k = sy.fcc_kmesh(3)[1]             # (1/3, 1/3, -1/3) 2 pi: C3v
    assert len(sy.little_group(k, sy.oh_operations())) == 6
    # A1: s, p_parallel, d_z2 per atom -> 6; E: p_perp + 2 d -> 2 x 6; A2: none
    assert sy.irrep_content(k, rs) == [(1, 6), (2, 6)]


@pytest.mark.parametrize("n,atoms,count", [(3, 2, 26), (3, 2, 36), (4, 4, 52)])
def test_representation_and_counts_on_the_mesh(n, atoms, count):
    ops = sy.oh_operations()
    b = sy.fcc_basis(count, atoms)
    assert b.size == count
    for i, k in enumerate(sy.fcc_kmesh(n)):
        G = sy.little_group(k, ops)
        if i % 5 == 0:                 # homomorphism D(R1) D(R2) = D(R1 R2) on G_k
            Ds = {tuple(R.ravel()): sy.bloch_representation(k, R, b) for R in G}
            for R1 in G[::3]:
                for R2 in G[::2]:
                    assert np.abs(Ds[tuple(R1.ravel())] @ Ds[tuple(R2.ravel())] -
                                  sy.bloch_representation(k, R1 @ R2, b)).max() < 1e-12
        content = sy.irrep_content(k, b, ops)
        assert sum(d * m for d, m in content) == count
        assert sum(d * d for d, _ in content) <= len(G)


def test_block_sizes_are_star_invariant():
    ops = sy.oh_operations()
    b = sy.fcc_basis(26, 2)
    ks = sy.fcc_kmesh(3)
    Brec = np.linalg.inv(sy.FCC_A).T
    for k in ks[:10]:
        ref = sorted(sy.block_sizes(k, b, ops))
        for R in ops[::7]:
            kr = R @ k
            assert sorted(sy.block_sizes(kr, b, ops)) == ref


def test_physical_crystal_layout():
    from mbsymmetry_gb300.crystal import CONFIGS, make_crystal
    for name in ("C1", "C2"):
        spec = CONFIGS[name]
        cr = make_crystal(spec, physical=True, with_V=False)
        L = cr.layout
        assert all(int(np.sum(a)) == spec.nao for a in L.ao_sizes)
        assert all(int(np.sum(a)) == spec.naux for a in L.aux_sizes)
        assert max(int(np.max(a)) for a in L.aux_sizes) <= 64     # inside the tensor-core kernels' limits

"""Hartree-Fock exchange: the oracle's Sigma contraction with P = identity and
G = rho at tau = 0 equals the direct density-fitted exchange
K(k) = -(1/nk) sum_k2 sum_Q V^Q(k, k2) rho(k2) V^Q(k, k2)^H (CPU)."""
import numpy as np

from _helpers import crystal
from oracle import Oracle


def hf_exchange_oracle(cr, tr, rho):
    """K through the oracle's Sigma (the checker for the GPU path)."""
    L, ns, nts = cr.layout, cr.ns, tr.nts
    fa = L.flat_ao_size
    orc = Oracle(L, ns, nts)
    G = np.zeros(nts * ns * fa, np.complex128)
    G[:ns * fa] = rho.ravel()
    P = np.zeros(nts * L.flat_aux_size, np.complex128)
    for r, q in enumerate(L.irre_list):
        base = nts * L.qaux_slice_offsets_irre[r]
        for iq, qb in enumerate(L.aux_sizes[q]):
            o = base + L.aux_offsets[q][iq]
            P[o:o + qb * qb] = np.eye(qb).ravel()
    S = orc.sigma(orc.rotate_G(G), orc.rotate_P(P), cr.V, nt_max=1)
    return S[:ns * fa].reshape(ns, fa)


def density(cr, seed=3):
    """A Hermitian block-diagonal rho ([s][flat_ao], stored k)."""
    L, ns = cr.layout, cr.ns
    rng = np.random.default_rng(seed)
    rho = np.zeros((ns, L.flat_ao_size), np.complex128)
    for s in range(ns):
        for ik, k in enumerate(L.irre_list):
            base = L.kao_slice_offsets_irre[ik]
            for b, n in enumerate(L.ao_sizes[k]):
                a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
                o = base + L.ao_offsets[k][b]
                rho[s, o:o + n * n] = (0.5 * (a + a.conj().T)).ravel()
    return rho


def test_oracle_exchange_equals_direct_formula():
    cr, tr = crystal("C1", rotate=False)
    L, ns = cr.layout, cr.ns
    rho = density(cr)
    K = hf_exchange_oracle(cr, tr, rho)
    Kd = np.zeros_like(K)
    for k1 in range(L.nk):
        for k2 in range(L.nk):
            p = k1 * L.nk + k2
            q = L.pair_q(k1, k2)
            for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
                qb, b1, b2 = L.aux_sizes[q][iq], L.ao_sizes[k1][i1], L.ao_sizes[k2][i2]
                o = L.kpair_slice_offsets[p] + L.tensor_offsets[p][b]
                V = cr.V[o:o + qb * b1 * b2].reshape(qb, b1, b2)
                for s in range(ns):
                    r2 = L.kao_slice_offsets[k2] + L.ao_offsets[k2][i2]
                    R = rho[s, r2:r2 + b2 * b2].reshape(b2, b2)
                    o1 = L.kao_slice_offsets[k1] + L.ao_offsets[k1][i1]
                    Kd[s, o1:o1 + b1 * b1] -= np.einsum("qim,mn,qjn->ij", V, R, V.conj()).ravel() / L.nk
    assert np.abs(K - Kd).max() < 1e-12 * max(1.0, np.abs(Kd).max())
    assert np.abs(Kd).max() > 1e-3


def hf_hartree_numpy(cr, tr, rho):
    """J(k) = sum_Q V^Q(k, k) c_Q, c_Q = (f/nk) sum_{k', s} Tr[V^Q(k', k') rho_s(k')]
    (f = 2 for ns = 1) on the diagonal AO blocks; rho of every k' from the oracle's
    rotation.  Returns (J [flat_ao], c)."""
    L, ns, nts = cr.layout, cr.ns, tr.nts
    fa, nk = L.flat_ao_size, L.nk
    orc = Oracle(L, ns, nts)
    G = np.zeros(nts * ns * fa, np.complex128)
    G[:ns * fa] = rho.ravel()
    Gf = orc.rotate_G(G)
    q0 = next(q for q in range(nk) if L.mom_cons(0, 0, q) == 0)
    f = (2.0 if ns == 1 else 1.0) / nk
    c = np.zeros(L.qaux_slice_sizes[q0], np.complex128)
    for k in range(nk):
        p = k * nk + k
        for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
            if i1 != i2:
                continue
            qb, bs = L.aux_sizes[q0][iq], L.ao_sizes[k][i1]
            o = L.kpair_slice_offsets[p] + L.tensor_offsets[p][b]
            V = cr.V[o:o + qb * bs * bs].reshape(qb, bs, bs)
            for s in range(ns):
                og = L.kao_slice_offsets[k] * ns * nts + s * L.kao_slice_sizes[k] + L.ao_offsets[k][i1]
                R = Gf[og:og + bs * bs].reshape(bs, bs)
                c[L.aux_offsets[q0][iq]:L.aux_offsets[q0][iq] + qb] += f * np.einsum("qab,ba->q", V, R)
    J = np.zeros(fa, np.complex128)
    for ik, k in enumerate(L.irre_list):
        p = k * nk + k
        for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
            if i1 != i2:
                continue
            qb, bs = L.aux_sizes[q0][iq], L.ao_sizes[k][i1]
            o = L.kpair_slice_offsets[p] + L.tensor_offsets[p][b]
            V = cr.V[o:o + qb * bs * bs].reshape(qb, bs, bs)
            oj = L.kao_slice_offsets_irre[ik] + L.ao_offsets[k][i1]
            J[oj:oj + bs * bs] += np.einsum("qij,q->ij", V, c[L.aux_offsets[q0][iq]:L.aux_offsets[q0][iq] + qb]).ravel()
    return J, c


def test_hartree_is_hermitian_with_real_density_coefficients():
    """V(k, k) is Hermitian for every Q and rho is Hermitian, so c_Q is real and every J block Hermitian."""
    cr, tr = crystal("C1")
    rho = density(cr)
    J, c = hf_hartree_numpy(cr, tr, rho)
    L = cr.layout
    assert np.abs(c.imag).max() < 1e-12 * max(1.0, np.abs(c).max()) and np.abs(c).max() > 1e-3
    for ik, k in enumerate(L.irre_list):
        for ib, bs in enumerate(L.ao_sizes[k]):
            o = L.kao_slice_offsets_irre[ik] + L.ao_offsets[k][ib]
            B = J[o:o + bs * bs].reshape(bs, bs)
            assert np.abs(B - B.conj().T).max() < 1e-12 * max(1.0, np.abs(J).max())

"""Generate the LiH golden fixtures from the reference's own data files.

Run in a checkout where the reference tree is available (it reads
``SymmetryMBPT/data`` under ``--ref``, or under $MBSYMMETRY_REF when the
option is not given):

    python tests/golden/make_golden.py --ref <path of the reference tree>

Outputs (committed; the GPU tests read only these):

* ``lih_inputs.npz``  – the LiH nk=2x2x2 block layout, V, F, S and the IR
  sampling data of ``ir_grid/1e3_72.h5`` (beta = 5, ni = 72, ns = 2).
* ``lih_golden.npz``  – reference results and the cross-relation residuals
  that pin the oracle:

  1. Dyson, block vs dense (the relation of the reference test
     ``Dyson.BlockDyson``, test/test_dyson.cpp:17-83): G(tau) from the block
     inputs (``input_flat.h5``) through the oracle vs a dense numpy Dyson on
     the dense adapted-basis inputs (``input_blk.h5``).  The stored golden G
     is the dense result mapped to the flat layout.
  2. P~, block vs dense (the relation of ``CuGWP.LiHnk2``,
     test/test_cugw.cpp:210-304): the oracle's block W~ solve vs a dense numpy
     restatement of ``gw_solver::compute_P_from_P0`` (src/cpu_ref/gw.cpp:129-160).
     The stored golden P~ is the dense result.
  3. V, block vs dense: the dense AO-basis integrals ``df_int/VQ_0.h5`` and the
     flat block integrals ``block/df_int/VQ_flat_0.h5`` are related by
     per-k unitaries, so the spectra of sum_Q V V^H (both AO sides) and of
     sum_ij V V^H (aux side) agree pair by pair; this pins the V reader and the
     block packing rule (q = k2 - k1 labelling).
  4. P0 and Sigma: the C oracle vs an independent numpy einsum restatement of
     ``gw_block.cpp`` on the same block inputs.
  5. P0 and Sigma, block vs dense: the oracle's block P0 and Sigma (on the
     block chain: input_flat.h5, VQ_flat_0.h5) vs a restatement of the
     reference's DENSE solver (``gw_solver::compute_full_P0_t`` /
     ``compute_Sigma_from_P_t``, src/cpu_ref/gw.cpp:65-127) on the dense chain
     (G from the dense Dyson on input_blk.h5, P~ from the dense W~ solve, V
     blocks in dense arrays) -- the route of the reference's own dense-solver
     test (test/test_cugw.cpp:250-291).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from mbsymmetry_gb300.h5lite import H5File, as_complex  # noqa: E402
from mbsymmetry_gb300.inputs import load_reference_inputs  # noqa: E402
from mbsymmetry_gb300.transformer import build_transforms, read_ir_file  # noqa: E402

NT_P0 = 10      # tau points of P0 kept (the reference test checks t < 10)
NT_SIG = 5      # tau points of Sigma kept (the reference test checks t < 5)
T_PT = (0, 1, 2, 36, 37, 72, 73)  # tau points of P~ kept


def numpy_p0(L, G_full_fn, V, ns, nts, nt_max):
    """Independent einsum restatement of gw_block.cpp:6-84 (all k, q = all)."""
    out = {}
    pref = -1.0 / L.nk * (2.0 if ns == 1 else 1.0)
    for iq_irr, q in enumerate(L.irre_list):
        res = np.zeros((nt_max, L.qaux_slice_sizes[q]), np.complex128)
        for k1 in range(L.nk):
            k2 = L.mom_cons(k1, 0, q)
            p = k1 * L.nk + k2
            base = L.kpair_slice_offsets[p]
            for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
                qb, b1, b2 = L.aux_sizes[q][iq], L.ao_sizes[k1][i1], L.ao_sizes[k2][i2]
                o = base + L.tensor_offsets[p][b]
                Vb = V[o:o + qb * b1 * b2].reshape(qb, b1, b2)
                po = L.aux_offsets[q][iq]
                for t in range(nt_max):
                    for s in range(ns):
                        Gm = G_full_fn(k1, nts - 1 - t, s, i1)
                        G2 = G_full_fn(k2, t, s, i2)
                        blk = np.einsum("tp,Qpm,Ptn,mn->QP", Gm, Vb, Vb.conj(), G2, optimize=True)
                        res[t, po:po + qb * qb] += blk.ravel()
        out[iq_irr] = res * pref
    return out


def numpy_sigma(L, G_full_fn, P_full_fn, V, ns, nts, nt_max):
    """Independent einsum restatement of gw_block.cpp:86-158."""
    out = {}
    for ik, k1 in enumerate(L.irre_list):
        res = np.zeros((nt_max, ns, L.kao_slice_sizes[k1]), np.complex128)
        for q in range(L.nk):
            k2 = L.mom_cons(k1, q, 0)
            p = k1 * L.nk + k2
            base = L.kpair_slice_offsets[p]
            for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
                qb, b1, b2 = L.aux_sizes[q][iq], L.ao_sizes[k1][i1], L.ao_sizes[k2][i2]
                o = base + L.tensor_offsets[p][b]
                Vb = V[o:o + qb * b1 * b2].reshape(qb, b1, b2)
                so = L.ao_offsets[k1][i1]
                for t in range(nt_max):
                    Pq = P_full_fn(q, t, iq)
                    for s in range(ns):
                        G2 = G_full_fn(k2, t, s, i2)
                        blk = np.einsum("Qim,mn,QP,Pjn->ij", Vb, G2, Pq, Vb.conj(), optimize=True)
                        res[t, s, so:so + b1 * b1] += blk.ravel()
        out[ik] = res * (-1.0 / L.nk)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MBSYMMETRY_REF"),
                    help="path of the reference tree (default: $MBSYMMETRY_REF)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref or set MBSYMMETRY_REF to the reference tree")
    from oracle import Oracle
    D = os.path.join(args.ref, "SymmetryMBPT", "data")
    blk = os.path.join(D, "LiH", "integral", "nk2", "block")
    ri = load_reference_inputs(blk)
    L = ri.layout
    ir = read_ir_file(os.path.join(D, "ir_grid", "1e3_72.h5"))
    beta, mu = 5.0, 0.0
    tr = build_transforms(ir, beta)
    ns, nts, nk = ri.ns, tr.nts, L.nk
    nao, naux = L.nao, L.naux
    orc = Oracle(L, ns, nts)
    rel = {}

    # 1. Dyson block vs dense
    G, leak = orc.dyson(np.zeros(nts * ns * L.flat_ao_size, np.complex128), ri.onebody.F, ri.onebody.S, tr, mu)
    fb = H5File(os.path.join(blk, "input_blk.h5"))
    Fd, Sd = as_complex(fb["HF/Fock-k"]), as_complex(fb["HF/S-k"])
    om = tr.omega_fermi()
    Gd = np.zeros((nts, ns, nk, nao, nao), np.complex128)
    for s in range(ns):
        for k in range(nk):
            Gw = np.array([np.linalg.inv((w + mu) * Sd[s, k] - Fd[s, k]) for w in om])
            Gd[:, s, k] = np.einsum("tw,wij->tij", tr.Ttn, Gw)
    G_dense_flat = L.G_block_to_flat(Gd).reshape(-1)
    rel["dyson_block_vs_dense"] = float(np.abs(G_dense_flat - G).max())

    # 3. V spectral invariants, dense AO-basis file vs flat block file
    vd = H5File(os.path.join(D, "LiH", "integral", "nk2", "df_int", "VQ_0.h5"))["0"]
    vd = vd.reshape(-1, naux, nao, nao, 2)
    vd = vd[..., 0] + 1j * vd[..., 1]

    def V_dense(k1, k2):
        if k1 >= k2:
            return vd[k1 * (k1 + 1) // 2 + k2]
        return vd[k2 * (k2 + 1) // 2 + k1].transpose(0, 2, 1).conj()

    def V_block_dense(k1, k2):
        p = k1 * nk + k2
        q = L.pair_q(k1, k2)
        out = np.zeros((naux, nao, nao), np.complex128)
        for b, (iq, i1, i2) in enumerate(L.tensor_irreps[p]):
            qb, b1, b2 = L.aux_sizes[q][iq], L.ao_sizes[k1][i1], L.ao_sizes[k2][i2]
            o = L.kpair_slice_offsets[p] + L.tensor_offsets[p][b]
            Q0, I0, J0 = L.aux_block_offsets[q][iq], L.ao_block_offsets[k1][i1], L.ao_block_offsets[k2][i2]
            out[Q0:Q0 + qb, I0:I0 + b1, J0:J0 + b2] = ri.V[o:o + qb * b1 * b2].reshape(qb, b1, b2)
        return out

    worst = 0.0
    for k1 in range(nk):
        for k2 in range(nk):
            A, B = V_dense(k1, k2), V_block_dense(k1, k2)
            for f in (lambda X: np.einsum("Qij,Qlj->il", X, X.conj()),
                      lambda X: np.einsum("Qij,Qil->jl", X, X.conj()),
                      lambda X: np.einsum("Qij,Pij->QP", X, X.conj())):
                ea, eb = np.linalg.eigvalsh(f(A)), np.linalg.eigvalsh(f(B))
                worst = max(worst, float(np.abs(ea - eb).max() / max(1.0, np.abs(ea).max())))
    rel["V_spectra_block_vs_dense"] = worst

    # 4. P0 / Sigma: C oracle vs numpy restatement
    Gf = orc.rotate_G(G)
    P0 = orc.p0(Gf, ri.V)

    def G_full_fn(k, t, s, ib):
        o = L.kao_slice_offsets[k] * ns * nts + (t * ns + s) * L.kao_slice_sizes[k] + L.ao_offsets[k][ib]
        b = L.ao_sizes[k][ib]
        return Gf[o:o + b * b].reshape(b, b)

    P0np = numpy_p0(L, G_full_fn, ri.V, ns, nts, NT_P0)
    d = 0.0
    for iq in range(L.ink):
        o, sz = L.qaux_slice_offsets_irre[iq], L.qaux_slice_sizes_irre[iq]
        c = P0[nts * o: nts * (o + sz)].reshape(nts, sz)[:NT_P0]
        d = max(d, float(np.abs(c - P0np[iq]).max()))
    rel["p0_oracle_vs_numpy"] = d

    # 2. P~ block vs dense
    P = orc.p_tilde(P0, tr)
    P0t = np.zeros((nts, L.flat_aux_size), np.complex128)
    for iq in range(L.ink):
        o, sz = L.qaux_slice_offsets_irre[iq], L.qaux_slice_sizes_irre[iq]
        P0t[:, o:o + sz] = P0[nts * o: nts * (o + sz)].reshape(nts, sz)
    Pd = L.P_flat_to_block(P0t)
    for t in range(nts // 2):
        Pd[nts - t - 1] = Pd[t]
    Pd = 0.5 * (Pd + Pd.conj().transpose(0, 1, 3, 2))
    Pw = np.einsum("wt,tqij->wqij", tr.Tnt_BF, Pd[1:nts - 1])
    eye = np.eye(naux)
    for n in range(tr.nw_b):
        for q in range(nk):
            tmp = np.linalg.inv(eye - Pw[n, q])
            tmp = 0.5 * (tmp + tmp.conj().T)
            Pw[n, q] = tmp @ Pw[n, q]
    Pd2 = np.einsum("tw,wqij->tqij", tr.Ttn_FB, Pw)
    Pd2 = 0.5 * (Pd2 + Pd2.conj().transpose(0, 1, 3, 2))
    P_dense_flat = L.P_block_to_flat(Pd2)
    d = 0.0
    for iq in range(L.ink):
        o, sz = L.qaux_slice_offsets_irre[iq], L.qaux_slice_sizes_irre[iq]
        d = max(d, float(np.abs(P[nts * o: nts * (o + sz)].reshape(nts, sz) - P_dense_flat[:, o:o + sz]).max()))
    rel["p_tilde_block_vs_dense"] = d

    # 5. P0, block oracle vs the reference's DENSE algorithm (gw_solver::compute_full_P0_t,
    #    src/cpu_ref/gw.cpp:65-100 with P0_contraction :203-216) on the dense chain: G from
    #    the dense Dyson on input_blk.h5, V(k1, k2) the block file's blocks in dense
    #    [NQ][nao][nao] arrays (the reference's P_flat_to_block / dense-solver test route,
    #    test/test_cugw.cpp:250-291).
    Vd = {(k1, k2): V_block_dense(k1, k2) for k1 in range(nk) for k2 in range(nk)}
    pref = -1.0 / nk * (2.0 if ns == 1 else 1.0)
    P0d = np.zeros((NT_P0, nk, naux, naux), np.complex128)
    for q in range(nk):
        for k1 in range(nk):
            k2 = L.mom_cons(k1, 0, q)  # k2 = k1 + q
            V = Vd[(k1, k2)]
            for t in range(NT_P0):
                for s in range(ns):
                    P0d[t, q] += np.einsum("tp,Qpm,Ptn,mn->QP", Gd[nts - 1 - t, s, k1], V, V.conj(), Gd[t, s, k2],
                                           optimize=True)
    P0d *= pref
    P0d_flat = L.P_block_to_flat(P0d)
    d = 0.0
    for iq in range(L.ink):
        o, sz = L.qaux_slice_offsets_irre[iq], L.qaux_slice_sizes_irre[iq]
        d = max(d, float(np.abs(P0[nts * o: nts * (o + sz)].reshape(nts, sz)[:NT_P0] - P0d_flat[:, o:o + sz]).max()))
    rel["p0_block_vs_dense_gw"] = d

    Pf = orc.rotate_P(P)
    Sig = orc.sigma(Gf, Pf, ri.V)

    # 6. Sigma, block oracle vs the dense algorithm (gw_solver::compute_Sigma_from_P_t,
    #    gw.cpp:102-127 with Sigma_contraction :218-231) on the dense chain's P~ (Pd2).
    Sd = np.zeros((NT_SIG, ns, nk, nao, nao), np.complex128)
    for q in range(nk):
        for k1 in range(nk):
            k2 = L.mom_cons(k1, q, 0)  # k2 = k1 - q
            V = Vd[(k1, k2)]
            for t in range(NT_SIG):
                for s in range(ns):
                    Sd[t, s, k1] += np.einsum("Qim,mn,QP,Pjn->ij", V, Gd[t, s, k2], Pd2[t, q], V.conj(),
                                              optimize=True)
    Sd *= -1.0 / nk
    Sd_flat = L.G_block_to_flat(Sd).reshape(NT_SIG, ns, L.flat_ao_size)
    rel["sigma_block_vs_dense_gw"] = float(np.abs(Sig.reshape(nts, ns, L.flat_ao_size)[:NT_SIG] - Sd_flat).max())

    def P_full_fn(q, t, iq):
        o = nts * L.qaux_slice_offsets[q] + t * L.qaux_slice_sizes[q] + L.aux_offsets[q][iq]
        b = L.aux_sizes[q][iq]
        return Pf[o:o + b * b].reshape(b, b)

    Snp = numpy_sigma(L, G_full_fn, P_full_fn, ri.V, ns, nts, NT_SIG)
    d = 0.0
    S3 = Sig.reshape(nts, ns, L.flat_ao_size)
    for ik in range(L.ink):
        o, sz = L.kao_slice_offsets_irre[ik], L.kao_slice_sizes_irre[ik]
        d = max(d, float(np.abs(S3[:NT_SIG, :, o:o + sz] - Snp[ik]).max()))
    rel["sigma_oracle_vs_numpy"] = d
    G2, leak2 = orc.dyson(Sig, ri.onebody.F, ri.onebody.S, tr, mu)

    for k, v in rel.items():
        print(f"{k:32s} {v:.3e}")
    assert rel["dyson_block_vs_dense"] < 1e-10
    assert rel["p_tilde_block_vs_dense"] < 1e-9
    assert rel["V_spectra_block_vs_dense"] < 1e-10
    assert rel["p0_oracle_vs_numpy"] < 1e-12
    assert rel["sigma_oracle_vs_numpy"] < 1e-12
    assert rel["p0_block_vs_dense_gw"] < 1e-10
    assert rel["sigma_block_vs_dense_gw"] < 1e-10

    # ---- inputs ----
    cat = lambda xs: np.concatenate([np.asarray(x).reshape(-1) for x in xs])  # noqa: E731
    ptr = lambda xs: np.concatenate([[0], np.cumsum([len(np.asarray(x).reshape(-1)) for x in xs])])  # noqa: E731
    np.savez_compressed(
        os.path.join(HERE, "lih_inputs.npz"),
        nk=nk, ns=ns, beta=beta, mu=mu, kmesh=L.kmesh,
        ao_sizes=cat(L.ao_sizes), ao_ptr=ptr(L.ao_sizes),
        aux_sizes=cat(L.aux_sizes), aux_ptr=ptr(L.aux_sizes),
        ao_block_offsets=cat(L.ao_block_offsets), aux_block_offsets=cat(L.aux_block_offsets),
        tensor_irreps=cat(L.tensor_irreps), tensor_ptr=ptr([t.reshape(-1) for t in L.tensor_irreps]),
        V=ri.V, F=ri.onebody.F, S=ri.onebody.S, H=ri.onebody.H,
        **{"ir_" + k.replace("/", "_"): v for k, v in ir.items()},
    )
    # ---- golden outputs ----
    P_sel = np.concatenate([P_dense_flat[t] for t in T_PT])
    P0_sel = np.concatenate([P0d_flat[t] for t in range(NT_P0)])  # the dense chain's P0
    np.savez_compressed(
        os.path.join(HERE, "lih_golden.npz"),
        G=G_dense_flat, P0_t=P0_sel, nt_p0=NT_P0, P_tilde_t=P_sel, t_pt=np.array(T_PT),
        Sigma_t=Sd_flat.reshape(-1), nt_sigma=NT_SIG, G_after_gw=G2,  # the dense chain's Sigma
        leakage_g0=leak, leakage_g1=leak2,
        **{"rel_" + k: v for k, v in rel.items()},
    )
    for f in ("lih_inputs.npz", "lih_golden.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)) // 1024, "KiB")


if __name__ == "__main__":
    main()

"""The reference's iBZ-vs-full-BZ relation on the GPU
(SymmetryMBPT/test/test_cugw.cpp:306-436, CuGWRotP0 / CuGWRotSigma) on
group-consistent crystals: one handle on the irreducible k points with the
rotations, one on every k point of the mesh (no rotations), each from its
own Dyson G0.  P~ at the irreducible q and Sigma and G at the irreducible k
agree to 1e-10 on the FP64 path and to 1e-7 (the stated bound) on the sliced
path."""
import dataclasses

import numpy as np
import pytest

from mbsymmetry_gb300.crystal import CONFIGS, load_ir, make_crystal
from mbsymmetry_gb300.transformer import build_transforms

pytestmark = pytest.mark.gpu


def _run(cr, tr, mu, precision):
    from mbsymmetry_gb300.solver import GWSolver
    s = GWSolver(cr.layout, cr.ns, tr, precision=precision)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    s.dyson(mu)
    s.solve()
    out = [s.P0_q_t_QP(), s.Selfenergy()]
    s.dyson(mu)
    out.append(s.G_tau())
    s.close()
    return out


def _irr_diffs(cr, cf, rot, full, nts):
    Lr, Lf, ns = cr.layout, cf.layout, cr.ns
    dp = ds = dg = 0.0
    for iq, q in enumerate(Lr.irre_list):
        n = nts * Lr.qaux_slice_sizes[q]
        a = rot[0][nts * Lr.qaux_slice_offsets_irre[iq]:][:n]
        b = full[0][nts * Lf.qaux_slice_offsets_irre[q]:][:n]
        dp = max(dp, float(np.abs(a - b).max()))
    for x, y, which in ((rot[1], full[1], "s"), (rot[2], full[2], "g")):
        x, y = x.reshape(nts, ns, -1), y.reshape(nts, ns, -1)
        for ik, k in enumerate(Lr.irre_list):
            n = Lr.kao_slice_sizes[k]
            d = float(np.abs(x[:, :, Lr.kao_slice_offsets_irre[ik]:][:, :, :n]
                             - y[:, :, Lf.kao_slice_offsets_irre[k]:][:, :, :n]).max())
            if which == "s":
                ds = max(ds, d)
            else:
                dg = max(dg, d)
    return dp, ds, dg


@pytest.mark.parametrize("name,ns,precision,bound", [("C1", 1, "fp64", 1e-10), ("C1", 2, "fp64", 1e-10),
                                                     ("C2", 1, "fp64", 1e-10), ("C1", 2, "ozaki", 1e-7),
                                                     ("C2", 1, "ozaki", 1e-7)])
def test_irreducible_and_full_mesh_agree(name, ns, precision, bound):
    spec = dataclasses.replace(CONFIGS[name], ns=ns)
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = make_crystal(spec, rotate=True, symmetric=True)
    cf = make_crystal(spec, rotate=False, symmetric=True)
    rot = _run(cr, tr, cr.mu, precision)
    full = _run(cf, tr, cr.mu, precision)
    dp, ds, dg = _irr_diffs(cr, cf, rot, full, tr.nts)
    print(f"{name} ns={ns} {precision}: ink {cr.layout.ink} vs {cf.layout.ink}: P~ {dp:.1e}, Sigma {ds:.1e}, "
          f"G {dg:.1e} (max|Sigma| {np.abs(full[1]).max():.2f})")
    assert max(dp, ds, dg) < bound


def test_wurtzite_blocks_fp64_against_oracle_and_sliced_within_bound():
    """Block sizes from P6_3mc (projective representations at the zone boundary)
    on a 2x2x2 hexagonal mesh with time reversal: the FP64 path against the
    oracle at 1e-10 and the sliced path against FP64 at 1e-7."""
    from oracle import Oracle
    spec = dataclasses.replace(CONFIGS["C4"], name="wurtzite-2x2x2", mesh=(2, 2, 2), nao=24, naux=80, nts=62,
                               beta=50.0)
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    cr = make_crystal(spec, physical=True)
    L = cr.layout
    orc = Oracle(L, cr.ns, tr.nts)
    G0, _ = orc.dyson(np.zeros(tr.nts * cr.ns * L.flat_ao_size, np.complex128), cr.F, cr.S, tr, cr.mu)
    _, Sr, *_ = orc.iteration(G0, cr.V, cr.F, cr.S, tr, cr.mu)
    out = {}
    for precision in ("fp64", "ozaki"):
        from mbsymmetry_gb300.solver import GWSolver
        s = GWSolver(L, cr.ns, tr, precision=precision)
        s.set_shared_Coulomb(cr.V)
        s.set_fock(cr.F, cr.S)
        s.set_G(G0)
        s.solve()
        out[precision] = s.Selfenergy()
        s.close()
    e64, eoz = np.abs(out["fp64"] - Sr).max(), np.abs(out["ozaki"] - out["fp64"]).max()
    print(f"wurtzite 2x2x2 (ink {L.ink}, AO blocks {sorted({int(b) for k in L.irre_list for b in L.ao_sizes[k]})}): "
          f"FP64 vs oracle {e64:.1e}, sliced vs FP64 {eoz:.1e}")
    assert e64 < 1e-10 and eoz < 1e-7

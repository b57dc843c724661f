"""The autotuner times its candidates on the device and the settings it
returns give a handle whose mixed-precision Sigma keeps the FP64 error bound."""
import numpy as np
import pytest

from _helpers import crystal

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_candidate_and_keeps_accuracy(tmp_path):
    from mbsymmetry_gb300 import autotune
    from mbsymmetry_gb300.solver import GWSolver
    cr, tr = crystal("C1")
    cands = ({"uvt_smem_kb": 110, "sw_npk_max": 64, "uv_waves": 4}, {"uvt_smem_kb": 72, "sw_npk_max": 32, "uv_waves": 2})
    out = autotune.autotune(cr.layout, cr.ns, tr, cr.V, cr.F, cr.S, cr.mu, candidates=cands, reps=1,
                            cache=str(tmp_path / "t.json"))
    assert out["best"] in [dict(c) for c in cands]
    assert len(out["trials"]) == 2 and all(t["sigma_ms"] > 0 for t in out["trials"])
    ref = GWSolver(cr.layout, cr.ns, tr)
    ref.set_shared_Coulomb(cr.V)
    ref.set_fock(cr.F, cr.S)
    ref.set_Selfenergy(np.zeros(ref.g_size, np.complex128))
    ref.dyson(cr.mu)
    G0 = ref.G_tau()
    ref.solve()
    S64 = ref.Selfenergy()
    ref.close()
    for c in cands:
        s = GWSolver(cr.layout, cr.ns, tr, precision="tf32x3", tune=c)
        s.set_shared_Coulomb(cr.V)
        s.set_fock(cr.F, cr.S)
        s.set_G(G0)
        s.solve()
        err = np.abs(s.Selfenergy() - S64).max()
        s.close()
        assert err < 1e-5 * max(1.0, np.abs(S64).max())

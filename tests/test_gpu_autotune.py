"""The autotuner times its candidates on the device and the settings it
returns give a handle whose sliced-path Sigma stays within 1e-7 Ha of FP64."""
import numpy as np
import pytest

from _helpers import crystal

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_candidate_and_keeps_accuracy(tmp_path):
    from mbsymmetry_gb300 import autotune
    from mbsymmetry_gb300.solver import GWSolver
    cr, tr = crystal("C1")
    cands = autotune.OZAKI_CANDIDATES
    out = autotune.autotune(cr.layout, cr.ns, tr, cr.V, cr.F, cr.S, cr.mu, precision="ozaki", reps=1,
                            cache=str(tmp_path / "t.json"))
    assert out["best"] in [dict(c) for c in cands] and out["metric"] == "iteration_ms"
    assert len(out["trials"]) == len(cands) and all(t["iteration_ms"] > 0 for t in out["trials"])
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
        s = GWSolver(cr.layout, cr.ns, tr, precision="ozaki", tune=c)
        s.set_shared_Coulomb(cr.V)
        s.set_fock(cr.F, cr.S)
        s.set_G(G0)
        s.solve()
        err = np.abs(s.Selfenergy() - S64).max()
        s.close()
        assert err < 1e-7
